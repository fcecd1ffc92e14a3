// Post-Newtonian pair terms (tupan/lib/src/pn_terms.h, pnacc_kernel_common.h)
// in REAL precision.  The rational coefficients are built as REAL(p)/q like
// the reference's macros (pn_terms.h:7-123) and every sum keeps the
// reference's association, so with -fmad=false the result is bit-identical
// to the reference C.  Orders 1 and 3 are empty in the reference as well.
#pragma once

#include "tg_pairs.cuh"

namespace tg {

template <typename R>
__device__ __forceinline__ R rq(int p, int q) { return R(p) / R(q); }

template <typename R>
struct PnTerm { R a, b; };

// pn_terms.h:126-152
template <typename R>
__device__ PnTerm<R> pn2(R im, R jm, R inv_r, R iv2, R jv2, R ivjv, R niv,
                         R njv, R njv2, R inv2)
{
    PnTerm<R> p;
    p.a = -iv2 - R(2) * jv2 + R(4) * ivjv + rq<R>(3, 2) * njv2
          + inv_r * (R(5) * im + R(4) * jm);
    p.b = R(4) * niv - R(3) * njv;
    p.a *= inv2;
    p.b *= inv2;
    return p;
}

// pn_terms.h:155-213
template <typename R>
__device__ PnTerm<R> pn4(R im, R jm, R im2, R jm2, R imjm, R inv_r, R inv_r2,
                         R iv2, R jv2, R jv4, R ivjv, R ivjvivjv, R nv, R niv,
                         R njv, R niv2, R njv2, R nivnjv, R inv4)
{
    PnTerm<R> p;
    p.a = R(-2) * (jv4 + ivjvivjv)
          + R(4) * jv2 * ivjv
          + njv2 * (rq<R>(3, 2) * iv2 + rq<R>(9, 2) * jv2 - R(6) * ivjv
                    - rq<R>(15, 8) * njv2)
          - inv_r2 * (rq<R>(57, 4) * im2 + R(9) * jm2 + rq<R>(69, 2) * imjm)
          + inv_r * (im * (-rq<R>(15, 4) * iv2 + rq<R>(5, 4) * jv2
                           - rq<R>(5, 2) * ivjv + rq<R>(39, 2) * niv2
                           - R(39) * nivnjv + rq<R>(17, 2) * njv2)
                     + jm * (R(4) * jv2 - R(8) * ivjv + R(2) * niv2
                             - R(4) * nivnjv - R(6) * njv2));
    p.b = inv_r * (im * (-rq<R>(63, 4) * niv + rq<R>(55, 4) * njv)
                   - jm * R(2) * (niv + njv))
          + iv2 * njv
          - ivjv * nv * R(4)
          + jv2 * (R(4) * niv - R(5) * njv)
          + njv2 * (R(-6) * niv + rq<R>(9, 2) * njv);
    p.a *= inv4;
    p.b *= inv4;
    return p;
}

// pn_terms.h:216-237
template <typename R>
__device__ PnTerm<R> pn5(R im, R jm, R inv_r, R v2, R nv, R inv5)
{
    PnTerm<R> p;
    p.a = nv * (inv_r * (-rq<R>(24, 5) * im + rq<R>(208, 15) * jm)
                + rq<R>(12, 5) * v2);
    p.b = -v2 + inv_r * (rq<R>(8, 5) * im - rq<R>(32, 5) * jm);
    R s = (im * inv_r) * inv5;
    p.a *= s;
    p.b *= s;
    return p;
}

// pn_terms.h:240-372
template <typename R>
__device__ PnTerm<R> pn6(R im, R jm, R im2, R jm2, R imjm, R inv_r, R inv_r2,
                         R v2, R iv2, R jv2, R jv4, R ivjv, R ivjvivjv, R nv,
                         R nvnv, R niv, R njv, R niv2, R njv2, R nivnjv,
                         R inv6)
{
    const R pisq = R(9.869604401089358);
    PnTerm<R> p;
    R t_njv2 =
        njv2 * (R(3) * ivjvivjv
                + rq<R>(3, 2) * iv2 * jv2
                - R(12) * ivjv * jv2
                + rq<R>(15, 2) * jv4
                + njv2 * (rq<R>(15, 2) * (ivjv - jv2 - rq<R>(1, 4) * iv2)
                          + rq<R>(35, 16) * njv2));
    R t_jv2 = R(2) * jv2 * (-ivjvivjv + jv2 * (R(2) * ivjv - jv2));
    R t_im =
        im * inv_r *
        (niv * (njv * (R(244) * ivjv - rq<R>(205, 2) * iv2
                       - rq<R>(283, 2) * jv2 + rq<R>(383, 2) * njv2)
                + niv * (rq<R>(229, 4) * (iv2 + jv2 - R(2) * ivjv)
                         - rq<R>(723, 4) * njv2
                         + niv * (rq<R>(171, 2) *
                                  (njv - rq<R>(1, 4) * niv))))
         + njv2 * (rq<R>(191, 4) * iv2 + rq<R>(259, 4) * jv2
                   - rq<R>(225, 2) * ivjv - rq<R>(455, 8) * njv2)
         + ivjv * (rq<R>(91, 2) * iv2 + R(43) * jv2 - rq<R>(177, 4) * ivjv)
         - rq<R>(91, 8) * iv2 * (iv2 + R(2) * jv2)
         - rq<R>(81, 8) * jv4);
    R t_jm =
        jm * inv_r * R(4) *
        (jv4
         + njv * (niv * (ivjv - jv2)
                  + njv * (R(3) * (ivjv - jv2) - rq<R>(3, 2) * niv2
                           + njv * (R(3) * niv + rq<R>(3, 2) * njv)))
         + ivjv * (ivjv - R(2) * jv2));
    R t_jm2 = jm2 * inv_r2 *
              (-niv2 + R(2) * nivnjv + rq<R>(43, 2) * njv2 + R(18) * ivjv
               - R(9) * jv2);
    R t_imjm = imjm * inv_r2 *
               (rq<R>(415, 8) * niv2 - rq<R>(375, 4) * nivnjv
                + rq<R>(1113, 8) * njv2 + R(18) * iv2
                + pisq * (rq<R>(123, 64) * v2 - rq<R>(615, 64) * nvnv)
                + R(33) * (ivjv - rq<R>(1, 2) * jv2));
    R t_im2 = im2 * inv_r2 *
              (-rq<R>(2069, 8) * niv2 + R(543) * nivnjv
               - rq<R>(939, 4) * njv2 + rq<R>(471, 8) * iv2
               + rq<R>(357, 8) * (jv2 - R(2) * ivjv));
    R t_cub = inv_r * inv_r2 *
              (R(16) * jm * jm2
               + im2 * jm * (rq<R>(547, 3) - rq<R>(41, 16) * pisq)
               - rq<R>(13, 12) * im * im2
               + im * jm2 * (rq<R>(545, 3) - rq<R>(41, 16) * pisq));
    p.a = t_njv2 + t_jv2 + t_im + t_jm + t_jm2 + t_imjm + t_im2 + t_cub;

    R u_njv =
        njv * (jv2 * (iv2 + R(8) * ivjv - R(7) * jv2)
               - R(2) * ivjvivjv
               + njv * (R(6) * niv * (ivjv - R(2) * jv2)
                        + njv * (R(6) * (R(2) * jv2 - ivjv
                                         - rq<R>(1, 4) * iv2)
                                 + njv * (rq<R>(15, 2) *
                                          (niv - rq<R>(3, 4) * njv)))));
    R u_niv = R(4) * niv * (jv4 - ivjv * jv2);
    R u_jm = jm * inv_r *
             (njv * (R(4) * (ivjv - jv2 - rq<R>(1, 2) * niv2)
                     + njv * (R(2) * (R(4) * niv + njv)))
              + R(2) * niv * (ivjv - jv2));
    R u_im = im * inv_r *
             (niv * (rq<R>(207, 8) * iv2 + rq<R>(81, 8) * jv2 - R(36) * ivjv
                     - rq<R>(269, 4) * njv2
                     + niv * (rq<R>(565, 4) * njv - rq<R>(243, 4) * niv))
              + njv * (rq<R>(83, 8) * jv2 + rq<R>(27, 4) * ivjv
                       - rq<R>(137, 8) * iv2 - rq<R>(95, 12) * njv2));
    R u_r2 = inv_r2 *
             (jm2 * (R(4) * niv + R(5) * njv)
              + im2 * (rq<R>(311, 4) * niv - rq<R>(357, 4) * njv)
              + imjm * (rq<R>(479, 8) * njv - rq<R>(307, 8) * niv
                        + rq<R>(123, 32) * pisq * nv));
    p.b = u_njv + u_niv + u_jm + u_im + u_r2;
    p.a *= inv6;
    p.b *= inv6;
    return p;
}

// pn_terms.h:375-470
template <typename R>
__device__ PnTerm<R> pn7(R im, R jm, R im2, R jm2, R imjm, R inv_r, R inv_r2,
                         R v2, R iv2, R jv2, R iv4, R jv4, R ivjv, R nv,
                         R nvnv, R niv, R njv, R niv2, R njv2, R nivnjv,
                         R inv7)
{
    PnTerm<R> p;
    R a_im2 = im2 * inv_r2 *
              (rq<R>(3992, 105) * niv - rq<R>(4328, 105) * njv);
    R a_imjm = imjm * inv_r * inv_r2 *
               (-rq<R>(13576, 105) * niv + rq<R>(2872, 21) * njv);
    R a_jm2 = jm2 * inv_r * inv_r2 * (-rq<R>(3172, 21) * nv);
    R a_im =
        im * inv_r *
        (niv * (R(48) * niv2 - rq<R>(4888, 105) * iv2
                + rq<R>(2056, 21) * ivjv - rq<R>(1028, 21) * jv2)
         + nivnjv * (-rq<R>(696, 5) * niv + rq<R>(744, 5) * njv)
         + njv * (-rq<R>(288, 5) * njv2 + rq<R>(5056, 105) * iv2
                  - rq<R>(2224, 21) * ivjv + rq<R>(5812, 105) * jv2));
    R a_jm =
        jm * inv_r *
        (niv * (-rq<R>(582, 5) * niv2 - rq<R>(2864, 35) * ivjv
                + rq<R>(1432, 35) * jv2)
         + nivnjv * (rq<R>(1746, 5) * niv - rq<R>(1954, 5) * njv)
         + rq<R>(3568, 105) * nv * iv2
         + njv * (R(158) * njv2 - rq<R>(5752, 105) * jv2
                  + rq<R>(10048, 105) * ivjv));
    R a_v =
        nv * (R(-56) * nvnv * nvnv - rq<R>(246, 35) * iv4)
        + niv * (v2 * (R(60) * niv2 - R(180) * nivnjv + R(174) * njv2)
                 + ivjv * (rq<R>(1068, 35) * (iv2 - ivjv)
                           + rq<R>(984, 35) * jv2)
                 - rq<R>(534, 35) * iv2 * jv2
                 - rq<R>(204, 35) * jv4)
        + njv * (R(-54) * njv2 * v2
                 + ivjv * (-rq<R>(984, 35) * iv2 + rq<R>(180, 7) * ivjv
                           - rq<R>(732, 35) * jv2)
                 + rq<R>(90, 7) * iv2 * jv2
                 + rq<R>(24, 7) * jv4);
    p.a = a_im2 + a_imjm + a_jm2 + a_im + a_jm + a_v;

    R b_m2 = -im2 * inv_r2 * rq<R>(184, 21)
             + imjm * inv_r2 * rq<R>(6224, 105)
             + jm2 * inv_r2 * rq<R>(6388, 105);
    R b_im = im * inv_r *
             (rq<R>(52, 15) * niv2 - rq<R>(56, 15) * nivnjv
              - rq<R>(44, 15) * njv2 - rq<R>(132, 35) * iv2
              + rq<R>(152, 35) * ivjv - rq<R>(48, 35) * jv2);
    R b_jm = jm * inv_r *
             (rq<R>(454, 15) * niv2 - rq<R>(372, 5) * nivnjv
              + rq<R>(854, 15) * njv2 - rq<R>(152, 21) * iv2
              + rq<R>(2864, 105) * ivjv - rq<R>(1768, 105) * jv2);
    R b_v = R(60) * nvnv * nvnv
            + v2 * (-rq<R>(348, 5) * niv2 + rq<R>(684, 5) * nivnjv
                    - R(66) * njv2)
            + rq<R>(334, 35) * iv4
            + ivjv * (-rq<R>(1336, 35) * iv2 + rq<R>(1308, 35) * ivjv
                      - rq<R>(1252, 35) * jv2)
            + rq<R>(654, 35) * iv2 * jv2
            + rq<R>(292, 35) * jv4;
    p.b = b_m2 + b_im + b_jm + b_v;
    R s = (im * inv_r) * inv7;
    p.a *= s;
    p.b *= s;
    return p;
}

// pnacc_kernel_common.h:8-70 with p2p_pnterms, pn_terms.h:473-567
template <typename R>
struct PnAccPair {
    static constexpr int NA = 8, NO = 3;
    __device__ static void init(R *o) { o[0] = o[1] = o[2] = R(0); }
    __device__ static void pair(const R *ip, const R *jp, R *o,
                                const Sweep &s)
    {
        const uint64_t order = (uint64_t)s.iscal;
        R im = ip[0], jm = jp[0];
        R ivx = ip[5], ivy = ip[6], ivz = ip[7];
        R jvx = jp[5], jvy = jp[6], jvz = jp[7];
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R ux = ivx - jvx, uy = ivy - jvy, uz = ivz - jvz;
        R r2 = dx * dx + dy * dy + dz * dz;
        R v2 = ux * ux + uy * uy + uz * uz;
        R inv_r2 = masked_inv_r2(r2, h2);
        R inv_r = sqrt(inv_r2);
        R inv_r3 = inv_r2 * inv_r;

        PnTerm<R> p2 = {0, 0}, p4 = {0, 0}, p5 = {0, 0}, p6 = {0, 0},
                  p7 = {0, 0};
        const PnTerm<R> p1 = {0, 0}, p3 = {0, 0};
        R nx = dx * inv_r, ny = dy * inv_r, nz = dz * inv_r;
        R iv2 = ivx * ivx + ivy * ivy + ivz * ivz;
        R jv2 = jvx * jvx + jvy * jvy + jvz * jvz;
        if (order > 1) {
            R niv = nx * ivx + ny * ivy + nz * ivz;
            R njv = nx * jvx + ny * jvy + nz * jvz;
            R njv2 = njv * njv;
            R ivjv = ivx * jvx + ivy * jvy + ivz * jvz;
            p2 = pn2<R>(im, jm, inv_r, iv2, jv2, ivjv, niv, njv, njv2,
                        R(s.scal[2]));
            if (order > 3) {
                R im2 = im * im, jm2 = jm * jm, imjm = im * jm;
                R jv4 = jv2 * jv2;
                R ivjvivjv = ivjv * ivjv;
                R nv = nx * ux + ny * uy + nz * uz;
                R niv2 = niv * niv;
                R nivnjv = niv * njv;
                p4 = pn4<R>(im, jm, im2, jm2, imjm, inv_r, inv_r2, iv2, jv2,
                            jv4, ivjv, ivjvivjv, nv, niv, njv, niv2, njv2,
                            nivnjv, R(s.scal[4]));
                if (order > 4) {
                    p5 = pn5<R>(im, jm, inv_r, v2, nv, R(s.scal[5]));
                    if (order > 5) {
                        R nvnv = nv * nv;
                        p6 = pn6<R>(im, jm, im2, jm2, imjm, inv_r, inv_r2,
                                    v2, iv2, jv2, jv4, ivjv, ivjvivjv, nv,
                                    nvnv, niv, njv, niv2, njv2, nivnjv,
                                    R(s.scal[6]));
                        if (order > 6) {
                            R iv4 = iv2 * iv2;
                            p7 = pn7<R>(im, jm, im2, jm2, imjm, inv_r,
                                        inv_r2, v2, iv2, jv2, iv4, jv4, ivjv,
                                        nv, nvnv, niv, njv, niv2, njv2,
                                        nivnjv, R(s.scal[7]));
                        }
                    }
                }
            }
        }
        R pa = R(0), pb = R(0);
        pa += ((((((p7.a + p6.a) + p5.a) + p4.a) + p3.a) + p2.a) + p1.a);
        pb += ((((((p7.b + p6.b) + p5.b) + p4.b) + p3.b) + p2.b) + p1.b);
        pa *= jm * inv_r3;
        pb *= jm * inv_r2;
        o[0] += pa * dx + pb * ux;
        o[1] += pa * dy + pb * uy;
        o[2] += pa * dz + pb * uz;
    }
    __device__ static void finish(const R *, R *, const Sweep &) {}
};

}  // namespace tg
