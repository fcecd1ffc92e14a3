/*
 * CPU oracle for the tupan pairwise-gravity kernel layer.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference C kernels (tupan/lib/src/*.c and *_common.h).  It is linked by
 * the test-suite, by the smoke check and by the CPU-baseline leg of the
 * benchmark, and never by the product library.
 *
 * Every pair routine evaluates its arithmetic in the same order as the
 * reference (same association of + - * /, no contraction: build with
 * -ffp-contract=off), so that in IEEE double (or float, -DORACLE_SP) the
 * results are bit-identical to the reference kernels built with
 * `gcc -O3 -std=c99` (which also does not contract).  The j loop runs in
 * source order for each i, exactly as in the reference; the i loop may be
 * spread over OpenMP threads because every i is independent.
 *
 * Two deliberate differences, both only reachable on inputs where the
 * reference never returns:
 *   - the step-halving retry of the Kepler solver
 *     (universal_kepler_solver.h:486-499) and the energy-check subdivision
 *     (universal_kepler_solver.h:580-606) are unbounded `goto` loops in the
 *     reference; here a pair solve stops after ORACLE_SOLVE_BUDGET
 *     single-step solves (or ORACLE_MAX_HALVINGS doublings) and counts the
 *     event in oracle_kepler_failures().  Softened eccentric orbits with a
 *     long step are such inputs: their energy check never passes.
 */
#include <tgmath.h>   /* type-generic, as the reference (c_common.h:5) */
#include <stddef.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_SP
typedef float real_t;
typedef uint32_t uint_t;
typedef int32_t int_t;
#define SYM(name) oracle_sp_##name
#define KEPLER_TOL ((real_t)1.52587890625e-5)          /* 2^-16 */
#else
typedef double real_t;
typedef uint64_t uint_t;
typedef int64_t int_t;
#define SYM(name) oracle_##name
#define KEPLER_TOL ((real_t)2.2737367544323205948e-13) /* 2^-42 */
#endif

#define ORACLE_MAX_HALVINGS 40
/* Upper bound on single-step solves spent on one pair solve.  The reference
 * has none; on softened orbits whose energy check never passes it runs
 * without end.  Below this budget the two behave identically. */
#define ORACLE_SOLVE_BUDGET (1L << 20)
#define KEPLER_MAXITER 64
#define LAGUERRE_ORDER 5

static long kepler_failures = 0;

long SYM(kepler_failures)(void) { return kepler_failures; }

void SYM(set_threads)(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int SYM(max_threads)(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * Softened inverse powers (smoothing.h:10-184).  The reference masks with
 * r2 > 0 after forming 1/(r2+h2); that is the only way self pairs drop out.
 * ------------------------------------------------------------------------- */
static inline real_t masked_inv_r2(real_t r2, real_t h2)
{
    real_t q = 1 / (r2 + h2);
    return (r2 > 0) ? q : (real_t)0;
}

/* phi_kernel_common.h:7-32 */
static inline void pair_phi(real_t irx, real_t iry, real_t irz, real_t ie2,
                            real_t jm, real_t jrx, real_t jry, real_t jrz,
                            real_t je2, real_t *phi)
{
    real_t dx = irx - jrx, dy = iry - jry, dz = irz - jrz;
    real_t h2 = ie2 + je2;
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t q = masked_inv_r2(r2, h2);
    real_t inv_r1 = sqrt(q);
    *phi -= jm * inv_r1;
}

/* acc_kernel_common.h:7-38 */
static inline void pair_acc(real_t irx, real_t iry, real_t irz, real_t ie2,
                            real_t jm, real_t jrx, real_t jry, real_t jrz,
                            real_t je2, real_t *a)
{
    real_t dx = irx - jrx, dy = iry - jry, dz = irz - jrz;
    real_t h2 = ie2 + je2;
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t q = masked_inv_r2(r2, h2);
    real_t k = q * sqrt(q);
    k *= jm;
    a[0] -= k * dx;
    a[1] -= k * dy;
    a[2] -= k * dz;
}

/* acc_jerk_kernel_common.h:7-56 */
static inline void pair_acc_jerk(const real_t *ip, const real_t *jp, real_t *o)
{
    /* ip/jp: m, rx, ry, rz, e2, vx, vy, vz */
    real_t dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
    real_t h2 = ip[4] + jp[4];
    real_t ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t rv = dx * ux + dy * uy + dz * uz;
    real_t q = masked_inv_r2(r2, h2);
    real_t k = q * sqrt(q);
    real_t alpha = 3 * rv * q;
    ux -= alpha * dx;
    uy -= alpha * dy;
    uz -= alpha * dz;
    k *= jp[0];
    o[0] -= k * dx;
    o[1] -= k * dy;
    o[2] -= k * dz;
    o[3] -= k * ux;
    o[4] -= k * uy;
    o[5] -= k * uz;
}

/* snap_crackle_kernel_common.h:7-95; ip/jp: m r(3) e2 v(3) a(3) j(3) */
static inline void pair_snap_crackle(const real_t *ip, const real_t *jp,
                                     real_t *o)
{
    real_t dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
    real_t h2 = ip[4] + jp[4];
    real_t ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
    real_t Ax = ip[8] - jp[8], Ay = ip[9] - jp[9], Az = ip[10] - jp[10];
    real_t Jx = ip[11] - jp[11], Jy = ip[12] - jp[12], Jz = ip[13] - jp[13];
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t rv = dx * ux + dy * uy + dz * uz;
    real_t v2 = ux * ux + uy * uy + uz * uz;
    real_t rJ = dx * Jx + dy * Jy + dz * Jz;
    real_t rA = dx * Ax + dy * Ay + dz * Az;
    real_t vA = ux * Ax + uy * Ay + uz * Az;
    real_t q = masked_inv_r2(r2, h2);
    real_t k = q * sqrt(q);

    real_t al = rv * q;
    real_t al2 = al * al;
    real_t be = 3 * ((v2 + rA) * q + al2);
    real_t ga = (3 * vA + rJ) * q + al * (be - 4 * al2);
    al *= 3;
    ga *= 3;

    ux -= al * dx;
    uy -= al * dy;
    uz -= al * dz;

    real_t two_al = 2 * al;
    Ax -= two_al * ux + be * dx;
    Ay -= two_al * uy + be * dy;
    Az -= two_al * uz + be * dz;

    al *= 3;
    be *= 3;
    Jx -= al * Ax + be * ux + ga * dx;
    Jy -= al * Ay + be * uy + ga * dy;
    Jz -= al * Az + be * uz + ga * dz;

    k *= jp[0];
    o[0] -= k * Ax;
    o[1] -= k * Ay;
    o[2] -= k * Az;
    o[3] -= k * Jx;
    o[4] -= k * Jy;
    o[5] -= k * Jz;
}

/* tstep_kernel_common.h:7-60; o[0] = sum of w2, o[1] = max of w2 */
static inline void pair_tstep(real_t eta, const real_t *ip, const real_t *jp,
                              real_t *o)
{
    real_t dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
    real_t h2 = ip[4] + jp[4];
    real_t ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
    real_t msum = ip[0] + jp[0];
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t rv = dx * ux + dy * uy + dz * uz;
    real_t v2 = ux * ux + uy * uy + uz * uz;
    int mask = (r2 > 0);
    real_t q = masked_inv_r2(r2, h2);
    real_t inv_r1 = sqrt(q);

    real_t two = 2;
    real_t b = (1 + two / 2) * q;
    real_t w2 = q;
    real_t g = q;
    real_t phi = msum * inv_r1;
    w2 *= (v2 + two * phi);
    g *= (w2 + b * phi);
    g *= (eta / sqrt(w2));
    w2 -= g * rv;
    w2 = mask ? w2 : (real_t)0;
    o[0] += w2;
    o[1] = fmax(w2, o[1]);
}

/* nreg_kernels_common.h:7-61; o: drx dry drz ax ay az u */
static inline void pair_nreg_x(real_t dt, const real_t *ip, const real_t *jp,
                               real_t *o)
{
    real_t dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
    real_t h2 = ip[4] + jp[4];
    real_t ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
    dx += ux * dt;
    dy += uy * dt;
    dz += uz * dt;
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t q = masked_inv_r2(r2, h2);
    real_t inv_r1 = sqrt(q);
    real_t k = q * inv_r1;
    real_t jm = jp[0];
    k *= jm;
    o[0] += jm * dx;
    o[1] += jm * dy;
    o[2] += jm * dz;
    o[3] -= k * dx;
    o[4] -= k * dy;
    o[5] -= k * dz;
    o[6] += jm * inv_r1;
}

/* nreg_kernels_common.h:63-102; ip/jp: m vx vy vz ax ay az; o: dvx dvy dvz k */
static inline void pair_nreg_v(real_t dt, const real_t *ip, const real_t *jp,
                               real_t *o)
{
    real_t ux = ip[1] - jp[1], uy = ip[2] - jp[2], uz = ip[3] - jp[3];
    real_t wx = ip[4] - jp[4], wy = ip[5] - jp[5], wz = ip[6] - jp[6];
    ux += wx * dt;
    uy += wy * dt;
    uz += wz * dt;
    real_t v2 = ux * ux + uy * uy + uz * uz;
    real_t jm = jp[0];
    o[0] += jm * ux;
    o[1] += jm * uy;
    o[2] += jm * uz;
    o[3] += jm * v2;
}

/* ---------------------------------------------------------------------------
 * Post-Newtonian pair terms (pn_terms.h).  Rational coefficients are formed
 * as (real)(p)/q exactly as the reference's macros do; the expression trees
 * below keep the reference's association so the sums round identically.
 * ------------------------------------------------------------------------- */
#define RQ(p, q) (((real_t)(p)) / (q))
#define PI_SQ ((real_t)(9.869604401089358))

typedef struct { real_t a, b; } pn_t;

/* pn_terms.h:126-152 */
static inline pn_t pn_order2(real_t im, real_t jm, real_t inv_r, real_t iv2,
                             real_t jv2, real_t ivjv, real_t niv, real_t njv,
                             real_t njv2, real_t inv2)
{
    pn_t p;
    p.a = -iv2 - 2 * jv2 + 4 * ivjv + RQ(3, 2) * njv2
          + inv_r * (5 * im + 4 * jm);
    p.b = 4 * niv - 3 * njv;
    p.a *= inv2;
    p.b *= inv2;
    return p;
}

/* pn_terms.h:155-213 */
static inline pn_t pn_order4(real_t im, real_t jm, real_t im2, real_t jm2,
                             real_t imjm, real_t inv_r, real_t inv_r2,
                             real_t iv2, real_t jv2, real_t jv4, real_t ivjv,
                             real_t ivjvivjv, real_t nv, real_t niv,
                             real_t njv, real_t niv2, real_t njv2,
                             real_t nivnjv, real_t inv4)
{
    pn_t p;
    p.a = -2 * (jv4 + ivjvivjv)
          + 4 * jv2 * ivjv
          + njv2 * (RQ(3, 2) * iv2 + RQ(9, 2) * jv2 - 6 * ivjv
                    - RQ(15, 8) * njv2)
          - inv_r2 * (RQ(57, 4) * im2 + 9 * jm2 + RQ(69, 2) * imjm)
          + inv_r * (im * (-RQ(15, 4) * iv2 + RQ(5, 4) * jv2
                           - RQ(5, 2) * ivjv + RQ(39, 2) * niv2
                           - 39 * nivnjv + RQ(17, 2) * njv2)
                     + jm * (4 * jv2 - 8 * ivjv + 2 * niv2
                             - 4 * nivnjv - 6 * njv2));
    p.b = inv_r * (im * (-RQ(63, 4) * niv + RQ(55, 4) * njv)
                   - jm * 2 * (niv + njv))
          + iv2 * njv
          - ivjv * nv * 4
          + jv2 * (4 * niv - 5 * njv)
          + njv2 * (-6 * niv + RQ(9, 2) * njv);
    p.a *= inv4;
    p.b *= inv4;
    return p;
}

/* pn_terms.h:216-237 */
static inline pn_t pn_order5(real_t im, real_t jm, real_t inv_r, real_t v2,
                             real_t nv, real_t inv5)
{
    pn_t p;
    p.a = nv * (inv_r * (-RQ(24, 5) * im + RQ(208, 15) * jm)
                + RQ(12, 5) * v2);
    p.b = -v2 + inv_r * (RQ(8, 5) * im - RQ(32, 5) * jm);
    real_t s = (im * inv_r) * inv5;
    p.a *= s;
    p.b *= s;
    return p;
}

/* pn_terms.h:240-372 */
static inline pn_t pn_order6(real_t im, real_t jm, real_t im2, real_t jm2,
                             real_t imjm, real_t inv_r, real_t inv_r2,
                             real_t v2, real_t iv2, real_t jv2, real_t jv4,
                             real_t ivjv, real_t ivjvivjv, real_t nv,
                             real_t nvnv, real_t niv, real_t njv,
                             real_t niv2, real_t njv2, real_t nivnjv,
                             real_t inv6)
{
    pn_t p;
    real_t t_njv2 =
        njv2 * (3 * ivjvivjv
                + RQ(3, 2) * iv2 * jv2
                - 12 * ivjv * jv2
                + RQ(15, 2) * jv4
                + njv2 * (RQ(15, 2) * (ivjv - jv2 - RQ(1, 4) * iv2)
                          + RQ(35, 16) * njv2));
    real_t t_jv2 = 2 * jv2 * (-ivjvivjv + jv2 * (2 * ivjv - jv2));
    real_t t_im =
        im * inv_r *
        (niv * (njv * (244 * ivjv - RQ(205, 2) * iv2 - RQ(283, 2) * jv2
                       + RQ(383, 2) * njv2)
                + niv * (RQ(229, 4) * (iv2 + jv2 - 2 * ivjv)
                         - RQ(723, 4) * njv2
                         + niv * (RQ(171, 2) * (njv - RQ(1, 4) * niv))))
         + njv2 * (RQ(191, 4) * iv2 + RQ(259, 4) * jv2 - RQ(225, 2) * ivjv
                   - RQ(455, 8) * njv2)
         + ivjv * (RQ(91, 2) * iv2 + 43 * jv2 - RQ(177, 4) * ivjv)
         - RQ(91, 8) * iv2 * (iv2 + 2 * jv2)
         - RQ(81, 8) * jv4);
    real_t t_jm =
        jm * inv_r * 4 *
        (jv4
         + njv * (niv * (ivjv - jv2)
                  + njv * (3 * (ivjv - jv2) - RQ(3, 2) * niv2
                           + njv * (3 * niv + RQ(3, 2) * njv)))
         + ivjv * (ivjv - 2 * jv2));
    real_t t_jm2 = jm2 * inv_r2 *
                   (-niv2 + 2 * nivnjv + RQ(43, 2) * njv2 + 18 * ivjv
                    - 9 * jv2);
    real_t t_imjm = imjm * inv_r2 *
                    (RQ(415, 8) * niv2 - RQ(375, 4) * nivnjv
                     + RQ(1113, 8) * njv2 + 18 * iv2
                     + PI_SQ * (RQ(123, 64) * v2 - RQ(615, 64) * nvnv)
                     + 33 * (ivjv - RQ(1, 2) * jv2));
    real_t t_im2 = im2 * inv_r2 *
                   (-RQ(2069, 8) * niv2 + 543 * nivnjv - RQ(939, 4) * njv2
                    + RQ(471, 8) * iv2 + RQ(357, 8) * (jv2 - 2 * ivjv));
    real_t t_cub = inv_r * inv_r2 *
                   (16 * jm * jm2
                    + im2 * jm * (RQ(547, 3) - RQ(41, 16) * PI_SQ)
                    - RQ(13, 12) * im * im2
                    + im * jm2 * (RQ(545, 3) - RQ(41, 16) * PI_SQ));
    p.a = t_njv2 + t_jv2 + t_im + t_jm + t_jm2 + t_imjm + t_im2 + t_cub;

    real_t u_njv =
        njv * (jv2 * (iv2 + 8 * ivjv - 7 * jv2)
               - 2 * ivjvivjv
               + njv * (6 * niv * (ivjv - 2 * jv2)
                        + njv * (6 * (2 * jv2 - ivjv - RQ(1, 4) * iv2)
                                 + njv * (RQ(15, 2) *
                                          (niv - RQ(3, 4) * njv)))));
    real_t u_niv = 4 * niv * (jv4 - ivjv * jv2);
    real_t u_jm = jm * inv_r *
                  (njv * (4 * (ivjv - jv2 - RQ(1, 2) * niv2)
                          + njv * (2 * (4 * niv + njv)))
                   + 2 * niv * (ivjv - jv2));
    real_t u_im = im * inv_r *
                  (niv * (RQ(207, 8) * iv2 + RQ(81, 8) * jv2 - 36 * ivjv
                          - RQ(269, 4) * njv2
                          + niv * (RQ(565, 4) * njv - RQ(243, 4) * niv))
                   + njv * (RQ(83, 8) * jv2 + RQ(27, 4) * ivjv
                            - RQ(137, 8) * iv2 - RQ(95, 12) * njv2));
    real_t u_r2 = inv_r2 *
                  (jm2 * (4 * niv + 5 * njv)
                   + im2 * (RQ(311, 4) * niv - RQ(357, 4) * njv)
                   + imjm * (RQ(479, 8) * njv - RQ(307, 8) * niv
                             + RQ(123, 32) * PI_SQ * nv));
    p.b = u_njv + u_niv + u_jm + u_im + u_r2;

    p.a *= inv6;
    p.b *= inv6;
    return p;
}

/* pn_terms.h:375-470 */
static inline pn_t pn_order7(real_t im, real_t jm, real_t im2, real_t jm2,
                             real_t imjm, real_t inv_r, real_t inv_r2,
                             real_t v2, real_t iv2, real_t jv2, real_t iv4,
                             real_t jv4, real_t ivjv, real_t nv, real_t nvnv,
                             real_t niv, real_t njv, real_t niv2,
                             real_t njv2, real_t nivnjv, real_t inv7)
{
    pn_t p;
    real_t a_im2 = im2 * inv_r2 * (RQ(3992, 105) * niv - RQ(4328, 105) * njv);
    real_t a_imjm = imjm * inv_r * inv_r2 *
                    (-RQ(13576, 105) * niv + RQ(2872, 21) * njv);
    real_t a_jm2 = jm2 * inv_r * inv_r2 * (-RQ(3172, 21) * nv);
    real_t a_im =
        im * inv_r *
        (niv * (48 * niv2 - RQ(4888, 105) * iv2 + RQ(2056, 21) * ivjv
                - RQ(1028, 21) * jv2)
         + nivnjv * (-RQ(696, 5) * niv + RQ(744, 5) * njv)
         + njv * (-RQ(288, 5) * njv2 + RQ(5056, 105) * iv2
                  - RQ(2224, 21) * ivjv + RQ(5812, 105) * jv2));
    real_t a_jm =
        jm * inv_r *
        (niv * (-RQ(582, 5) * niv2 - RQ(2864, 35) * ivjv
                + RQ(1432, 35) * jv2)
         + nivnjv * (RQ(1746, 5) * niv - RQ(1954, 5) * njv)
         + RQ(3568, 105) * nv * iv2
         + njv * (158 * njv2 - RQ(5752, 105) * jv2
                  + RQ(10048, 105) * ivjv));
    real_t a_v =
        nv * (-56 * nvnv * nvnv - RQ(246, 35) * iv4)
        + niv * (v2 * (60 * niv2 - 180 * nivnjv + 174 * njv2)
                 + ivjv * (RQ(1068, 35) * (iv2 - ivjv) + RQ(984, 35) * jv2)
                 - RQ(534, 35) * iv2 * jv2
                 - RQ(204, 35) * jv4)
        + njv * (-54 * njv2 * v2
                 + ivjv * (-RQ(984, 35) * iv2 + RQ(180, 7) * ivjv
                           - RQ(732, 35) * jv2)
                 + RQ(90, 7) * iv2 * jv2
                 + RQ(24, 7) * jv4);
    p.a = a_im2 + a_imjm + a_jm2 + a_im + a_jm + a_v;

    real_t b_m2 = -im2 * inv_r2 * RQ(184, 21)
                  + imjm * inv_r2 * RQ(6224, 105)
                  + jm2 * inv_r2 * RQ(6388, 105);
    real_t b_im = im * inv_r *
                  (RQ(52, 15) * niv2 - RQ(56, 15) * nivnjv
                   - RQ(44, 15) * njv2 - RQ(132, 35) * iv2
                   + RQ(152, 35) * ivjv - RQ(48, 35) * jv2);
    real_t b_jm = jm * inv_r *
                  (RQ(454, 15) * niv2 - RQ(372, 5) * nivnjv
                   + RQ(854, 15) * njv2 - RQ(152, 21) * iv2
                   + RQ(2864, 105) * ivjv - RQ(1768, 105) * jv2);
    real_t b_v = 60 * nvnv * nvnv
                 + v2 * (-RQ(348, 5) * niv2 + RQ(684, 5) * nivnjv
                         - 66 * njv2)
                 + RQ(334, 35) * iv4
                 + ivjv * (-RQ(1336, 35) * iv2 + RQ(1308, 35) * ivjv
                           - RQ(1252, 35) * jv2)
                 + RQ(654, 35) * iv2 * jv2
                 + RQ(292, 35) * jv4;
    p.b = b_m2 + b_im + b_jm + b_v;

    real_t s = (im * inv_r) * inv7;
    p.a *= s;
    p.b *= s;
    return p;
}

typedef struct {
    uint_t order;
    real_t inv[8];  /* inv[k] = 1/c^k, k = 1..7 */
} clight_t;

/* pn_terms.h:473-567 and pnacc_kernel_common.h:8-70 */
static inline void pair_pnacc(const clight_t *cl, const real_t *ip,
                              const real_t *jp, real_t *o)
{
    real_t im = ip[0], jm = jp[0];
    real_t ivx = ip[5], ivy = ip[6], ivz = ip[7];
    real_t jvx = jp[5], jvy = jp[6], jvz = jp[7];
    real_t dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
    real_t h2 = ip[4] + jp[4];
    real_t ux = ivx - jvx, uy = ivy - jvy, uz = ivz - jvz;
    real_t r2 = dx * dx + dy * dy + dz * dz;
    real_t v2 = ux * ux + uy * uy + uz * uz;
    real_t inv_r2 = masked_inv_r2(r2, h2);
    real_t inv_r = sqrt(inv_r2);
    real_t inv_r3 = inv_r2 * inv_r;

    pn_t p2 = {0, 0}, p4 = {0, 0}, p5 = {0, 0}, p6 = {0, 0}, p7 = {0, 0};
    const pn_t p1 = {0, 0}, p3 = {0, 0};   /* orders 1 and 3 are empty */

    real_t nx = dx * inv_r, ny = dy * inv_r, nz = dz * inv_r;
    real_t iv2 = ivx * ivx + ivy * ivy + ivz * ivz;
    real_t jv2 = jvx * jvx + jvy * jvy + jvz * jvz;

    if (cl->order > 1) {
        real_t niv = nx * ivx + ny * ivy + nz * ivz;
        real_t njv = nx * jvx + ny * jvy + nz * jvz;
        real_t njv2 = njv * njv;
        real_t ivjv = ivx * jvx + ivy * jvy + ivz * jvz;
        p2 = pn_order2(im, jm, inv_r, iv2, jv2, ivjv, niv, njv, njv2,
                       cl->inv[2]);
        if (cl->order > 3) {
            real_t im2 = im * im, jm2 = jm * jm, imjm = im * jm;
            real_t jv4 = jv2 * jv2;
            real_t ivjvivjv = ivjv * ivjv;
            real_t nv = nx * ux + ny * uy + nz * uz;
            real_t niv2 = niv * niv;
            real_t nivnjv = niv * njv;
            p4 = pn_order4(im, jm, im2, jm2, imjm, inv_r, inv_r2, iv2, jv2,
                           jv4, ivjv, ivjvivjv, nv, niv, njv, niv2, njv2,
                           nivnjv, cl->inv[4]);
            if (cl->order > 4) {
                p5 = pn_order5(im, jm, inv_r, v2, nv, cl->inv[5]);
                if (cl->order > 5) {
                    real_t nvnv = nv * nv;
                    p6 = pn_order6(im, jm, im2, jm2, imjm, inv_r, inv_r2, v2,
                                   iv2, jv2, jv4, ivjv, ivjvivjv, nv, nvnv,
                                   niv, njv, niv2, njv2, nivnjv, cl->inv[6]);
                    if (cl->order > 6) {
                        real_t iv4 = iv2 * iv2;
                        p7 = pn_order7(im, jm, im2, jm2, imjm, inv_r, inv_r2,
                                       v2, iv2, jv2, iv4, jv4, ivjv, nv,
                                       nvnv, niv, njv, niv2, njv2, nivnjv,
                                       cl->inv[7]);
                    }
                }
            }
        }
    }
    real_t pa = 0, pb = 0;
    pa += ((((((p7.a + p6.a) + p5.a) + p4.a) + p3.a) + p2.a) + p1.a);
    pb += ((((((p7.b + p6.b) + p5.b) + p4.b) + p3.b) + p2.b) + p1.b);
    pa *= jm * inv_r3;
    pb *= jm * inv_r2;
    o[0] += pa * dx + pb * ux;
    o[1] += pa * dy + pb * uy;
    o[2] += pa * dz + pb * uz;
}

/* ---------------------------------------------------------------------------
 * Universal-variable Kepler solver (universal_kepler_solver.h).
 * ------------------------------------------------------------------------- */
static inline int sgn(real_t x) { return (x > 0) - (x < 0); }

/* Stumpff functions c0..c3 (universal_kepler_solver.h:17-79) */
static inline real_t stumpff0(real_t z)
{
    if (z < 0) return cos(sqrt(-z));
    if (z > 0) return cosh(sqrt(z));
    return 1;
}
static inline real_t stumpff1(real_t z)
{
    if (z < 0) { real_t w = sqrt(-z); return sin(w) / w; }
    if (z > 0) { real_t w = sqrt(z); return sinh(w) / w; }
    return 1;
}
static inline real_t stumpff2(real_t z)
{
    if (z < 0) { real_t w = sqrt(-z); return (cos(w) - 1) / z; }
    if (z > 0) { real_t w = sqrt(z); return (cosh(w) - 1) / z; }
    return 1 / ((real_t)2);
}
static inline real_t stumpff3(real_t z)
{
    if (z < 0) { real_t w = sqrt(-z); return (sin(w) / w - 1) / z; }
    if (z > 0) { real_t w = sqrt(z); return (sinh(w) / w - 1) / z; }
    return 1 / ((real_t)6);
}

/* S0..S3 (universal_kepler_solver.h:82-120) */
static inline real_t uS0(real_t s, real_t al) { real_t s2 = s * s; return stumpff0(al * s2); }
static inline real_t uS1(real_t s, real_t al) { real_t s2 = s * s; return s * stumpff1(al * s2); }
static inline real_t uS2(real_t s, real_t al) { real_t s2 = s * s; return s2 * stumpff2(al * s2); }
static inline real_t uS3(real_t s, real_t al)
{
    real_t s2 = s * s;
    real_t s3 = s * s2;
    return s3 * stumpff3(al * s2);
}

typedef struct { real_t dt, r0, rv0, m, al; } kep_arg_t;

/* universal_kepler and derivatives (universal_kepler_solver.h:166-222) */
static inline real_t kep_f(real_t s, const kep_arg_t *k)
{
    return (k->r0 * s + k->rv0 * uS2(s, k->al) + (k->m + k->al * k->r0) * uS3(s, k->al)) - k->dt;
}
static inline real_t kep_df(real_t s, const kep_arg_t *k)
{
    return k->r0 + k->rv0 * uS1(s, k->al) + (k->m + k->al * k->r0) * uS2(s, k->al);
}
static inline real_t kep_ddf(real_t s, const kep_arg_t *k)
{
    return k->rv0 * uS0(s, k->al) + (k->m + k->al * k->r0) * uS1(s, k->al);
}

/* Laguerre iteration of order 5 (universal_kepler_solver.h:225-254).
 * *iters receives the number of updates applied. */
static int kep_laguerre(real_t x0, real_t *x, const kep_arg_t *k, int *iters)
{
    int it = 0;
    real_t delta;
    *x = x0;
    do {
        real_t fv = kep_f(*x, k);
        real_t dfv = kep_df(*x, k);
        real_t ddfv = kep_ddf(*x, k);
        real_t a = dfv;
        real_t a2 = a * a;
        real_t b = a2 - fv * ddfv;
        real_t g = LAGUERRE_ORDER * fv;
        real_t h = a + sgn(a) * sqrt(fabs((LAGUERRE_ORDER - 1) *
                                          (LAGUERRE_ORDER * b - a2)));
        if (h == 0) { *iters = it; return -1; }
        delta = -g / h;
        (*x) += delta;
        it += 1;
        if (it > KEPLER_MAXITER) { *iters = it; return -2; }
    } while (fabs(delta) > KEPLER_TOL);
    *iters = it;
    if (sgn(*x) != sgn(x0)) return -3;
    return 0;
}

/* set_new_pos_vel (universal_kepler_solver.h:312-357) */
static void kep_update(real_t dt, real_t s, real_t r0, real_t m, real_t e2,
                       real_t al, real_t *p)
{
    real_t r0x = p[0], r0y = p[1], r0z = p[2];
    real_t v0x = p[3], v0y = p[4], v0z = p[5];
    real_t lf = 1 - m * uS2(s, al) / r0;
    real_t lg = dt - m * uS3(s, al);
    real_t r1x = r0x * lf + v0x * lg;
    real_t r1y = r0y * lf + v0y * lg;
    real_t r1z = r0z * lf + v0z * lg;
    real_t r1sq = r1x * r1x + r1y * r1y + r1z * r1z;
    real_t r1 = sqrt(r1sq + e2);
    real_t ldf = -m * uS1(s, al) / (r0 * r1);
    real_t ldg = (1 + lg * ldf) / lf;
    p[0] = r1x;
    p[1] = r1y;
    p[2] = r1z;
    p[3] = r0x * ldf + v0x * ldg;
    p[4] = r0y * ldf + v0y * ldg;
    p[5] = r0z * ldf + v0z * ldg;
}

/* Statistics of the last solve, read by the instrumented entry points. */
typedef struct {
    long solves;      /* calls of the single-step solver */
    long iterations;  /* Laguerre updates summed over solves */
} kep_stats_t;

/* _universal_kepler_solver (universal_kepler_solver.h:360-463).  p holds
 * r(3), v(3) and is updated in place when the root finder succeeds. */
static int kep_single(real_t dt0, real_t m, real_t e2, real_t *p,
                      kep_stats_t *st, real_t *s_root, real_t *s_guess)
{
    if (st && st->solves >= ORACLE_SOLVE_BUDGET) return -4;
    real_t rx = p[0], ry = p[1], rz = p[2];
    real_t vx = p[3], vy = p[4], vz = p[5];
    real_t r2 = rx * rx + ry * ry + rz * rz;
    if (!(r2 > 0)) return 0;
    r2 += e2;
    real_t r = sqrt(r2);
    real_t v2 = vx * vx + vy * vy + vz * vz;
    real_t rv = rx * vx + ry * vy + rz * vz;
    real_t beta = 2 - (e2 / r2);
    real_t al = v2 - beta * m / r;

    real_t dt = dt0;
    if (al < 0) {
        real_t a = m / fabs(al);
        real_t T = 2 * ((real_t)(3.141592653589793)) * a * sqrt(a / m);
        real_t ratio = dt0 / T;
        dt = (ratio - (int_t)(ratio)) * T;
    }
    real_t s0 = dt / r;
    if (al > 0) {
        real_t sal = sqrt(al);
        real_t ss = fabs(2 * al * dt / (rv + (m + al * r) / sal));
        if (ss > 1) s0 = sgn(dt) * log(ss) / sal;
    }
    kep_arg_t k = {dt, r, rv, m, al};
    real_t s;
    int it = 0;
    int err = kep_laguerre(s0, &s, &k, &it);
    if (st) { st->solves += 1; st->iterations += it; }
    if (s_root) *s_root = s;
    if (s_guess) *s_guess = s0;
    if (err == 0) kep_update(dt, s, r, m, e2, al, p);
    return err;
}

/* __universal_kepler_solver (universal_kepler_solver.h:466-507): retry with
 * n equal sub-steps, doubling n while any sub-step fails. */
static void kep_substeps(real_t dt, real_t m, real_t e2, const real_t *p0,
                         real_t *p, kep_stats_t *st)
{
    long n = 1;
    for (int h = 0; h <= ORACLE_MAX_HALVINGS; ++h, n *= 2) {
        for (int c = 0; c < 6; ++c) p[c] = p0[c];
        long i;
        for (i = 0; i < n; ++i) {
            if (kep_single(dt / n, m, e2, p, st, NULL, NULL) != 0) break;
        }
        if (i == n) return;
        if (st && st->solves >= ORACLE_SOLVE_BUDGET) break;
    }
#ifdef _OPENMP
#pragma omp atomic
#endif
    kepler_failures += 1;
}

/* universal_kepler_solver (universal_kepler_solver.h:510-614) */
static void kep_solve(real_t dt, real_t m, real_t e2, const real_t *p0,
                      real_t *p1, kep_stats_t *st_in)
{
    kep_stats_t local = {0, 0};
    kep_stats_t *st = st_in ? st_in : &local;
    real_t p[6];
    kep_substeps(dt, m, e2, p0, p, st);
    if (e2 == 0) {
        for (int c = 0; c < 6; ++c) p1[c] = p[c];
        return;
    }
    real_t r2 = p0[0] * p0[0] + p0[1] * p0[1] + p0[2] * p0[2];
    if (!(r2 > 0)) {
        for (int c = 0; c < 6; ++c) p1[c] = p0[c];
        return;
    }
    r2 += e2;
    real_t r = sqrt(r2);
    real_t v2 = p0[3] * p0[3] + p0[4] * p0[4] + p0[5] * p0[5];
    real_t u0 = 2 * m / r;
    real_t e0 = v2 - u0;

    r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    r2 += e2;
    r = sqrt(r2);
    v2 = p[3] * p[3] + p[4] * p[4] + p[5] * p[5];
    real_t u1 = 2 * m / r;
    real_t e1 = v2 - u1;

    real_t tol = 64 * KEPLER_TOL;
    real_t err = fabs(e1 - e0);
    if (2 * err < tol * (u1 + u0)) {
        for (int c = 0; c < 6; ++c) p1[c] = p[c];
        return;
    }
    long n = 1;
    for (int h = 0; h < ORACLE_MAX_HALVINGS; ++h) {
        n *= 2;
        for (int c = 0; c < 6; ++c) p[c] = p0[c];
        long i;
        for (i = 0; i < n; ++i) {
            real_t q[6];
            for (int c = 0; c < 6; ++c) q[c] = p[c];
            kep_substeps(dt / n, m, e2, q, p, st);
            r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
            r2 += e2;
            r = sqrt(r2);
            v2 = p[3] * p[3] + p[4] * p[4] + p[5] * p[5];
            u1 = 2 * m / r;
            e1 = v2 - u1;
            err = fabs(e1 - e0);
            if (2 * err > tol * (u1 + u0)) break;
        }
        if (i == n) {
            for (int c = 0; c < 6; ++c) p1[c] = p[c];
            return;
        }
        if (st->solves >= ORACLE_SOLVE_BUDGET) break;
    }
#ifdef _OPENMP
#pragma omp atomic
#endif
    kepler_failures += 1;
    for (int c = 0; c < 6; ++c) p1[c] = p[c];
}

/* leapfrog and get_acc (sakura_kernel_common.h:24-91) */
static void two_body_leapfrog(real_t dt, real_t m, real_t e2, const real_t *p0,
                              real_t *p1)
{
    real_t half = dt / 2;
    real_t rx = p0[0], ry = p0[1], rz = p0[2];
    real_t vx = p0[3], vy = p0[4], vz = p0[5];
    rx += vx * half;
    ry += vy * half;
    rz += vz * half;
    real_t r2 = rx * rx + ry * ry + rz * rz;
    real_t q = masked_inv_r2(r2, e2);
    real_t k = q * sqrt(q);
    real_t mk = m * k;
    real_t ax = -mk * rx, ay = -mk * ry, az = -mk * rz;
    vx += ax * dt;
    vy += ay * dt;
    vz += az * dt;
    rx += vx * half;
    ry += vy * half;
    rz += vz * half;
    p1[0] = rx; p1[1] = ry; p1[2] = rz;
    p1[3] = vx; p1[4] = vy; p1[5] = vz;
}

/* twobody_solver (sakura_kernel_common.h:94-123) */
static void two_body(real_t dt, real_t m, real_t e2, const real_t *p0,
                     real_t *p1, kep_stats_t *st, long *n_kepler)
{
    real_t r2 = p0[0] * p0[0] + p0[1] * p0[1] + p0[2] * p0[2];
    real_t v2 = p0[3] * p0[3] + p0[4] * p0[4] + p0[5] * p0[5];
    real_t R = 64 * (m / v2);
    if (r2 > R * R) {
        two_body_leapfrog(dt, m, e2, p0, p1);
    } else {
        if (n_kepler) *n_kepler += 1;
        kep_solve(dt, m, e2, p0, p1, st);
    }
}

/* evolve_twobody (sakura_kernel_common.h:126-191) */
static void evolve_pair(real_t dt, int_t flag, real_t m, real_t e2,
                        const real_t *p0, real_t *p1, kep_stats_t *st,
                        long *n_kepler)
{
    real_t p[6], q[6];
    for (int c = 0; c < 6; ++c) p[c] = p0[c];
    if (flag == -1) {
        p[0] -= p[3] * dt;
        p[1] -= p[4] * dt;
        p[2] -= p[5] * dt;
        two_body(dt, m, e2, p, q, st, n_kepler);
        for (int c = 0; c < 6; ++c) p[c] = q[c];
    }
    if (flag == 1) {
        two_body(dt, m, e2, p, q, st, n_kepler);
        for (int c = 0; c < 6; ++c) p[c] = q[c];
        p[0] -= p[3] * dt;
        p[1] -= p[4] * dt;
        p[2] -= p[5] * dt;
    }
    if (flag == -2) {
        p[0] -= p[3] * dt / 2;
        p[1] -= p[4] * dt / 2;
        p[2] -= p[5] * dt / 2;
        two_body(dt, m, e2, p, q, st, n_kepler);
        for (int c = 0; c < 6; ++c) p[c] = q[c];
        p[0] -= p[3] * dt / 2;
        p[1] -= p[4] * dt / 2;
        p[2] -= p[5] * dt / 2;
    }
    if (flag == 2) {
        two_body(dt / 2, m, e2, p, q, st, n_kepler);
        for (int c = 0; c < 6; ++c) p[c] = q[c];
        p[0] -= p[3] * dt;
        p[1] -= p[4] * dt;
        p[2] -= p[5] * dt;
        two_body(dt / 2, m, e2, p, q, st, n_kepler);
        for (int c = 0; c < 6; ++c) p[c] = q[c];
    }
    for (int c = 0; c < 6; ++c) p1[c] = p[c];
}

/* sakura_kernel_core (sakura_kernel_common.h:194-242) */
static inline void pair_sakura(real_t dt, int_t flag, const real_t *ip,
                               const real_t *jp, real_t *o, kep_stats_t *st,
                               long *n_kepler)
{
    real_t p0[6], p1[6];
    p0[0] = ip[1] - jp[1];
    p0[1] = ip[2] - jp[2];
    p0[2] = ip[3] - jp[3];
    real_t e2 = ip[4] + jp[4];
    p0[3] = ip[5] - jp[5];
    p0[4] = ip[6] - jp[6];
    p0[5] = ip[7] - jp[7];
    real_t m = ip[0] + jp[0];
    evolve_pair(dt, flag, m, e2, p0, p1, st, n_kepler);
    real_t mu = jp[0] / m;
    for (int c = 0; c < 6; ++c) o[c] += mu * (p1[c] - p0[c]);
}

/* ---------------------------------------------------------------------------
 * Entry points: same argument order and meaning as libtupan.h:2-246.
 * ------------------------------------------------------------------------- */
#define LOAD8(dst, k, m, rx, ry, rz, e2, vx, vy, vz)                         \
    do {                                                                     \
        dst[0] = m[k]; dst[1] = rx[k]; dst[2] = ry[k]; dst[3] = rz[k];       \
        dst[4] = e2[k]; dst[5] = vx[k]; dst[6] = vy[k]; dst[7] = vz[k];      \
    } while (0)

void SYM(phi_kernel)(const uint_t ni, const real_t *im, const real_t *irx,
                     const real_t *iry, const real_t *irz, const real_t *ie2,
                     const uint_t nj, const real_t *jm, const real_t *jrx,
                     const real_t *jry, const real_t *jrz, const real_t *je2,
                     real_t *iphi)
{
    (void)im;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t phi = 0;
        for (uint_t j = 0; j < nj; ++j)
            pair_phi(irx[i], iry[i], irz[i], ie2[i], jm[j], jrx[j], jry[j],
                     jrz[j], je2[j], &phi);
        iphi[i] = phi;
    }
}

void SYM(acc_kernel)(const uint_t ni, const real_t *im, const real_t *irx,
                     const real_t *iry, const real_t *irz, const real_t *ie2,
                     const uint_t nj, const real_t *jm, const real_t *jrx,
                     const real_t *jry, const real_t *jrz, const real_t *je2,
                     real_t *iax, real_t *iay, real_t *iaz)
{
    (void)im;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t a[3] = {0, 0, 0};
        for (uint_t j = 0; j < nj; ++j)
            pair_acc(irx[i], iry[i], irz[i], ie2[i], jm[j], jrx[j], jry[j],
                     jrz[j], je2[j], a);
        iax[i] = a[0];
        iay[i] = a[1];
        iaz[i] = a[2];
    }
}

void SYM(acc_jerk_kernel)(
    const uint_t ni, const real_t *im, const real_t *irx, const real_t *iry,
    const real_t *irz, const real_t *ie2, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const uint_t nj, const real_t *jm, const real_t *jrx,
    const real_t *jry, const real_t *jrz, const real_t *je2, const real_t *jvx,
    const real_t *jvy, const real_t *jvz, real_t *iax, real_t *iay,
    real_t *iaz, real_t *ijx, real_t *ijy, real_t *ijz)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[8], jp[8], o[6] = {0, 0, 0, 0, 0, 0};
        LOAD8(ip, i, im, irx, iry, irz, ie2, ivx, ivy, ivz);
        for (uint_t j = 0; j < nj; ++j) {
            LOAD8(jp, j, jm, jrx, jry, jrz, je2, jvx, jvy, jvz);
            pair_acc_jerk(ip, jp, o);
        }
        iax[i] = o[0]; iay[i] = o[1]; iaz[i] = o[2];
        ijx[i] = o[3]; ijy[i] = o[4]; ijz[i] = o[5];
    }
}

void SYM(snap_crackle_kernel)(
    const uint_t ni, const real_t *im, const real_t *irx, const real_t *iry,
    const real_t *irz, const real_t *ie2, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const real_t *iax, const real_t *iay, const real_t *iaz,
    const real_t *ijx, const real_t *ijy, const real_t *ijz, const uint_t nj,
    const real_t *jm, const real_t *jrx, const real_t *jry, const real_t *jrz,
    const real_t *je2, const real_t *jvx, const real_t *jvy, const real_t *jvz,
    const real_t *jax, const real_t *jay, const real_t *jaz, const real_t *jjx,
    const real_t *jjy, const real_t *jjz, real_t *isx, real_t *isy,
    real_t *isz, real_t *icx, real_t *icy, real_t *icz)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[14], jp[14], o[6] = {0, 0, 0, 0, 0, 0};
        LOAD8(ip, i, im, irx, iry, irz, ie2, ivx, ivy, ivz);
        ip[8] = iax[i]; ip[9] = iay[i]; ip[10] = iaz[i];
        ip[11] = ijx[i]; ip[12] = ijy[i]; ip[13] = ijz[i];
        for (uint_t j = 0; j < nj; ++j) {
            LOAD8(jp, j, jm, jrx, jry, jrz, je2, jvx, jvy, jvz);
            jp[8] = jax[j]; jp[9] = jay[j]; jp[10] = jaz[j];
            jp[11] = jjx[j]; jp[12] = jjy[j]; jp[13] = jjz[j];
            pair_snap_crackle(ip, jp, o);
        }
        isx[i] = o[0]; isy[i] = o[1]; isz[i] = o[2];
        icx[i] = o[3]; icy[i] = o[4]; icz[i] = o[5];
    }
}

void SYM(tstep_kernel)(
    const uint_t ni, const real_t *im, const real_t *irx, const real_t *iry,
    const real_t *irz, const real_t *ie2, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const uint_t nj, const real_t *jm, const real_t *jrx,
    const real_t *jry, const real_t *jrz, const real_t *je2, const real_t *jvx,
    const real_t *jvy, const real_t *jvz, const real_t eta, real_t *idt_a,
    real_t *idt_b)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[8], jp[8], o[2] = {0, 0};
        LOAD8(ip, i, im, irx, iry, irz, ie2, ivx, ivy, ivz);
        for (uint_t j = 0; j < nj; ++j) {
            LOAD8(jp, j, jm, jrx, jry, jrz, je2, jvx, jvy, jvz);
            pair_tstep(eta, ip, jp, o);
        }
        /* tstep_kernel.c:46-47 */
        idt_a[i] = eta / sqrt(1 + o[0]);
        idt_b[i] = eta / sqrt(1 + o[1]);
    }
}

void SYM(pnacc_kernel)(
    const uint_t ni, const real_t *im, const real_t *irx, const real_t *iry,
    const real_t *irz, const real_t *ie2, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const uint_t nj, const real_t *jm, const real_t *jrx,
    const real_t *jry, const real_t *jrz, const real_t *je2, const real_t *jvx,
    const real_t *jvy, const real_t *jvz, uint_t order, const real_t inv1,
    const real_t inv2, const real_t inv3, const real_t inv4, const real_t inv5,
    const real_t inv6, const real_t inv7, real_t *ipnax, real_t *ipnay,
    real_t *ipnaz)
{
    clight_t cl = {order, {0, inv1, inv2, inv3, inv4, inv5, inv6, inv7}};
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[8], jp[8], o[3] = {0, 0, 0};
        LOAD8(ip, i, im, irx, iry, irz, ie2, ivx, ivy, ivz);
        for (uint_t j = 0; j < nj; ++j) {
            LOAD8(jp, j, jm, jrx, jry, jrz, je2, jvx, jvy, jvz);
            pair_pnacc(&cl, ip, jp, o);
        }
        ipnax[i] = o[0]; ipnay[i] = o[1]; ipnaz[i] = o[2];
    }
}

void SYM(nreg_Xkernel)(
    const uint_t ni, const real_t *im, const real_t *irx, const real_t *iry,
    const real_t *irz, const real_t *ie2, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const uint_t nj, const real_t *jm, const real_t *jrx,
    const real_t *jry, const real_t *jrz, const real_t *je2, const real_t *jvx,
    const real_t *jvy, const real_t *jvz, const real_t dt, real_t *idrx,
    real_t *idry, real_t *idrz, real_t *iax, real_t *iay, real_t *iaz,
    real_t *iu)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[8], jp[8], o[7] = {0, 0, 0, 0, 0, 0, 0};
        LOAD8(ip, i, im, irx, iry, irz, ie2, ivx, ivy, ivz);
        for (uint_t j = 0; j < nj; ++j) {
            LOAD8(jp, j, jm, jrx, jry, jrz, je2, jvx, jvy, jvz);
            pair_nreg_x(dt, ip, jp, o);
        }
        idrx[i] = o[0]; idry[i] = o[1]; idrz[i] = o[2];
        iax[i] = o[3]; iay[i] = o[4]; iaz[i] = o[5];
        iu[i] = im[i] * o[6];          /* nreg_kernels.c:66 */
    }
}

void SYM(nreg_Vkernel)(
    const uint_t ni, const real_t *im, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const real_t *iax, const real_t *iay, const real_t *iaz,
    const uint_t nj, const real_t *jm, const real_t *jvx, const real_t *jvy,
    const real_t *jvz, const real_t *jax, const real_t *jay, const real_t *jaz,
    const real_t dt, real_t *idvx, real_t *idvy, real_t *idvz, real_t *ik)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[7], jp[7], o[4] = {0, 0, 0, 0};
        ip[0] = im[i]; ip[1] = ivx[i]; ip[2] = ivy[i]; ip[3] = ivz[i];
        ip[4] = iax[i]; ip[5] = iay[i]; ip[6] = iaz[i];
        for (uint_t j = 0; j < nj; ++j) {
            jp[0] = jm[j]; jp[1] = jvx[j]; jp[2] = jvy[j]; jp[3] = jvz[j];
            jp[4] = jax[j]; jp[5] = jay[j]; jp[6] = jaz[j];
            pair_nreg_v(dt, ip, jp, o);
        }
        idvx[i] = o[0]; idvy[i] = o[1]; idvz[i] = o[2];
        ik[i] = im[i] * o[3];          /* nreg_kernels.c:114 */
    }
}

void SYM(sakura_kernel)(
    const uint_t ni, const real_t *im, const real_t *irx, const real_t *iry,
    const real_t *irz, const real_t *ie2, const real_t *ivx, const real_t *ivy,
    const real_t *ivz, const uint_t nj, const real_t *jm, const real_t *jrx,
    const real_t *jry, const real_t *jrz, const real_t *je2, const real_t *jvx,
    const real_t *jvy, const real_t *jvz, const real_t dt, const int_t flag,
    real_t *idrx, real_t *idry, real_t *idrz, real_t *idvx, real_t *idvy,
    real_t *idvz)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < (long)ni; ++i) {
        real_t ip[8], jp[8], o[6] = {0, 0, 0, 0, 0, 0};
        LOAD8(ip, i, im, irx, iry, irz, ie2, ivx, ivy, ivz);
        for (uint_t j = 0; j < nj; ++j) {
            LOAD8(jp, j, jm, jrx, jry, jrz, je2, jvx, jvy, jvz);
            pair_sakura(dt, flag, ip, jp, o, NULL, NULL);
        }
        idrx[i] = o[0]; idry[i] = o[1]; idrz[i] = o[2];
        idvx[i] = o[3]; idvy[i] = o[4]; idvz[i] = o[5];
    }
}

/* kepler_solver_kernel (kepler_solver_kernel.c:5-49, core
 * kepler_solver_kernel_common.h:8-80): two particles, in place allowed. */
void SYM(kepler_solver_kernel)(
    const real_t *im, const real_t *irx, const real_t *iry, const real_t *irz,
    const real_t *ie2, const real_t *ivx, const real_t *ivy, const real_t *ivz,
    const real_t dt, real_t *ir1x, real_t *ir1y, real_t *ir1z, real_t *iv1x,
    real_t *iv1y, real_t *iv1z)
{
    real_t a[8], b[8];
    LOAD8(a, 0, im, irx, iry, irz, ie2, ivx, ivy, ivz);
    LOAD8(b, 1, im, irx, iry, irz, ie2, ivx, ivy, ivz);
    real_t p0[6], p1[6];
    p0[0] = a[1] - b[1];
    p0[1] = a[2] - b[2];
    p0[2] = a[3] - b[3];
    real_t e2 = a[4] + b[4];
    p0[3] = a[5] - b[5];
    p0[4] = a[6] - b[6];
    p0[5] = a[7] - b[7];
    real_t m = a[0] + b[0];
    real_t amu = a[0] / m;
    real_t bmu = b[0] / m;
    real_t cm[6];
    for (int c = 0; c < 3; ++c) cm[c] = amu * a[1 + c] + bmu * b[1 + c];
    for (int c = 0; c < 3; ++c) cm[3 + c] = amu * a[5 + c] + bmu * b[5 + c];
    for (int c = 0; c < 3; ++c) cm[c] += cm[3 + c] * dt;
    kep_solve(dt, m, e2, p0, p1, NULL);
    ir1x[0] = cm[0] + bmu * p1[0];
    ir1y[0] = cm[1] + bmu * p1[1];
    ir1z[0] = cm[2] + bmu * p1[2];
    iv1x[0] = cm[3] + bmu * p1[3];
    iv1y[0] = cm[4] + bmu * p1[4];
    iv1z[0] = cm[5] + bmu * p1[5];
    ir1x[1] = cm[0] - amu * p1[0];
    ir1y[1] = cm[1] - amu * p1[1];
    ir1z[1] = cm[2] - amu * p1[2];
    iv1x[1] = cm[3] - amu * p1[3];
    iv1y[1] = cm[4] - amu * p1[4];
    iv1z[1] = cm[5] - amu * p1[5];
}

/* ---------------------------------------------------------------------------
 * Instrumented helpers (not part of the reference ABI): one universal-Kepler
 * solve per pair with its iteration count, the Laguerre root and the plain
 * starting guess.  Used to build learned-start training data and to report
 * iteration histograms.  p: n x 6 relative states (r, v); out: n x 6.
 * ------------------------------------------------------------------------- */
void SYM(kepler_pairs)(long n, real_t dt, const real_t *m, const real_t *e2,
                       const real_t *p, real_t *out, long *iters,
                       long *solves)
{
#pragma omp parallel for schedule(dynamic, 64)
    for (long k = 0; k < n; ++k) {
        kep_stats_t st = {0, 0};
        kep_solve(dt, m[k], e2[k], p + 6 * k, out + 6 * k, &st);
        if (iters) iters[k] = st.iterations;
        if (solves) solves[k] = st.solves;
    }
}

/* One single-step Laguerre solve from a caller-given start s0 (NaN means
 * the plain guess dt/r).  Returns status per pair, iterations and root. */
void SYM(kepler_root)(long n, real_t dt, const real_t *m, const real_t *e2,
                      const real_t *p, const real_t *s_start, real_t *s_root,
                      real_t *s_plain, int *status, int *iters)
{
#pragma omp parallel for schedule(dynamic, 64)
    for (long k = 0; k < n; ++k) {
        const real_t *q = p + 6 * k;
        real_t mm = m[k], ee = e2[k];
        real_t rx = q[0], ry = q[1], rz = q[2];
        real_t vx = q[3], vy = q[4], vz = q[5];
        real_t r2 = rx * rx + ry * ry + rz * rz + ee;
        real_t r = sqrt(r2);
        real_t v2 = vx * vx + vy * vy + vz * vz;
        real_t rv = rx * vx + ry * vy + rz * vz;
        real_t beta = 2 - (ee / r2);
        real_t al = v2 - beta * mm / r;
        real_t dtt = dt;
        if (al < 0) {
            real_t a = mm / fabs(al);
            real_t T = 2 * ((real_t)(3.141592653589793)) * a * sqrt(a / mm);
            real_t ratio = dt / T;
            dtt = (ratio - (int_t)(ratio)) * T;
        }
        real_t s0 = dtt / r;
        if (al > 0) {
            real_t sal = sqrt(al);
            real_t ss = fabs(2 * al * dtt / (rv + (mm + al * r) / sal));
            if (ss > 1) s0 = sgn(dtt) * log(ss) / sal;
        }
        s_plain[k] = s0;
        real_t start = s_start ? s_start[k] : s0;
        if (start != start) start = s0;
        kep_arg_t ka = {dtt, r, rv, mm, al};
        real_t s;
        int it = 0;
        status[k] = kep_laguerre(start, &s, &ka, &it);
        iters[k] = it;
        s_root[k] = s;
    }
}
