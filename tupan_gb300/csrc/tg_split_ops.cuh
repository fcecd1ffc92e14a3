// Scalar SPLIT-mode pair operators: FP32 pair arithmetic on double-single
// positions (x = xh + xl), shared by the sweep kernels (split.cu) and the
// single-CTA SIA recursion (sia.cu).  Each operator has NF float4 per
// packed record, NO outputs, MAXC (index of a max-reduced output or -1),
// a register image P of a record, pair() accumulating into float acc[NO]
// and finish() in double on the reduced result.

#pragma once

#include "tg_common.cuh"

namespace tg {

__device__ __forceinline__ void split2(double x, float &h, float &l)
{
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
}

// ---------------------------------------------------------------------------
// Pair operators.  Each has:
//   NF   float4 per record, NO outputs, MAXC index of a max-reduced output
//   (or -1), I/J  register images of an i / j record, pair() accumulating
//   into float acc[NO], finish() in double on the reduced result.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float rsqrt_nr(float s)
{
    // MUFU approximation refined by one Newton-Raphson step:
    //   y1 = y0 (3 - s y0^2) / 2
    float y = rsqrtf(s);
    float t = s * y;
    float e = fmaf(-t, y, 1.0f);
    return fmaf(0.5f * y, e, y);
}

struct PhiS {
    static constexpr int NF = 2, NO = 1, MAXC = -1;
    struct P { float xh, yh, zh, m, xl, yl, zl, e2; };
    __device__ static P load(const float4 *r)
    {
        float4 a = r[0], b = r[1];
        return {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    }
    __device__ static void pair(const P &i, const P &j, float *acc, float)
    {
        float dx = (j.xh - i.xh) + (j.xl - i.xl);
        float dy = (j.yh - i.yh) + (j.yl - i.yl);
        float dz = (j.zh - i.zh) + (j.zl - i.zl);
        float h2 = i.e2 + j.e2;
        float s = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, h2)));
        float y = rsqrt_nr(s);
        y = (s > h2) ? y : 0.0f;
        acc[0] = fmaf(-j.m, y, acc[0]);
    }
    __device__ static void finish(double *, double) {}
};

struct AccS {
    static constexpr int NF = 2, NO = 3, MAXC = -1;
    using P = PhiS::P;
    __device__ static P load(const float4 *r) { return PhiS::load(r); }
    __device__ static void pair(const P &i, const P &j, float *acc, float)
    {
        float dx = (j.xh - i.xh) + (j.xl - i.xl);
        float dy = (j.yh - i.yh) + (j.yl - i.yl);
        float dz = (j.zh - i.zh) + (j.zl - i.zl);
        float h2 = i.e2 + j.e2;
        float s = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, h2)));
        float y = rsqrt_nr(s);
        y = (s > h2) ? y : 0.0f;
        float mk = (j.m * y) * (y * y);
        acc[0] = fmaf(mk, dx, acc[0]);
        acc[1] = fmaf(mk, dy, acc[1]);
        acc[2] = fmaf(mk, dz, acc[2]);
    }
    __device__ static void finish(double *, double) {}
};

struct AccJerkS {
    static constexpr int NF = 3, NO = 6, MAXC = -1;
    struct P { float xh, yh, zh, m, xl, yl, zl, e2, vx, vy, vz; };
    __device__ static P load(const float4 *r)
    {
        float4 a = r[0], b = r[1], c = r[2];
        return {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z};
    }
    __device__ static void pair(const P &i, const P &j, float *acc, float)
    {
        float dx = (j.xh - i.xh) + (j.xl - i.xl);
        float dy = (j.yh - i.yh) + (j.yl - i.yl);
        float dz = (j.zh - i.zh) + (j.zl - i.zl);
        float ux = j.vx - i.vx, uy = j.vy - i.vy, uz = j.vz - i.vz;
        float h2 = i.e2 + j.e2;
        float s = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, h2)));
        float rv = fmaf(dz, uz, fmaf(dy, uy, dx * ux));
        float y = rsqrt_nr(s);
        y = (s > h2) ? y : 0.0f;
        float y2 = y * y;
        float mk = (j.m * y) * y2;
        float al = (3.0f * rv) * y2;
        acc[0] = fmaf(mk, dx, acc[0]);
        acc[1] = fmaf(mk, dy, acc[1]);
        acc[2] = fmaf(mk, dz, acc[2]);
        acc[3] = fmaf(mk, fmaf(-al, dx, ux), acc[3]);
        acc[4] = fmaf(mk, fmaf(-al, dy, uy), acc[4]);
        acc[5] = fmaf(mk, fmaf(-al, dz, uz), acc[5]);
    }
    __device__ static void finish(double *, double) {}
};

// tstep_kernel_common.h:7-60 in FP32; output 0 sums w2, output 1 is max w2.
struct TstepS {
    static constexpr int NF = 3, NO = 2, MAXC = 1;
    using P = AccJerkS::P;
    __device__ static P load(const float4 *r) { return AccJerkS::load(r); }
    __device__ static void pair(const P &i, const P &j, float *acc, float eta)
    {
        float dx = (j.xh - i.xh) + (j.xl - i.xl);
        float dy = (j.yh - i.yh) + (j.yl - i.yl);
        float dz = (j.zh - i.zh) + (j.zl - i.zl);
        float ux = j.vx - i.vx, uy = j.vy - i.vy, uz = j.vz - i.vz;
        float h2 = i.e2 + j.e2;
        float msum = i.m + j.m;
        float s = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, h2)));
        float rv = fmaf(dz, uz, fmaf(dy, uy, dx * ux));
        float v2 = fmaf(uz, uz, fmaf(uy, uy, ux * ux));
        float y = rsqrt_nr(s);
        float q = y * y;
        float phi = msum * y;
        float w2 = q * fmaf(2.0f, phi, v2);
        float g = q * fmaf(2.0f * q, phi, w2);
        g *= eta * rsqrt_nr(w2);
        w2 = fmaf(-g, rv, w2);
        w2 = (s > h2) ? w2 : 0.0f;
        acc[0] += w2;
        acc[1] = fmaxf(w2, acc[1]);
    }
    __device__ static void finish(double *v, double eta)
    {
        v[0] = eta / sqrt(1.0 + v[0]);
        v[1] = eta / sqrt(1.0 + v[1]);
    }
};

// snap_crackle_kernel_common.h:7-95 in FP32 (all differences j - i).
struct SnapS {
    static constexpr int NF = 5, NO = 6, MAXC = -1;
    struct P {
        float xh, yh, zh, m, xl, yl, zl, e2, vx, vy, vz, ax, ay, az, jx, jy,
            jz;
    };
    __device__ static P load(const float4 *r)
    {
        float4 a = r[0], b = r[1], c = r[2], d = r[3], e = r[4];
        return {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x,
                c.y, c.z, d.x, d.y, d.z, d.w, e.x, e.y};
    }
    __device__ static void pair(const P &i, const P &j, float *acc, float)
    {
        float dx = (j.xh - i.xh) + (j.xl - i.xl);
        float dy = (j.yh - i.yh) + (j.yl - i.yl);
        float dz = (j.zh - i.zh) + (j.zl - i.zl);
        float ux = j.vx - i.vx, uy = j.vy - i.vy, uz = j.vz - i.vz;
        float Ax = j.ax - i.ax, Ay = j.ay - i.ay, Az = j.az - i.az;
        float Jx = j.jx - i.jx, Jy = j.jy - i.jy, Jz = j.jz - i.jz;
        float h2 = i.e2 + j.e2;
        float s = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, h2)));
        float rv = fmaf(dz, uz, fmaf(dy, uy, dx * ux));
        float v2 = fmaf(uz, uz, fmaf(uy, uy, ux * ux));
        float rJ = fmaf(dz, Jz, fmaf(dy, Jy, dx * Jx));
        float rA = fmaf(dz, Az, fmaf(dy, Ay, dx * Ax));
        float vA = fmaf(uz, Az, fmaf(uy, Ay, ux * Ax));
        float y = rsqrt_nr(s);
        y = (s > h2) ? y : 0.0f;
        float q = y * y;
        float al = rv * q;
        float al2 = al * al;
        float be = 3.0f * fmaf(v2 + rA, q, al2);
        float ga = fmaf(fmaf(3.0f, vA, rJ), q, al * fmaf(-4.0f, al2, be));
        al *= 3.0f;
        ga *= 3.0f;
        ux = fmaf(-al, dx, ux);
        uy = fmaf(-al, dy, uy);
        uz = fmaf(-al, dz, uz);
        float two_al = 2.0f * al;
        Ax -= fmaf(two_al, ux, be * dx);
        Ay -= fmaf(two_al, uy, be * dy);
        Az -= fmaf(two_al, uz, be * dz);
        al *= 3.0f;
        be *= 3.0f;
        Jx -= fmaf(al, Ax, fmaf(be, ux, ga * dx));
        Jy -= fmaf(al, Ay, fmaf(be, uy, ga * dy));
        Jz -= fmaf(al, Az, fmaf(be, uz, ga * dz));
        float mk = (j.m * y) * q;
        acc[0] = fmaf(mk, Ax, acc[0]);
        acc[1] = fmaf(mk, Ay, acc[1]);
        acc[2] = fmaf(mk, Az, acc[2]);
        acc[3] = fmaf(mk, Jx, acc[3]);
        acc[4] = fmaf(mk, Jy, acc[4]);
        acc[5] = fmaf(mk, Jz, acc[5]);
    }
    __device__ static void finish(double *, double) {}
};

}  // namespace tg
