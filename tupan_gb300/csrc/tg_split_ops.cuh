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

// 1/sqrt(s): with the Newton step (NR) or the MUFU approximation alone,
// four FP32 operations less per pair.  Measured on an N = 262144 Plummer
// sphere against the fp64 sweep: max |da|/|a| 1.0e-7 without the step,
// 1.3e-7 with it (the step's own FP32 rounding), both inside 1e-6.
template <bool NR>
__device__ __forceinline__ float rsq(float s)
{
    if constexpr (NR) return rsqrt_nr(s);
    else return rsqrtf(s);
}

// Register images of a packed record: position (+ mass, softening) and
// position-velocity.
struct PosRec { float xh, yh, zh, m, xl, yl, zl, e2; };
struct PosVelRec { float xh, yh, zh, m, xl, yl, zl, e2, vx, vy, vz; };

template <bool NR>
struct PhiSN {
    static constexpr int NF = 2, NO = 1, MAXC = -1;
    using P = PosRec;
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
        float y = rsq<NR>(s);
        y = (s > h2) ? y : 0.0f;
        acc[0] = fmaf(-j.m, y, acc[0]);
    }
    __device__ static void finish(double *, double) {}
};
using PhiS = PhiSN<true>;

template <bool NR>
struct AccSN {
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
        float y = rsq<NR>(s);
        y = (s > h2) ? y : 0.0f;
        float mk = (j.m * y) * (y * y);
        acc[0] = fmaf(mk, dx, acc[0]);
        acc[1] = fmaf(mk, dy, acc[1]);
        acc[2] = fmaf(mk, dz, acc[2]);
    }
    __device__ static void finish(double *, double) {}
};
using AccS = AccSN<true>;

template <bool NR>
struct AccJerkSN {
    static constexpr int NF = 3, NO = 6, MAXC = -1;
    using P = PosVelRec;
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
        float y = rsq<NR>(s);
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
using AccJerkS = AccJerkSN<true>;

// tstep_kernel_common.h:7-60 in FP32; output 0 sums w2, output 1 is max w2.
template <bool NR>
struct TstepSN {
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
        float y = rsq<NR>(s);
        float q = y * y;
        float phi = msum * y;
        float w2 = q * fmaf(2.0f, phi, v2);
        float g = q * fmaf(2.0f * q, phi, w2);
        g *= eta * rsq<NR>(w2);
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
using TstepS = TstepSN<true>;

// snap_crackle_kernel_common.h:7-95 in FP32 (all differences j - i).
// Register image of a SnapCrackle record (position, velocity, a, j).
struct SnapRec {
    float xh, yh, zh, m, xl, yl, zl, e2, vx, vy, vz, ax, ay, az, jx, jy,
        jz;
};

template <bool NR>
struct SnapSN {
    static constexpr int NF = 5, NO = 6, MAXC = -1;
    using P = SnapRec;
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
        float y = rsq<NR>(s);
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
using SnapS = SnapSN<true>;

// Kahan-compensated FP32 accumulation of one run of pair terms.
__device__ __forceinline__ void kahan_add(float &sum, float &corr, float x)
{
    float y = x - corr;
    float t = sum + y;
    corr = (t - sum) - y;
    sum = t;
}

// ---------------------------------------------------------------------------
// Two i-particles per thread in packed FP32 (f32x2: .x first i, .y second).
// One FFMA2/FADD2/FMUL2 does the same operation for both i against the same
// j, halving the instructions issued per interaction so that the FMA pipe,
// not instruction issue, bounds the sweep.  i-side positions and velocities
// are kept negated so that every difference is an addition.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// kahan_add on both lanes, operation for operation (b - a is formed as
// fma(a, -1, b): one rounding, the same value as the subtraction).
__device__ __forceinline__ void kahan_add2(float2 &sum, float2 &corr,
                                           float2 x)
{
    const float2 m1 = dup(-1.0f);
    const float2 y = fma2(corr, m1, x);
    const float2 t = add2(sum, y);
    corr = fma2(y, m1, fma2(sum, m1, t));
    sum = t;
}

struct PosI2 { float2 nxh, nyh, nzh, nxl, nyl, nzl, e2; };
struct PosVelI2 { float2 nxh, nyh, nzh, nxl, nyl, nzl, e2, nvx, nvy, nvz; };

// rsqrt with one Newton step on both lanes: y (3/2 - s y^2 / 2), masked to 0
// where s == h2 (r2 == 0: self pairs and coincident particles).
__device__ __forceinline__ float2 rsqrt_nr2(float2 s, float2 h2)
{
    float2 y = make_float2(rsqrtf(s.x), rsqrtf(s.y));
    float2 u = mul2(mul2(s, y), y);
    y = mul2(y, fma2(u, dup(-0.5f), dup(1.5f)));
    y.x = (s.x > h2.x) ? y.x : 0.0f;
    y.y = (s.y > h2.y) ? y.y : 0.0f;
    return y;
}

template <bool NR>
__device__ __forceinline__ float2 rsq2(float2 s, float2 h2)
{
    if constexpr (NR) return rsqrt_nr2(s, h2);
    float2 y = make_float2(rsqrtf(s.x), rsqrtf(s.y));
    y.x = (s.x > h2.x) ? y.x : 0.0f;
    y.y = (s.y > h2.y) ? y.y : 0.0f;
    return y;
}

template <bool NR>
struct PhiS2N {
    using P = PhiS::P;
    using I = PosI2;
    __device__ static I pack(const P &a, const P &b)
    {
        return {make_float2(-a.xh, -b.xh), make_float2(-a.yh, -b.yh),
                make_float2(-a.zh, -b.zh), make_float2(-a.xl, -b.xl),
                make_float2(-a.yl, -b.yl), make_float2(-a.zl, -b.zl),
                make_float2(a.e2, b.e2)};
    }
    static constexpr bool HAS_H2 = true;
    // h2 = e2_i + e2_j given (formed once per tile when the tile's records
    // share one softening)
    __device__ static void pair_h2(const I &i, const P &j, float2 *acc,
                                   float2 h2)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 y = rsq2<NR>(s, h2);
        acc[0] = fma2(dup(-j.m), y, acc[0]);
    }
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        pair_h2(i, j, acc, add2(i.e2, dup(j.e2)));
    }
};

template <bool NR>
struct AccS2N {
    using P = PhiS::P;
    using I = PosI2;
    __device__ static I pack(const P &a, const P &b) { return PhiS2N<NR>::pack(a, b); }
    static constexpr bool HAS_H2 = true;
    __device__ static void pair_h2(const I &i, const P &j, float2 *acc,
                                   float2 h2)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 y = rsq2<NR>(s, h2);
        float2 mk = mul2(mul2(dup(j.m), y), mul2(y, y));
        acc[0] = fma2(mk, dx, acc[0]);
        acc[1] = fma2(mk, dy, acc[1]);
        acc[2] = fma2(mk, dz, acc[2]);
    }
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        pair_h2(i, j, acc, add2(i.e2, dup(j.e2)));
    }
};

template <bool NR>
struct AccJerkS2N {
    using P = AccJerkS::P;
    using I = PosVelI2;
    __device__ static I pack(const P &a, const P &b)
    {
        return {make_float2(-a.xh, -b.xh), make_float2(-a.yh, -b.yh),
                make_float2(-a.zh, -b.zh), make_float2(-a.xl, -b.xl),
                make_float2(-a.yl, -b.yl), make_float2(-a.zl, -b.zl),
                make_float2(a.e2, b.e2),   make_float2(-a.vx, -b.vx),
                make_float2(-a.vy, -b.vy), make_float2(-a.vz, -b.vz)};
    }
    static constexpr bool HAS_H2 = true;
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        pair_h2(i, j, acc, add2(i.e2, dup(j.e2)));
    }
    __device__ static void pair_h2(const I &i, const P &j, float2 *acc,
                                   float2 h2)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 ux = add2(dup(j.vx), i.nvx);
        float2 uy = add2(dup(j.vy), i.nvy);
        float2 uz = add2(dup(j.vz), i.nvz);
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 rv = fma2(dz, uz, fma2(dy, uy, mul2(dx, ux)));
        float2 y = rsq2<NR>(s, h2);
        float2 y2 = mul2(y, y);
        float2 mk = mul2(mul2(dup(j.m), y), y2);
        float2 nal = mul2(mul2(rv, dup(-3.0f)), y2);
        acc[0] = fma2(mk, dx, acc[0]);
        acc[1] = fma2(mk, dy, acc[1]);
        acc[2] = fma2(mk, dz, acc[2]);
        acc[3] = fma2(mk, fma2(nal, dx, ux), acc[3]);
        acc[4] = fma2(mk, fma2(nal, dy, uy), acc[4]);
        acc[5] = fma2(mk, fma2(nal, dz, uz), acc[5]);
    }
};

// Tstep on both lanes (TstepS's arithmetic); the i image also carries m.
struct PosVelMI2 {
    float2 nxh, nyh, nzh, nxl, nyl, nzl, e2, nvx, nvy, nvz, m;
};

__device__ __forceinline__ float2 rsqrt_nr2_raw(float2 s)
{
    float2 y = make_float2(rsqrtf(s.x), rsqrtf(s.y));
    float2 u = mul2(mul2(s, y), y);
    return mul2(y, fma2(u, dup(-0.5f), dup(1.5f)));
}

template <bool NR>
__device__ __forceinline__ float2 rsq2_unmasked(float2 s)
{
    if constexpr (NR) return rsqrt_nr2_raw(s);
    return make_float2(rsqrtf(s.x), rsqrtf(s.y));
}

template <bool NR>
struct TstepS2N {
    static constexpr bool HAS_H2 = false;
    using P = AccJerkS::P;
    using I = PosVelMI2;
    __device__ static I pack(const P &a, const P &b)
    {
        return {make_float2(-a.xh, -b.xh), make_float2(-a.yh, -b.yh),
                make_float2(-a.zh, -b.zh), make_float2(-a.xl, -b.xl),
                make_float2(-a.yl, -b.yl), make_float2(-a.zl, -b.zl),
                make_float2(a.e2, b.e2),   make_float2(-a.vx, -b.vx),
                make_float2(-a.vy, -b.vy), make_float2(-a.vz, -b.vz),
                make_float2(a.m, b.m)};
    }
    __device__ static void pair(const I &i, const P &j, float2 *acc, float eta)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 ux = add2(dup(j.vx), i.nvx);
        float2 uy = add2(dup(j.vy), i.nvy);
        float2 uz = add2(dup(j.vz), i.nvz);
        float2 h2 = add2(i.e2, dup(j.e2));
        float2 msum = add2(i.m, dup(j.m));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 rv = fma2(dz, uz, fma2(dy, uy, mul2(dx, ux)));
        float2 v2 = fma2(uz, uz, fma2(uy, uy, mul2(ux, ux)));
        float2 y = rsq2_unmasked<NR>(s);
        float2 q = mul2(y, y);
        float2 phi = mul2(msum, y);
        float2 w2 = mul2(q, fma2(dup(2.0f), phi, v2));
        float2 g = mul2(q, fma2(mul2(dup(2.0f), q), phi, w2));
        g = mul2(g, mul2(dup(eta), rsq2_unmasked<NR>(w2)));
        w2 = fma2(make_float2(-g.x, -g.y), rv, w2);
        w2.x = (s.x > h2.x) ? w2.x : 0.0f;
        w2.y = (s.y > h2.y) ? w2.y : 0.0f;
        acc[0] = add2(acc[0], w2);
        acc[1] = make_float2(fmaxf(w2.x, acc[1].x), fmaxf(w2.y, acc[1].y));
    }
};

// Snap and crackle on both lanes (SnapS's arithmetic).
struct SnapI2 {
    float2 nxh, nyh, nzh, nxl, nyl, nzl, e2, nvx, nvy, nvz, nax, nay, naz,
        njx, njy, njz;
};

template <bool NR>
struct SnapS2N {
    static constexpr bool HAS_H2 = false;
    using P = SnapS::P;
    using I = SnapI2;
    __device__ static I pack(const P &a, const P &b)
    {
        return {make_float2(-a.xh, -b.xh), make_float2(-a.yh, -b.yh),
                make_float2(-a.zh, -b.zh), make_float2(-a.xl, -b.xl),
                make_float2(-a.yl, -b.yl), make_float2(-a.zl, -b.zl),
                make_float2(a.e2, b.e2),   make_float2(-a.vx, -b.vx),
                make_float2(-a.vy, -b.vy), make_float2(-a.vz, -b.vz),
                make_float2(-a.ax, -b.ax), make_float2(-a.ay, -b.ay),
                make_float2(-a.az, -b.az), make_float2(-a.jx, -b.jx),
                make_float2(-a.jy, -b.jy), make_float2(-a.jz, -b.jz)};
    }
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 ux = add2(dup(j.vx), i.nvx);
        float2 uy = add2(dup(j.vy), i.nvy);
        float2 uz = add2(dup(j.vz), i.nvz);
        float2 Ax = add2(dup(j.ax), i.nax);
        float2 Ay = add2(dup(j.ay), i.nay);
        float2 Az = add2(dup(j.az), i.naz);
        float2 Jx = add2(dup(j.jx), i.njx);
        float2 Jy = add2(dup(j.jy), i.njy);
        float2 Jz = add2(dup(j.jz), i.njz);
        float2 h2 = add2(i.e2, dup(j.e2));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 rv = fma2(dz, uz, fma2(dy, uy, mul2(dx, ux)));
        float2 v2 = fma2(uz, uz, fma2(uy, uy, mul2(ux, ux)));
        float2 rJ = fma2(dz, Jz, fma2(dy, Jy, mul2(dx, Jx)));
        float2 rA = fma2(dz, Az, fma2(dy, Ay, mul2(dx, Ax)));
        float2 vA = fma2(uz, Az, fma2(uy, Ay, mul2(ux, Ax)));
        float2 y = rsq2<NR>(s, h2);
        float2 q = mul2(y, y);
        float2 al = mul2(rv, q);
        float2 al2 = mul2(al, al);
        float2 be = mul2(dup(3.0f), fma2(add2(v2, rA), q, al2));
        float2 ga = fma2(fma2(dup(3.0f), vA, rJ), q,
                         mul2(al, fma2(dup(-4.0f), al2, be)));
        al = mul2(al, dup(3.0f));
        ga = mul2(ga, dup(3.0f));
        const float2 nal = make_float2(-al.x, -al.y);
        ux = fma2(nal, dx, ux);
        uy = fma2(nal, dy, uy);
        uz = fma2(nal, dz, uz);
        float2 two_al = mul2(dup(2.0f), al);
        float2 tx = fma2(two_al, ux, mul2(be, dx));
        float2 ty = fma2(two_al, uy, mul2(be, dy));
        float2 tz = fma2(two_al, uz, mul2(be, dz));
        Ax = add2(Ax, make_float2(-tx.x, -tx.y));
        Ay = add2(Ay, make_float2(-ty.x, -ty.y));
        Az = add2(Az, make_float2(-tz.x, -tz.y));
        al = mul2(al, dup(3.0f));
        be = mul2(be, dup(3.0f));
        float2 kx = fma2(al, Ax, fma2(be, ux, mul2(ga, dx)));
        float2 ky = fma2(al, Ay, fma2(be, uy, mul2(ga, dy)));
        float2 kz = fma2(al, Az, fma2(be, uz, mul2(ga, dz)));
        Jx = add2(Jx, make_float2(-kx.x, -kx.y));
        Jy = add2(Jy, make_float2(-ky.x, -ky.y));
        Jz = add2(Jz, make_float2(-kz.x, -kz.y));
        float2 mk = mul2(mul2(dup(j.m), y), q);
        acc[0] = fma2(mk, Ax, acc[0]);
        acc[1] = fma2(mk, Ay, acc[1]);
        acc[2] = fma2(mk, Az, acc[2]);
        acc[3] = fma2(mk, Jx, acc[3]);
        acc[4] = fma2(mk, Jy, acc[4]);
        acc[5] = fma2(mk, Jz, acc[5]);
    }
};

// Packed-pair partner of each scalar operator (void: none).
template <class Op> struct X2Of { using type = void; };
template <bool NR> struct X2Of<PhiSN<NR>> { using type = PhiS2N<NR>; };
template <bool NR> struct X2Of<AccSN<NR>> { using type = AccS2N<NR>; };
template <bool NR> struct X2Of<AccJerkSN<NR>> { using type = AccJerkS2N<NR>; };
template <bool NR> struct X2Of<TstepSN<NR>> { using type = TstepS2N<NR>; };
template <bool NR> struct X2Of<SnapSN<NR>> { using type = SnapS2N<NR>; };

}  // namespace tg
