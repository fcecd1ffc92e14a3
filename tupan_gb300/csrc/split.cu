// SPLIT-mode sweeps: FP32 pair arithmetic on double-single positions with
// compensated accumulation, for inputs and outputs in double.
//
//  * Positions are split once per call into hi + lo floats (pack kernel), so
//    x_j - x_i is formed as (xh_j - xh_i) + (xl_j - xl_i): the difference of
//    two nearby positions keeps ~48 bits instead of FP32's 24.
//  * 1/sqrt(r^2 + eps^2) is rsqrt (MUFU) plus one Newton step.
//  * Each lane sums a run of pair terms in FP32, then folds the run into a
//    Kahan-compensated (sum, correction) pair; the final value is formed in
//    double.  j-split lanes of one i are combined with warp shuffles, grid
//    j-splits through a partial-sum buffer reduced in a fixed order.
//  * j-records are staged into shared memory by bulk asynchronous copies
//    (TMA, cp.async.bulk) into a two-stage ring guarded by mbarriers; i-data
//    stay in registers.
//
// The j - i sign convention is used throughout (the reference forms i - j
// and subtracts); every output is the same quantity.

#include <type_traits>

#include "tg_common.cuh"
#include "tg_split_ops.cuh"
#include "tg_tma.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// Packed FP32 particle records (float4 units):
//   [0] = {xh, yh, zh, m}   [1] = {xl, yl, zl, e2}   [2] = {vx, vy, vz, 0}
//   [3] = {ax, ay, az, jx}  [4] = {jy, jz, 0, 0}
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int split_nf(int k)
{
    return (k == K_PHI || k == K_ACC) ? 2 : (k == K_SNAP_CRACKLE ? 5 : 3);
}

struct PackArgs {
    const double *a[MAX_ATTR];
    int na;      // attributes present (5, 8 or 14)
    int nf;      // float4 per record
};

__global__ void pack_records(const PackArgs p, uint64_t n, float4 *out)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float xh, xl, yh, yl, zh, zl;
        split2(p.a[1][i], xh, xl);
        split2(p.a[2][i], yh, yl);
        split2(p.a[3][i], zh, zl);
        float4 *r = out + i * p.nf;
        r[0] = make_float4(xh, yh, zh, (float)p.a[0][i]);
        r[1] = make_float4(xl, yl, zl, (float)p.a[4][i]);
        if (p.nf >= 3)
            r[2] = make_float4((float)p.a[5][i], (float)p.a[6][i],
                               (float)p.a[7][i], 0.f);
        if (p.nf >= 5) {
            r[3] = make_float4((float)p.a[8][i], (float)p.a[9][i],
                               (float)p.a[10][i], (float)p.a[11][i]);
            r[4] = make_float4((float)p.a[12][i], (float)p.a[13][i], 0.f, 0.f);
        }
    }
}

cudaError_t launch_pack(int kernel, uint64_t n, const void *const *attrs,
                        float4 *out, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    PackArgs p;
    p.na = n_attr(kernel);
    p.nf = split_nf(kernel);
    for (int a = 0; a < MAX_ATTR; ++a)
        p.a[a] = a < p.na ? (const double *)attrs[a] : nullptr;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    pack_records<<<(unsigned)blocks, 256, 0, st>>>(p, n, out);
    g_launch_count += 1;
    return cudaGetLastError();
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

struct PhiS2 {
    using P = PhiS::P;
    using I = PosI2;
    __device__ static I pack(const P &a, const P &b)
    {
        return {make_float2(-a.xh, -b.xh), make_float2(-a.yh, -b.yh),
                make_float2(-a.zh, -b.zh), make_float2(-a.xl, -b.xl),
                make_float2(-a.yl, -b.yl), make_float2(-a.zl, -b.zl),
                make_float2(a.e2, b.e2)};
    }
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 h2 = add2(i.e2, dup(j.e2));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 y = rsqrt_nr2(s, h2);
        acc[0] = fma2(dup(-j.m), y, acc[0]);
    }
};

struct AccS2 {
    using P = PhiS::P;
    using I = PosI2;
    __device__ static I pack(const P &a, const P &b) { return PhiS2::pack(a, b); }
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 h2 = add2(i.e2, dup(j.e2));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 y = rsqrt_nr2(s, h2);
        float2 mk = mul2(mul2(dup(j.m), y), mul2(y, y));
        acc[0] = fma2(mk, dx, acc[0]);
        acc[1] = fma2(mk, dy, acc[1]);
        acc[2] = fma2(mk, dz, acc[2]);
    }
};

struct AccJerkS2 {
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
    __device__ static void pair(const I &i, const P &j, float2 *acc, float)
    {
        float2 dx = add2(add2(dup(j.xh), i.nxh), add2(dup(j.xl), i.nxl));
        float2 dy = add2(add2(dup(j.yh), i.nyh), add2(dup(j.yl), i.nyl));
        float2 dz = add2(add2(dup(j.zh), i.nzh), add2(dup(j.zl), i.nzl));
        float2 ux = add2(dup(j.vx), i.nvx);
        float2 uy = add2(dup(j.vy), i.nvy);
        float2 uz = add2(dup(j.vz), i.nvz);
        float2 h2 = add2(i.e2, dup(j.e2));
        float2 s = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, h2)));
        float2 rv = fma2(dz, uz, fma2(dy, uy, mul2(dx, ux)));
        float2 y = rsqrt_nr2(s, h2);
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

struct TstepS2 {
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
        float2 y = rsqrt_nr2_raw(s);
        float2 q = mul2(y, y);
        float2 phi = mul2(msum, y);
        float2 w2 = mul2(q, fma2(dup(2.0f), phi, v2));
        float2 g = mul2(q, fma2(mul2(dup(2.0f), q), phi, w2));
        g = mul2(g, mul2(dup(eta), rsqrt_nr2_raw(w2)));
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

struct SnapS2 {
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
        float2 y = rsqrt_nr2(s, h2);
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
template <> struct X2Of<PhiS> { using type = PhiS2; };
template <> struct X2Of<AccS> { using type = AccS2; };
template <> struct X2Of<AccJerkS> { using type = AccJerkS2; };
template <> struct X2Of<TstepS> { using type = TstepS2; };
template <> struct X2Of<SnapS> { using type = SnapS2; };

// ---------------------------------------------------------------------------
// The sweep kernel.
// ---------------------------------------------------------------------------
struct SplitLaunch {
    const float4 *irec;
    const float4 *jrec;
    uint64_t ni, nj;
    uint64_t jchunk;      // j-particles per grid j-split
    double *out[MAX_OUT]; // final outputs (gsplit == 1)
    double *partial;      // gsplit x NO x ni (gsplit > 1)
    float eta;
    double eta_d;
    unsigned *err;
};

constexpr int SPLIT_TILE = 256;   // j-records per pipeline stage

__device__ __forceinline__ void kahan_add(float &sum, float &corr, float x)
{
    float y = x - corr;
    float t = sum + y;
    corr = (t - sum) - y;
    sum = t;
}

template <class Op, int NI, int JS, int NT, int MINB, bool X2>
__global__ void __launch_bounds__(NT, MINB)
split_sweep(const SplitLaunch L)
{
    using OpX2 = typename X2Of<Op>::type;
    static_assert(!X2 || NI % 2 == 0, "packed variants take i in pairs");
    constexpr int NP = X2 ? NI / 2 : 1;       // packed i pairs per thread
    constexpr int NF = Op::NF, NO = Op::NO, MAXC = Op::MAXC;
    constexpr int NJF = NF;                   // float4 per j-record
    constexpr int TJ = SPLIT_TILE;
    // Records per lane summed in FP32 before a Kahan fold: short runs keep
    // the FP32 rounding of each run small next to the particle's |a|.
    constexpr int FOLD = (TJ / JS) < 16 ? (TJ / JS) : 16;
    static_assert(TJ % (JS * FOLD) == 0, "fold must divide the tile");
    constexpr int GROUPS = NT / JS;          // i-groups per CTA
    constexpr int IPC = GROUPS * NI;         // i-particles per CTA

    __shared__ __align__(128) float4 ring[2][TJ * NJF];
    __shared__ __align__(8) uint64_t bar[2];

    const int tid = threadIdx.x;
    const int js = tid % JS;
    const int grp = tid / JS;
    const uint64_t ibase = (uint64_t)blockIdx.x * IPC + (uint64_t)grp * NI;

    const uint64_t jb = (uint64_t)blockIdx.y * L.jchunk;
    const uint64_t je = jb + L.jchunk < L.nj ? jb + L.jchunk : L.nj;
    const uint64_t jcount = je > jb ? je - jb : 0;
    const int ntiles = (int)((jcount + TJ - 1) / TJ);

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();

    auto issue = [&](int t) {
        const uint64_t j0 = jb + (uint64_t)t * TJ;
        const uint64_t nrec = (je - j0) < (uint64_t)TJ ? (je - j0) : TJ;
        const uint32_t bytes = (uint32_t)(nrec * NJF * sizeof(float4));
        mbar_arrive_expect_tx(&bar[t & 1], bytes);
        bulk_g2s(&ring[t & 1][0], L.jrec + j0 * NJF, bytes, &bar[t & 1]);
    };
    if (tid == 0) {
        if (ntiles > 0) issue(0);
        if (ntiles > 1) issue(1);
    }

    typename Op::P ip[NI];
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        uint64_t i = ibase + k;
        if (i >= L.ni) i = L.ni - 1;
        ip[k] = Op::load(L.irec + i * NF);
    }

    float sum[NI][NO], corr[NI][NO], part[NI][NO];
#pragma unroll
    for (int k = 0; k < NI; ++k)
#pragma unroll
        for (int c = 0; c < NO; ++c) sum[k][c] = corr[k][c] = part[k][c] = 0.f;

    auto fold = [&]() {
#pragma unroll
        for (int k = 0; k < NI; ++k)
#pragma unroll
            for (int c = 0; c < NO; ++c) {
                if (c == MAXC) sum[k][c] = fmaxf(sum[k][c], part[k][c]);
                else kahan_add(sum[k][c], corr[k][c], part[k][c]);
                part[k][c] = 0.f;
            }
    };

    bool ok = true;
    for (int t = 0; t < ntiles; ++t) {
        bool got = mbar_wait_bounded(&bar[t & 1], (uint32_t)((t >> 1) & 1),
                                     L.err);
        if (!__syncthreads_and(got)) { ok = false; break; }
        const float4 *tile = &ring[t & 1][0];
        const uint64_t j0 = jb + (uint64_t)t * TJ;
        const int n = (int)((je - j0) < (uint64_t)TJ ? (je - j0) : TJ);
        if constexpr (X2) {
            // packed path: the i of this thread in pairs, one float2 per
            // quantity and pair
            typename OpX2::I ip2[NP];
#pragma unroll
            for (int q = 0; q < NP; ++q)
                ip2[q] = OpX2::pack(ip[2 * q], ip[2 * q + 1]);
#pragma unroll 1
            for (int r0 = js; r0 < n; r0 += JS * FOLD) {
                float2 p2[NP][NO];
#pragma unroll
                for (int q = 0; q < NP; ++q)
#pragma unroll
                    for (int c = 0; c < NO; ++c) p2[q][c] = make_float2(0.f, 0.f);
                if (n == TJ) {
#pragma unroll
                    for (int u = 0; u < FOLD; ++u) {
                        const typename Op::P jp =
                            Op::load(tile + (r0 + u * JS) * NF);
#pragma unroll
                        for (int q = 0; q < NP; ++q)
                            OpX2::pair(ip2[q], jp, p2[q], L.eta);
                    }
                } else {
#pragma unroll 1
                    for (int u = 0; u < FOLD && r0 + u * JS < n; ++u) {
                        const typename Op::P jp =
                            Op::load(tile + (r0 + u * JS) * NF);
#pragma unroll
                        for (int q = 0; q < NP; ++q)
                            OpX2::pair(ip2[q], jp, p2[q], L.eta);
                    }
                }
#pragma unroll
                for (int q = 0; q < NP; ++q)
#pragma unroll
                    for (int c = 0; c < NO; ++c) {
                        part[(2 * q) % NI][c] = p2[q][c].x;
                        part[(2 * q + 1) % NI][c] = p2[q][c].y;
                    }
                fold();
            }
        } else if (n == TJ) {
#pragma unroll 1
            for (int r0 = 0; r0 < TJ; r0 += JS * FOLD) {
#pragma unroll
                for (int u = 0; u < FOLD; ++u) {
                    const typename Op::P jp =
                        Op::load(tile + (r0 + u * JS + js) * NF);
#pragma unroll
                    for (int k = 0; k < NI; ++k)
                        Op::pair(ip[k], jp, part[k], L.eta);
                }
                fold();
            }
        } else {
#pragma unroll 1
            for (int r = js; r < n; r += JS) {
                const typename Op::P jp = Op::load(tile + r * NF);
#pragma unroll
                for (int k = 0; k < NI; ++k)
                    Op::pair(ip[k], jp, part[k], L.eta);
            }
            fold();
        }
        __syncthreads();
        if (tid == 0 && t + 2 < ntiles) issue(t + 2);
    }
    if (!ok) {
        // A copy did not complete in time: wait (bounded) for whatever is
        // still in flight before the shared memory goes away, then leave
        // without writing results (the host reports the error word).
        if (tid == 0)
            for (int s = 0; s < 2; ++s) mbar_wait_bounded(&bar[s], 0, L.err);
        return;
    }

    // Combine the lanes that share an i (j-split within the warp).
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        double v[NO];
#pragma unroll
        for (int c = 0; c < NO; ++c) {
            v[c] = (c == MAXC) ? (double)sum[k][c]
                               : (double)sum[k][c] - (double)corr[k][c];
#pragma unroll
            for (int off = JS / 2; off > 0; off >>= 1) {
                double w = __shfl_xor_sync(0xffffffffu, v[c], off);
                v[c] = (c == MAXC) ? fmax(v[c], w) : v[c] + w;
            }
        }
        const uint64_t i = ibase + k;
        if (js == 0 && i < L.ni) {
            if (gridDim.y == 1) {
                Op::finish(v, L.eta_d);
#pragma unroll
                for (int c = 0; c < NO; ++c) L.out[c][i] = v[c];
            } else {
#pragma unroll
                for (int c = 0; c < NO; ++c)
                    L.partial[((uint64_t)blockIdx.y * NO + c) * L.ni + i] = v[c];
            }
        }
    }
}

// Reduce grid j-split partials in a fixed order and apply the finish step.
template <class Op>
__global__ void split_finalize(const SplitLaunch L, int gsplit)
{
    constexpr int NO = Op::NO, MAXC = Op::MAXC;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
         i < L.ni; i += (uint64_t)gridDim.x * blockDim.x) {
        double v[NO];
#pragma unroll
        for (int c = 0; c < NO; ++c) {
            double a = L.partial[(uint64_t)c * L.ni + i];
            for (int y = 1; y < gsplit; ++y) {
                double b = L.partial[((uint64_t)y * NO + c) * L.ni + i];
                a = (c == MAXC) ? fmax(a, b) : a + b;
            }
            v[c] = a;
        }
        Op::finish(v, L.eta_d);
#pragma unroll
        for (int c = 0; c < NO; ++c) L.out[c][i] = v[c];
    }
}


// ---------------------------------------------------------------------------
// Batched sweep over an ensemble of independent systems (one persistent
// launch).  System s owns particles [off[s], off[s+1]); each i interacts only
// with the j of its own system.  CTAs take systems from an atomic work queue
// (largest first, by the host-sorted order), stage the system's packed
// records in shared memory with one bulk copy per tile, and give each i
// `lanes` threads (a power of two chosen from the system size) that split
// the j loop and combine through shuffles.  Systems whose `active` flag is 0
// are skipped.
// ---------------------------------------------------------------------------
struct BatchLaunch {
    const float4 *rec;        // packed records of all systems
    const uint64_t *off;      // n_sys + 1 offsets
    const unsigned *order;    // systems in processing order
    const int *active;        // per system (may be null: all active)
    unsigned n_sys;
    const unsigned *n_dev;    // if set: item count in device memory
    const uint2 *items;       // if set: (system, ib | ie << 16) of each
                              // item: the i-block [ib, ie) of the system
    unsigned *queue;          // work counter (zeroed before the launch)
    double *out[MAX_OUT];
    float eta;
    double eta_d;
    unsigned *err;
};

constexpr int BATCH_NT = 256;
constexpr int BATCH_MAXN = 512;           // largest system held in smem

// One system's i-range against all of its j: i-data in registers, j-records
// in shared memory; `lanes` threads share each i (or packed i pair) and
// split the j loop; FP32 runs of 16 terms folded into Kahan sums.
template <class Op, bool X2>
__device__ __forceinline__ void batched_block(const BatchLaunch &L,
                                              const float4 *rec, uint64_t b,
                                              int n, int ib, int ni)
{
    constexpr int NF = Op::NF, NO = Op::NO, MAXC = Op::MAXC;
    constexpr int NI = X2 ? 2 : 1;               // i per thread
    const int tid = threadIdx.x;
    const int units = (ni + NI - 1) / NI;        // i (pairs) of the block
    int lanes = 1;
    while (lanes < 32 && lanes * 2 * units <= BATCH_NT) lanes *= 2;
    const int groups = BATCH_NT / lanes;
    const int lane = tid % lanes;
    for (int u0 = tid / lanes; u0 - tid / lanes < units; u0 += groups) {
        const int u = u0 < units ? u0 : units - 1;
        int iv[NI];
#pragma unroll
        for (int k = 0; k < NI; ++k) {
            const int q = u * NI + k;
            iv[k] = ib + (q < ni ? q : ni - 1);
        }
        float sum[NI][NO], corr[NI][NO], part[NI][NO];
#pragma unroll
        for (int k = 0; k < NI; ++k)
#pragma unroll
            for (int c = 0; c < NO; ++c) sum[k][c] = corr[k][c] = part[k][c] = 0.f;
        auto fold = [&]() {
#pragma unroll
            for (int k = 0; k < NI; ++k)
#pragma unroll
                for (int c = 0; c < NO; ++c) {
                    if (c == MAXC) sum[k][c] = fmaxf(sum[k][c], part[k][c]);
                    else kahan_add(sum[k][c], corr[k][c], part[k][c]);
                    part[k][c] = 0.f;
                }
        };
        if constexpr (X2) {
            using OpX2 = typename X2Of<Op>::type;
            const typename OpX2::I ip2 = OpX2::pack(
                Op::load(rec + iv[0] * NF), Op::load(rec + iv[1] * NF));
            for (int j0 = lane; j0 < n; j0 += 16 * lanes) {
                float2 p2[NO];
#pragma unroll
                for (int c = 0; c < NO; ++c) p2[c] = make_float2(0.f, 0.f);
                const int je = j0 + 16 * lanes < n ? j0 + 16 * lanes : n;
                for (int j = j0; j < je; j += lanes)
                    OpX2::pair(ip2, Op::load(rec + j * NF), p2, L.eta);
#pragma unroll
                for (int c = 0; c < NO; ++c) {
                    part[0][c] = p2[c].x;
                    part[NI - 1][c] = p2[c].y;
                }
                fold();
            }
        } else {
            const typename Op::P ip = Op::load(rec + iv[0] * NF);
            for (int j0 = lane; j0 < n; j0 += 16 * lanes) {
                const int je = j0 + 16 * lanes < n ? j0 + 16 * lanes : n;
                for (int j = j0; j < je; j += lanes)
                    Op::pair(ip, Op::load(rec + j * NF), part[0], L.eta);
                fold();
            }
        }
#pragma unroll
        for (int k = 0; k < NI; ++k) {
            double v[NO];
#pragma unroll
            for (int c = 0; c < NO; ++c) {
                v[c] = (c == MAXC) ? (double)sum[k][c]
                                   : (double)sum[k][c] - (double)corr[k][c];
                for (int o = lanes / 2; o > 0; o >>= 1) {
                    double w = __shfl_xor_sync(0xffffffffu, v[c], o, lanes);
                    v[c] = (c == MAXC) ? fmax(v[c], w) : v[c] + w;
                }
            }
            const int q = u0 * NI + k;
            if (lane == 0 && u0 < units && q < ni) {
                Op::finish(v, L.eta_d);
#pragma unroll
                for (int c = 0; c < NO; ++c) L.out[c][b + iv[k]] = v[c];
            }
        }
    }
}

template <class Op>
__global__ void __launch_bounds__(BATCH_NT, 2)
split_sweep_batched(const BatchLaunch L)
{
    constexpr int NF = Op::NF;
    constexpr bool X2 = !std::is_void<typename X2Of<Op>::type>::value;
    __shared__ __align__(128) float4 rec[BATCH_MAXN * NF];
    __shared__ __align__(8) uint64_t bar;
    __shared__ unsigned item;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    const unsigned n_items = L.n_dev ? *L.n_dev : L.n_sys;
    uint32_t phase = 0;
    for (;;) {
        if (tid == 0) item = atomicAdd(L.queue, 1u);
        __syncthreads();
        const unsigned w = item;
        if (w >= n_items) break;
        const unsigned sys = L.items ? L.items[w].x : L.order[w];
        if (L.active && !L.active[sys]) {
            __syncthreads();
            continue;
        }
        const uint64_t b = L.off[sys];
        const int n = (int)(L.off[sys + 1] - b);
        // i-range of this item: an i-block [ib, ie) or the whole system
        const int ib = L.items ? (int)(L.items[w].y & 0xffffu) : 0;
        const int ie = L.items ? (int)(L.items[w].y >> 16) : n;
        if (n > BATCH_MAXN || ie > n || ib >= ie) {
            if (tid == 0) atomicOr(L.err, (unsigned)DERR_BAD_LAUNCH);
            __syncthreads();
            continue;
        }
        if (tid == 0) {
            const uint32_t bytes = (uint32_t)(n * NF * sizeof(float4));
            mbar_arrive_expect_tx(&bar, bytes);
            bulk_g2s(rec, L.rec + b * NF, bytes, &bar);
        }
        bool got = mbar_wait_bounded(&bar, phase, L.err);
        phase ^= 1u;
        if (!__syncthreads_and(got)) break;
        batched_block<Op, X2>(L, rec, b, n, ib, ie - ib);
        __syncthreads();   // the records of this system are no longer read
    }
}

cudaError_t launch_split_batched(int kernel, const float4 *rec,
                                 const uint64_t *off, const unsigned *order,
                                 const int *active, unsigned n_sys,
                                 unsigned *queue, void *const *out, double eta,
                                 unsigned *err, int sms, cudaStream_t st,
                                 const unsigned *n_dev, const uint2 *items)
{
    BatchLaunch L;
    L.items = items;
    L.rec = rec;
    L.off = off;
    L.order = order;
    L.active = active;
    L.n_sys = n_sys;
    L.n_dev = n_dev;
    L.queue = queue;
    for (int c = 0; c < MAX_OUT; ++c)
        L.out[c] = c < n_out(kernel) ? (double *)out[c] : nullptr;
    L.eta = (float)eta;
    L.eta_d = eta;
    L.err = err;
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    // persistent CTAs; with i-block items (at least 32 i each) a system can
    // occupy up to BATCH_MAXN / 32 of them
    const uint64_t max_items = (uint64_t)n_sys * (items ? BATCH_MAXN / 32 : 1);
    const unsigned grid =
        (unsigned)((uint64_t)sms * 2 < max_items ? (uint64_t)sms * 2 : max_items);
    if (grid == 0) return cudaSuccess;
    switch (kernel) {
    case K_ACC: split_sweep_batched<AccS><<<grid, BATCH_NT, 0, st>>>(L); break;
    case K_ACC_JERK: split_sweep_batched<AccJerkS><<<grid, BATCH_NT, 0, st>>>(L); break;
    case K_TSTEP: split_sweep_batched<TstepS><<<grid, BATCH_NT, 0, st>>>(L); break;
    case K_PHI: split_sweep_batched<PhiS><<<grid, BATCH_NT, 0, st>>>(L); break;
    default: return cudaErrorInvalidValue;
    }
    g_launch_count += 1;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Variant table and launcher.
// ---------------------------------------------------------------------------
struct VariantInfo {
    int ni_per_thread, jsplit, threads;
};

// Variants compiled for every operator; the C-ABI layer picks one.
static const VariantInfo kVariants[] = {
    {2, 1, 256},   // large sweeps: two i per thread, whole warp on one j
    {1, 1, 256},
    {1, 4, 256},   // fewer i: lanes share an i and split the j-tile
    {1, 16, 256},
    {1, 32, 128},
    {2, 1, 256},   // as 0 with packed FP32 pairs
    {2, 4, 256},   // packed, lanes split the j-tile
    {4, 1, 256},   // packed, two pairs per thread (one CTA per SM)
    {2, 1, 256},   // as 5 with the registers of one CTA per SM
};
constexpr int N_VARIANTS = sizeof(kVariants) / sizeof(kVariants[0]);

int split_variant_count() { return N_VARIANTS; }

void split_variant_info(int v, int *ni_per_thread, int *jsplit, int *threads)
{
    *ni_per_thread = kVariants[v].ni_per_thread;
    *jsplit = kVariants[v].jsplit;
    *threads = kVariants[v].threads;
}

// Kernels with a packed-pair (f32x2) operator: variants 5 to 8 use it.
bool split_has_x2(int kernel)
{
    return kernel == K_PHI || kernel == K_ACC || kernel == K_ACC_JERK ||
           kernel == K_TSTEP || kernel == K_SNAP_CRACKLE;
}

bool split_supported(int kernel)
{
    return kernel == K_PHI || kernel == K_ACC || kernel == K_ACC_JERK ||
           kernel == K_TSTEP || kernel == K_SNAP_CRACKLE;
}

template <class Op, int NI, int JS, int NT, int MINB, bool X2 = false>
static cudaError_t run_variant(const SplitLaunch &L, int gsplit,
                               cudaStream_t st)
{
    constexpr uint64_t IPC = (uint64_t)(NT / JS) * NI;
    const uint64_t gx = (L.ni + IPC - 1) / IPC;
    dim3 grid((unsigned)gx, (unsigned)gsplit);
    split_sweep<Op, NI, JS, NT, MINB, X2><<<grid, NT, 0, st>>>(L);
    g_launch_count += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || gsplit == 1) return e;
    uint64_t blocks = (L.ni + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    split_finalize<Op><<<(unsigned)blocks, 256, 0, st>>>(L, gsplit);
    g_launch_count += 1;
    return cudaGetLastError();
}

template <class Op>
static cudaError_t run_op(const SplitLaunch &L, int variant, int gsplit,
                          cudaStream_t st)
{
    switch (variant) {
    case 0: return run_variant<Op, 2, 1, 256, 2>(L, gsplit, st);
    case 1: return run_variant<Op, 1, 1, 256, 2>(L, gsplit, st);
    case 2: return run_variant<Op, 1, 4, 256, 2>(L, gsplit, st);
    case 3: return run_variant<Op, 1, 16, 256, 2>(L, gsplit, st);
    case 4: return run_variant<Op, 1, 32, 128, 4>(L, gsplit, st);
    case 5:
    case 6:
        if constexpr (!std::is_void<typename X2Of<Op>::type>::value) {
            if (variant == 5) return run_variant<Op, 2, 1, 256, 2, true>(L, gsplit, st);
            return run_variant<Op, 2, 4, 256, 2, true>(L, gsplit, st);
        } else {
            if (variant == 5) return run_variant<Op, 2, 1, 256, 2>(L, gsplit, st);
            return run_variant<Op, 1, 4, 256, 2>(L, gsplit, st);
        }
    case 7:
    case 8:
        if constexpr (!std::is_void<typename X2Of<Op>::type>::value) {
            if (variant == 7) return run_variant<Op, 4, 1, 256, 1, true>(L, gsplit, st);
            return run_variant<Op, 2, 1, 256, 1, true>(L, gsplit, st);
        } else {
            return run_variant<Op, 2, 1, 256, 2>(L, gsplit, st);
        }
    default: return cudaErrorInvalidValue;
    }
}

// irec/jrec: packed records (launch_pack); out: NO double arrays;
// partial: gsplit x NO x ni doubles when gsplit > 1.
cudaError_t launch_split(int kernel, const float4 *irec, const float4 *jrec,
                         uint64_t ni, uint64_t nj, void *const *out,
                         double *partial, int variant, int gsplit, double eta,
                         unsigned *err, cudaStream_t st)
{
    if (ni == 0) return cudaSuccess;
    if (gsplit < 1) gsplit = 1;
    SplitLaunch L;
    L.irec = irec;
    L.jrec = jrec;
    L.ni = ni;
    L.nj = nj;
    uint64_t chunk = (nj + gsplit - 1) / gsplit;
    chunk = (chunk + SPLIT_TILE - 1) / SPLIT_TILE * SPLIT_TILE;
    if (chunk == 0) chunk = SPLIT_TILE;
    L.jchunk = chunk;
    for (int c = 0; c < MAX_OUT; ++c)
        L.out[c] = c < n_out(kernel) ? (double *)out[c] : nullptr;
    L.partial = partial;
    L.eta = (float)eta;
    L.eta_d = eta;
    L.err = err;
    switch (kernel) {
    case K_PHI: return run_op<PhiS>(L, variant, gsplit, st);
    case K_ACC: return run_op<AccS>(L, variant, gsplit, st);
    case K_ACC_JERK: return run_op<AccJerkS>(L, variant, gsplit, st);
    case K_TSTEP: return run_op<TstepS>(L, variant, gsplit, st);
    case K_SNAP_CRACKLE: return run_op<SnapS>(L, variant, gsplit, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tg
