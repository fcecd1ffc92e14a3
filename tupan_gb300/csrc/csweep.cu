// Centred SPLIT sweeps: Phi, Acc and AccJerk over large particle sets
// (phi_kernel_common.h:7-32, acc_kernel_common.h:7-38,
// acc_jerk_kernel_common.h:7-56), with FP32 pair arithmetic and the accuracy
// of the double-single sweeps of split.cu at fewer FP32 operations per
// interaction.
//
//  * The particles are put in Morton order (48-bit keys over the common
//    bounding box of the i and j sets; a stable LSD radix sort of our own),
//    so that 256 consecutive j-particles form a compact tile and 32
//    consecutive i-particles a compact warp.
//  * A j-tile stores its particles relative to a centre c (one float per
//    axis, on a grid common to all tile and warp centres): delta_j = x_j - c
//    as a normalised double-single (dh, dl), formed by ds_sub() from the
//    double-single split of x_j.
//  * Per (warp, tile) each i forms D' = (xh_i - c) + xl_i (within an ulp of
//    x_i - c); the tile is near if some i of the warp lies within 1.25 R of
//    c (R the tile radius), mid if some i lies within 3 R (the reach is
//    settable), else far.  On the N = 262144 Plummer sphere 7.5 % of
//    (warp, tile) pairs are near and 35 % mid.
//  * Far tiles take x_j - x_i = dh_j - D': ONE FP32 operation per axis
//    instead of the three of the double-single difference, and no r2 > 0
//    mask (no pair of a far tile can coincide).  Mid tiles take both
//    positions relative to the warp's centre w instead (also one operation
//    per axis; the tile's positions are shifted to w once per warp and
//    tile).  Near tiles form D = x_i - c with the tile's own ds_sub(), so a
//    particle seen from itself, or from another at the same position,
//    differs by exactly zero, and take the double-single difference
//    (dh_j - Dh) + (dl_j - Dl) and the mask.  ct_diff() gives the emulated
//    accuracy of each form.
//  * The tile is stored field by field (structure of arrays), so one 128-bit
//    shared-memory load gives a field of four j; each packed FP32 operation
//    (FFMA2/FADD2/FMUL2) evaluates one i against two j, and the i operands,
//    constant over a tile, are duplicated into register pairs once per tile
//    instead of duplicating every j operand.
//  * Sums run in FP32 over runs of 64 j per lane half in far and mid tiles
//    (128, a whole tile, for the jerk sums; 4 in near tiles), then fold into
//    a Kahan (sum, correction) pair; the result is formed in
//    double, scattered back to the caller's particle order.  A grid j-split
//    writes partial sums that a second kernel reduces in a fixed order.
//  * Tiles reach shared memory by bulk asynchronous copies (cp.async.bulk)
//    through a three-stage ring of mbarriers; every wait is bounded.

#include <float.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <type_traits>

#include "tg_common.cuh"
#include "tg_split_ops.cuh"
#include "tg_tma.cuh"

namespace tg {

constexpr int CT = 256;           // j-records per tile
constexpr int CT_HDR = 8;         // header floats in front of a tile's fields
constexpr int CT_STAGES = 3;      // shared-memory ring depth
constexpr float CT_NEAR = 1.25f;  // near: some i of the warp within 1.25 R

// Classes of a (warp, tile) pair, from the i of the warp nearest to the
// tile's centre.
enum CtClass : int { CT_FAR = 0, CT_MIDDLE = 1, CT_NEARBY = 2 };

// Fields of a j-record in a tile block (each an array of CT floats).
enum CtField : int {
    F_DHX = 0, F_DHY, F_DHZ, F_DLX, F_DLY, F_DLZ, F_M, F_E2, F_VX, F_VY, F_VZ
};

__host__ __device__ constexpr int ct_nf(int k)
{
    return k == K_ACC_JERK ? 11 : 8;
}

__host__ __device__ constexpr int ct_block_floats(int k)
{
    return CT_HDR + ct_nf(k) * CT;
}

bool centred_supported(int k)
{
    return k == K_PHI || k == K_ACC || k == K_ACC_JERK;
}

// (ah + al) - b as a normalised double-single (h, l): a two-sum of ah and
// -b, then the low word.  Every operation is an explicitly rounded IEEE
// operation (never contracted), so the tile builder and the sweep, which
// both call this on the same inputs, get the same bits.
__device__ __forceinline__ void ds_sub(float ah, float al, float b, float &h,
                                       float &l)
{
    const float s = __fsub_rn(ah, b);
    const float bb = __fsub_rn(s, ah);
    float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(-b, bb));
    e = __fadd_rn(e, al);
    h = __fadd_rn(s, e);
    l = __fsub_rn(e, __fsub_rn(h, s));
}

// ---------------------------------------------------------------------------
// Bounding box and Morton keys.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ord_of(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float float_of_ord(uint32_t o)
{
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// Exponent e of the grid 2^e that tile and warp centres are rounded to,
// from the common bounding box: any multiple of 2^e inside the box (or half
// a step outside it) is an exact float, and so is the difference of any two
// of them (at most 2^20 + 1 steps apart), so the sweep forms c_tile - c_warp
// without rounding.
__device__ __forceinline__ int ct_grid_exp(const uint32_t *box)
{
    float ext = 0.f, amax = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float lo = float_of_ord(box[d]), hi = float_of_ord(box[3 + d]);
        ext = fmaxf(ext, hi - lo);
        amax = fmaxf(amax, fmaxf(fabsf(lo), fabsf(hi)));
    }
    int e1 = 0, e2 = 0;
    frexpf(ext, &e1);     // ext < 2^e1
    frexpf(amax, &e2);    // amax < 2^e2
    int e = max(e1 - 20, e2 - 24);
    return (isfinite(ext) && isfinite(amax)) ? max(e, -100) : 0;
}

// v rounded to the nearest multiple of 2^e (exact float by ct_grid_exp).
__device__ __forceinline__ float ct_round_grid(double v, int e)
{
    return (float)ldexp(rint(ldexp(v, -e)), e);
}

// box[0..2]: ordered minima, box[3..5]: ordered maxima (initialised to
// 0xffffffff and 0 by the host).
__global__ void ct_bbox(const double *x, const double *y, const double *z,
                        uint64_t n, uint32_t *box)
{
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float v[3] = {(float)x[i], (float)y[i], (float)z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            lo[d] = fminf(lo[d], v[d]);
            hi[d] = fmaxf(hi[d], v[d]);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
        }
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            atomicMin(&box[d], ord_of(lo[d]));
            atomicMax(&box[3 + d], ord_of(hi[d]));
        }
}

__device__ __forceinline__ uint64_t spread3(uint32_t v)
{
    uint64_t x = v & 0xffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// 48-bit Morton key of each position on a 2^16 grid per axis over the
// cubic hull of the box; val = the particle's index.
__global__ void ct_keys(const double *x, const double *y, const double *z,
                        uint64_t n, const uint32_t *box, uint64_t *key,
                        uint32_t *val)
{
    double lo[3], ext = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = (double)float_of_ord(box[d]);
        const double e = (double)float_of_ord(box[3 + d]) - lo[d];
        ext = e > ext ? e : ext;
    }
    const double scale = ext > 0.0 ? 65535.0 / ext : 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const double p[3] = {x[i], y[i], z[i]};
        uint32_t q[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double t = (p[d] - lo[d]) * scale;
            t = t > 0.0 ? (t < 65535.0 ? t : 65535.0) : 0.0;   // NaN -> 0
            q[d] = (uint32_t)t;
        }
        key[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
        val[i] = (uint32_t)i;
    }
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (48-bit key, 32-bit value) pairs, 8 bits a pass:
// per-block digit counts, one exclusive scan over (digit, block), then a
// stable scatter (warp-level ranks by __match_any_sync, warps in order).
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_PASSES = 6;

__global__ void __launch_bounds__(RS_THREADS)
rs_count(const uint64_t *key, uint32_t n, int shift, uint32_t *counts)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const uint32_t i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(uint32_t)(key[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan in place of `total` counts, one CTA of 1024 threads.
__global__ void __launch_bounds__(1024)
rs_scan(uint32_t *counts, uint32_t total)
{
    __shared__ uint32_t wsum[32];
    const uint32_t t = threadIdx.x;
    const uint32_t chunk = (total + 1023) / 1024;
    const uint32_t b = t * chunk;
    const uint32_t e = b + chunk < total ? b + chunk : total;
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += counts[i];
    uint32_t incl = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
        if ((t & 31) >= (uint32_t)off) incl += v;
    }
    if ((t & 31) == 31) wsum[t >> 5] = incl;
    __syncthreads();
    if (t < 32) {
        uint32_t w = wsum[t], wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, wi, off);
            if (t >= (uint32_t)off) wi += v;
        }
        wsum[t] = wi - w;
    }
    __syncthreads();
    uint32_t run = wsum[t >> 5] + incl - s;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t c = counts[i];
        counts[i] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(RS_THREADS)
rs_scatter(const uint64_t *kin, const uint32_t *vin, uint64_t *kout,
           uint32_t *vout, uint32_t n, int shift, const uint32_t *offs)
{
    constexpr int NW = RS_THREADS / 32;
    __shared__ uint32_t base_d[256];
    __shared__ uint32_t wcnt[NW][256];
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    base_d[t] = offs[t * gridDim.x + blockIdx.x];
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        for (int d = lane; d < 256; d += 32) wcnt[w][d] = 0;
        __syncthreads();
        const uint32_t i = base + r * RS_THREADS + t;
        const bool ok = i < n;
        const uint64_t k = ok ? kin[i] : 0;
        const uint32_t v = ok ? vin[i] : 0;
        const uint32_t dg = ok ? ((uint32_t)(k >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, dg);
        const uint32_t rank = __popc(peers & lt);
        if (ok && rank == 0) wcnt[w][dg] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = base_d[t];
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                const uint32_t c = wcnt[q][t];
                wcnt[q][t] = run;
                run += c;
            }
            base_d[t] = run;
        }
        __syncthreads();
        if (ok) {
            const uint32_t pos = wcnt[w][dg] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

// Sorts n (key, val) pairs; the result ends in (ka, va) (an even number of
// passes); kb, vb are scratch of n entries, counts 256 x ceil(n / RS_TILE).
static cudaError_t radix_sort(uint64_t *ka, uint32_t *va, uint64_t *kb,
                              uint32_t *vb, uint32_t *counts, uint32_t n,
                              cudaStream_t st)
{
    const uint32_t nb = (n + RS_TILE - 1) / RS_TILE;
    for (int p = 0; p < RS_PASSES; ++p) {
        const int shift = 8 * p;
        uint64_t *ki = (p & 1) ? kb : ka, *ko = (p & 1) ? ka : kb;
        uint32_t *vi = (p & 1) ? vb : va, *vo = (p & 1) ? va : vb;
        rs_count<<<nb, RS_THREADS, 0, st>>>(ki, n, shift, counts);
        rs_scan<<<1, 1024, 0, st>>>(counts, 256u * nb);
        rs_scatter<<<nb, RS_THREADS, 0, st>>>(ki, vi, ko, vo, n, shift,
                                              counts);
        g_launch_count += 3;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Tile blocks and i-records.
// ---------------------------------------------------------------------------
struct CtAttrs {
    const double *a[8];   // m, rx, ry, rz, e2, vx, vy, vz (v: AccJerk only)
};

// One CTA of CT threads per tile: centre (bounding-box midpoint rounded to
// float), double-single offsets, radius, uniform-softening flag, fields.
// Records past nj are padding: zero mass at the centre, which adds exactly
// zero to every Phi / Acc / AccJerk sum.
template <int K>
__global__ void __launch_bounds__(CT)
ct_tiles(const CtAttrs A, uint64_t nj, const uint32_t *perm,
         const uint32_t *box, float *tiles)
{
    constexpr int NF = ct_nf(K), TB = ct_block_floats(K);
    __shared__ double red[6][CT / 32];
    __shared__ float redf[CT / 32];
    __shared__ float cen[3];
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const uint64_t s = (uint64_t)blockIdx.x * CT + t;
    const bool ok = s < nj;
    const uint32_t o0 = perm[(uint64_t)blockIdx.x * CT];
    const uint32_t o = ok ? perm[s] : o0;
    const double p[3] = {A.a[1][o], A.a[2][o], A.a[3][o]};
    double lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = ok ? p[d] : DBL_MAX;
        hi[d] = ok ? p[d] : -DBL_MAX;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
        }
        if (lane == 0) {
            red[d][w] = lo[d];
            red[3 + d][w] = hi[d];
        }
    }
    __syncthreads();
    if (t < 3) {
        double l = red[t][0], h = red[3 + t][0];
        for (int q = 1; q < CT / 32; ++q) {
            l = fmin(l, red[t][q]);
            h = fmax(h, red[3 + t][q]);
        }
        cen[t] = ct_round_grid(0.5 * l + 0.5 * h, ct_grid_exp(box));
    }
    __syncthreads();
    float dh[3] = {0.f, 0.f, 0.f}, dl[3] = {0.f, 0.f, 0.f};
    if (ok)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float xh, xl;
            split2(p[d], xh, xl);
            ds_sub(xh, xl, cen[d], dh[d], dl[d]);
        }
    float r2 = fmaf(dh[2], dh[2], fmaf(dh[1], dh[1], dh[0] * dh[0]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, off));
    if (lane == 0) redf[w] = r2;
    const float e20 = (float)A.a[4][o0];
    const float e2 = ok ? (float)A.a[4][o] : e20;
    const bool uni = __syncthreads_and(e2 == e20);
    float *B = tiles + (uint64_t)blockIdx.x * TB;
    float *F = B + CT_HDR;
    F[F_DHX * CT + t] = dh[0];
    F[F_DHY * CT + t] = dh[1];
    F[F_DHZ * CT + t] = dh[2];
    F[F_DLX * CT + t] = dl[0];
    F[F_DLY * CT + t] = dl[1];
    F[F_DLZ * CT + t] = dl[2];
    F[F_M * CT + t] = ok ? (float)A.a[0][o] : 0.f;
    F[F_E2 * CT + t] = e2;
    if constexpr (NF > 8) {
        F[F_VX * CT + t] = ok ? (float)A.a[5][o] : 0.f;
        F[F_VY * CT + t] = ok ? (float)A.a[6][o] : 0.f;
        F[F_VZ * CT + t] = ok ? (float)A.a[7][o] : 0.f;
    }
    if (t == 0) {
        float m = redf[0];
        for (int q = 1; q < CT / 32; ++q) m = fmaxf(m, redf[q]);
        // an upper bound of max |dh| (sqrtf is correctly rounded; the
        // factor covers the rounding of the sum of squares)
        B[0] = cen[0];
        B[1] = cen[1];
        B[2] = cen[2];
        B[3] = sqrtf(m) * 1.0001f;
        B[4] = e20;
        B[5] = uni ? 1.f : 0.f;
        B[6] = 0.f;
        B[7] = 0.f;
    }
}

// i-records in sorted order: {xh, yh, zh, e2}, {xl, yl, zl, m},
// {vx, vy, vz, 0}.
template <int K>
__global__ void ct_pack_i(const CtAttrs A, uint64_t ni, const uint32_t *perm,
                          float4 *irec)
{
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ni;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o = perm[s];
        float xh, xl, yh, yl, zh, zl;
        split2(A.a[1][o], xh, xl);
        split2(A.a[2][o], yh, yl);
        split2(A.a[3][o], zh, zl);
        irec[3 * s] = make_float4(xh, yh, zh, (float)A.a[4][o]);
        irec[3 * s + 1] = make_float4(xl, yl, zl, (float)A.a[0][o]);
        irec[3 * s + 2] =
            K == K_ACC_JERK
                ? make_float4((float)A.a[5][o], (float)A.a[6][o],
                              (float)A.a[7][o], 0.f)
                : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// ---------------------------------------------------------------------------
// Pair operators on one i and a pair of j (float2 lanes = two j).
// ---------------------------------------------------------------------------
struct CtI {
    float xh[3], xl[3], e2;
    float2 ndh[3], ndl[3], nv[3], h2;   // -(x_i - c) or, mid, -(x_i - w)
};

// j operands of one pair of records
struct CtJ {
    float2 dh[3], dl[3], m, e2, v[3];
};

__device__ __forceinline__ float2 lo2(float4 a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ float2 hi2(float4 a) { return make_float2(a.z, a.w); }

// x_j - x_i.  Near tiles: the double-single difference relative to the
// tile's centre c, (dh_j - Dh) + (dl_j - Dl).  Far tiles: dh_j - D' with
// D' = (xh_i - c) + xl_i rounded, within about an ulp of |x_i - c| of the
// exact D: an error shared by every pair of the tile, so the tile's pull
// on i is evaluated at a slightly shifted point.  Where the tile is close
// (mid tiles, within 3 R) that shift is the largest error left on a
// particle whose net force is a near-cancelling sum, so mid tiles take
// both positions relative to the warp's centre w instead: w_j - W_i,
// w_j = dh_j + (c - w) formed once per warp and tile into shared memory
// (c and w on a common grid, so c - w is exact; one rounding per j),
// W_i = (xh_i - w) + xl_i (small: the warp is compact in Morton order).  Emulated in FP32 on the N = 262144
// Plummer sphere (the 64 particles nearest its centre, pair terms summed
// in fp64): max |da|/|a| 6.5e-6 with the far form everywhere outside
// 1.25 R, 3.0e-6 with the i's low part added within 3 R, 2.0e-6 with the
// double-single difference everywhere.
template <int CLS>
__device__ __forceinline__ void ct_diff(const CtI &i, const CtJ &j,
                                        float2 *d)
{
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if constexpr (CLS == CT_NEARBY)
            d[a] = add2(add2(j.dh[a], i.ndh[a]), add2(j.dl[a], i.ndl[a]));
        else
            d[a] = add2(j.dh[a], i.ndh[a]);
    }
}

// 1/sqrt(s): the MUFU approximation alone; near tiles mask r2 == 0 (self
// pairs, coincident particles).  A Newton step on the near tiles' values
// (y (3/2 - s y^2 / 2)) measured no better on the worst particles of small
// spheres (max |da|/|a| 1.16e-6 with it, 1.44e-6 without on N = 3000, seed
// 12; 6.7e-7 and 9.0e-7 on N = 20000; 9.2e-7 and 7.8e-7 on the 256
// particles nearest the centre of N = 65536) and cost 0.7 % of the AccJerk
// sweep.
template <bool NEAR>
__device__ __forceinline__ float2 ct_rsq(float2 s, float2 h2)
{
    float2 y = make_float2(rsqrtf(s.x), rsqrtf(s.y));
    if constexpr (NEAR) {
        y.x = (s.x > h2.x) ? y.x : 0.0f;
        y.y = (s.y > h2.y) ? y.y : 0.0f;
    }
    return y;
}

struct CtPhi {
    static constexpr int K = K_PHI, NO = 1;
    static constexpr bool VEL = false;
    template <int CLS>
    __device__ static void pair(const CtI &i, const CtJ &j, float2 h2,
                                float2 *acc)
    {
        float2 d[3];
        ct_diff<CLS>(i, j, d);
        const float2 s = fma2(d[2], d[2], fma2(d[1], d[1], fma2(d[0], d[0], h2)));
        const float2 y = ct_rsq<CLS == CT_NEARBY>(s, h2);
        acc[0] = fma2(make_float2(-j.m.x, -j.m.y), y, acc[0]);
    }
};

struct CtAcc {
    static constexpr int K = K_ACC, NO = 3;
    static constexpr bool VEL = false;
    template <int CLS>
    __device__ static void pair(const CtI &i, const CtJ &j, float2 h2,
                                float2 *acc)
    {
        float2 d[3];
        ct_diff<CLS>(i, j, d);
        const float2 s = fma2(d[2], d[2], fma2(d[1], d[1], fma2(d[0], d[0], h2)));
        const float2 y = ct_rsq<CLS == CT_NEARBY>(s, h2);
        const float2 mk = mul2(mul2(j.m, y), mul2(y, y));
        acc[0] = fma2(mk, d[0], acc[0]);
        acc[1] = fma2(mk, d[1], acc[1]);
        acc[2] = fma2(mk, d[2], acc[2]);
    }
};

struct CtAccJerk {
    static constexpr int K = K_ACC_JERK, NO = 6;
    static constexpr bool VEL = true;
    template <int CLS>
    __device__ static void pair(const CtI &i, const CtJ &j, float2 h2,
                                float2 *acc)
    {
        float2 d[3];
        ct_diff<CLS>(i, j, d);
        const float2 ux = add2(j.v[0], i.nv[0]);
        const float2 uy = add2(j.v[1], i.nv[1]);
        const float2 uz = add2(j.v[2], i.nv[2]);
        const float2 s = fma2(d[2], d[2], fma2(d[1], d[1], fma2(d[0], d[0], h2)));
        const float2 rv = fma2(d[2], uz, fma2(d[1], uy, mul2(d[0], ux)));
        const float2 y = ct_rsq<CLS == CT_NEARBY>(s, h2);
        const float2 y2 = mul2(y, y);
        const float2 mk = mul2(mul2(j.m, y), y2);
        const float2 nal = mul2(mul2(rv, dup(-3.0f)), y2);
        acc[0] = fma2(mk, d[0], acc[0]);
        acc[1] = fma2(mk, d[1], acc[1]);
        acc[2] = fma2(mk, d[2], acc[2]);
        acc[3] = fma2(mk, fma2(nal, d[0], ux), acc[3]);
        acc[4] = fma2(mk, fma2(nal, d[1], uy), acc[4]);
        acc[5] = fma2(mk, fma2(nal, d[2], uz), acc[5]);
    }
};

// ---------------------------------------------------------------------------
// The sweep.
// ---------------------------------------------------------------------------
struct CtLaunch {
    const float4 *irec;
    const uint32_t *perm;      // sorted i position -> caller's index
    const float *tiles;
    uint64_t ni;
    uint32_t ntiles, tiles_per_chunk;
    double *out[MAX_OUT];
    double *partial;           // gsplit x NO x ni (grid j-split)
    unsigned *err;
    uint32_t spin;             // main-loop wait limit
    float mid;                 // mid-tile reach in tile radii
    const uint32_t *box;       // common bounding box (centre grid)
};

// Shared memory of a sweep CTA: the tile ring, then per warp a mid tile's
// positions relative to the warp's centre (3 x CT floats).
template <class Op, int NT>
constexpr size_t ct_smem_bytes()
{
    return ((size_t)CT_STAGES * ct_block_floats(Op::K) +
            (size_t)(NT / 32) * 3 * CT) * sizeof(float);
}

template <class Op, int NI, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) ct_sweep(const CtLaunch L)
{
    constexpr int NO = Op::NO, K = Op::K;
    constexpr int TB = ct_block_floats(K);
    static_assert((TB * 4) % 16 == 0, "tile blocks must stay 16-byte aligned");
    extern __shared__ __align__(128) float ct_smem[];
    float *ring = ct_smem;
    __shared__ __align__(8) uint64_t bar[CT_STAGES];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t ibase =
        (uint64_t)blockIdx.x * (NT * NI) + (uint64_t)warp * (32 * NI) + lane;
    const uint32_t t0 = blockIdx.y * L.tiles_per_chunk;
    const uint32_t t1 = t0 + L.tiles_per_chunk < L.ntiles
                            ? t0 + L.tiles_per_chunk : L.ntiles;
    const int nt = t1 > t0 ? (int)(t1 - t0) : 0;

    if (tid == 0) {
        for (int q = 0; q < CT_STAGES; ++q) mbar_init(&bar[q], 1);
        mbar_init_fence();
    }
    __syncthreads();
    auto issue = [&](int t) {
        const uint32_t bytes = (uint32_t)(TB * sizeof(float));
        uint64_t *b = &bar[t % CT_STAGES];
        mbar_arrive_expect_tx(b, bytes);
        bulk_g2s(&ring[(t % CT_STAGES) * TB],
                 L.tiles + (uint64_t)(t0 + t) * TB, bytes, b);
    };
    if (tid == 0)
        for (int q = 0; q < CT_STAGES && q < nt; ++q) issue(q);

    CtI ip[NI];
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        uint64_t s = ibase + 32 * k;
        if (s >= L.ni) s = L.ni - 1;
        const float4 a = L.irec[3 * s], b = L.irec[3 * s + 1];
        ip[k].xh[0] = a.x; ip[k].xh[1] = a.y; ip[k].xh[2] = a.z;
        ip[k].e2 = a.w;
        ip[k].xl[0] = b.x; ip[k].xl[1] = b.y; ip[k].xl[2] = b.z;
        if constexpr (Op::VEL) {
            const float4 c = L.irec[3 * s + 2];
            ip[k].nv[0] = dup(-c.x);
            ip[k].nv[1] = dup(-c.y);
            ip[k].nv[2] = dup(-c.z);
        }
    }
    // the warp's centre w on the tile centres' grid (mid tiles)
    float wc[3];
    {
        const int ge = ct_grid_exp(L.box);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float lo = ip[0].xh[a], hi = ip[0].xh[a];
#pragma unroll
            for (int k = 1; k < NI; ++k) {
                lo = fminf(lo, ip[k].xh[a]);
                hi = fmaxf(hi, ip[k].xh[a]);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
                hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
            }
            wc[a] = ct_round_grid(0.5 * (double)lo + 0.5 * (double)hi, ge);
        }
    }
    float *Wb = ct_smem + CT_STAGES * TB + warp * 3 * CT;

    float sum[NI][NO], corr[NI][NO];
#pragma unroll
    for (int k = 0; k < NI; ++k)
#pragma unroll
        for (int c = 0; c < NO; ++c) sum[k][c] = corr[k][c] = 0.f;

    // One tile: per run of RUNQ quads, two packed pairs per quad and i,
    // then the run folds into the Kahan pairs.  Far tiles run 8 quads (16 j
    // per lane half).  Near tiles hold the i's close neighbours, whose pair
    // terms can exceed the particle's net |a| several times; in Morton order
    // they fall into the same runs, and the FP32 rounding of a run holding
    // them would dominate the error (emulated: max |da|/|a| 1.5e-6 at
    // N = 3000 with 8 quads everywhere, 6.3e-7 with 2 quads in near tiles,
    // which is the pair arithmetic's own floor there), so near tiles fold
    // every 2 quads.
    // Far (and mid) tiles fold the Phi/Acc sums every fourth run (128
    // records) and the jerk sums (outputs 3..5 of AccJerk, whose bound is
    // the loose one) once per tile (256): the terms of a far tile are small
    // next to the running sum.  Emulated with the kernel's order of FP32
    // runs and Kahan folds (N = 262144 sphere, the 24 particles nearest its
    // centre and 24 random ones, mid form): max |da|/|a| 3.35e-6 with
    // 32-record folds, 3.0e-6 with 64; random particles 3.4e-8 and 3.5e-8.
    // On the GPU, 128/256-record folds against 64/128: centre particles of
    // N = 262144 3.4e-6 against 3.8e-6, of N = 2^20 9.0e-7 against 6.3e-7;
    // AccJerk 0.2 % and Acc 0.6 % faster.
    auto run_tile = [&](const float *F, auto cls_tag, auto uni_tag) {
        constexpr int CLS = decltype(cls_tag)::value;
        constexpr bool NEAR = CLS == CT_NEARBY;
        constexpr bool UNI = decltype(uni_tag)::value;
        constexpr int RUNQ = NEAR ? 2 : 8;
        constexpr int PA = NEAR ? 1 : 4;     // runs per fold: Phi, Acc sums
        constexpr int PJ = NEAR ? 1 : 8;     // runs per fold: jerk sums
        static_assert(CT % (4 * RUNQ * PJ) == 0, "a tile ends on a fold");
        float2 p[NI][NO];
#pragma unroll
        for (int k = 0; k < NI; ++k)
#pragma unroll
            for (int c = 0; c < NO; ++c) p[k][c] = make_float2(0.f, 0.f);
#pragma unroll 1
        for (int q0 = 0; q0 < CT; q0 += 4 * RUNQ) {
#pragma unroll
            for (int u = 0; u < RUNQ; ++u) {
                const int r = q0 + 4 * u;
                float4 DH[3], DL[3], M, E2;
                [[maybe_unused]] float4 V[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    DH[a] = CLS == CT_MIDDLE
                                ? *(const float4 *)(Wb + a * CT + r)
                                : *(const float4 *)(F + (F_DHX + a) * CT + r);
                    if constexpr (NEAR)
                        DL[a] = *(const float4 *)(F + (F_DLX + a) * CT + r);
                    if constexpr (Op::VEL)
                        V[a] = *(const float4 *)(F + (F_VX + a) * CT + r);
                }
                M = *(const float4 *)(F + F_M * CT + r);
                if constexpr (!UNI) E2 = *(const float4 *)(F + F_E2 * CT + r);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    CtJ j;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        j.dh[a] = h ? hi2(DH[a]) : lo2(DH[a]);
                        if constexpr (NEAR) j.dl[a] = h ? hi2(DL[a]) : lo2(DL[a]);
                        if constexpr (Op::VEL) j.v[a] = h ? hi2(V[a]) : lo2(V[a]);
                    }
                    j.m = h ? hi2(M) : lo2(M);
                    if constexpr (!UNI) j.e2 = h ? hi2(E2) : lo2(E2);
#pragma unroll
                    for (int k = 0; k < NI; ++k) {
                        const float2 h2 = UNI ? ip[k].h2 : add2(dup(ip[k].e2), j.e2);
                        Op::template pair<CLS>(ip[k], j, h2, p[k]);
                    }
                }
            }
            const int run = q0 / (4 * RUNQ);
            const bool fold_a = (run + 1) % PA == 0;
            const bool fold_j = (run + 1) % PJ == 0;
#pragma unroll
            for (int k = 0; k < NI; ++k)
#pragma unroll
                for (int c = 0; c < NO; ++c) {
                    if (!((NO == 6 && c >= 3) ? fold_j : fold_a)) continue;
                    kahan_add(sum[k][c], corr[k][c], p[k][c].x + p[k][c].y);
                    p[k][c] = make_float2(0.f, 0.f);
                }
        }
    };

    bool ok = true;
    int tfail = 0;
    for (int t = 0; t < nt; ++t) {
        const bool got = mbar_wait_bounded(&bar[t % CT_STAGES],
                                           (uint32_t)((t / CT_STAGES) & 1),
                                           L.err, L.spin);
        if (!__syncthreads_and(got)) {
            ok = false;
            tfail = t;
            break;
        }
        const float *B = &ring[(t % CT_STAGES) * TB];
        const float c[3] = {B[0], B[1], B[2]};
        const float Rn = B[3] * CT_NEAR, Rm = B[3] * L.mid;
        const float lim = fmaxf(Rn * Rn, 1e-30f);
        const float lim_mid = fmaxf(Rm * Rm, 1e-30f);
        const bool uni = B[5] != 0.f;
        // x_i - c to within an ulp, (xh - c) + xl: the class test and the
        // far difference; near tiles redo it exactly below
        bool near = false, mid = false;
#pragma unroll
        for (int k = 0; k < NI; ++k) {
            float dh[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                dh[a] = __fadd_rn(__fsub_rn(ip[k].xh[a], c[a]), ip[k].xl[a]);
                ip[k].ndh[a] = dup(-dh[a]);
            }
            const float d2 = fmaf(dh[2], dh[2], fmaf(dh[1], dh[1], dh[0] * dh[0]));
            near = near || !(d2 > lim);
            mid = mid || !(d2 > lim_mid);
            ip[k].h2 = dup(ip[k].e2 + B[4]);
        }
        near = __any_sync(0xffffffffu, near);
        mid = __any_sync(0xffffffffu, mid);
        const float *F = B + CT_HDR;
        using T_ = std::true_type;
        using F_ = std::false_type;
        using CN = std::integral_constant<int, CT_NEARBY>;
        using CM = std::integral_constant<int, CT_MIDDLE>;
        using CF = std::integral_constant<int, CT_FAR>;
        if (near) {
            // D = x_i - c by the tile's own ds_sub(): a particle seen from
            // itself (or from another at its position) differs by zero
#pragma unroll
            for (int k = 0; k < NI; ++k)
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    float dh, dl;
                    ds_sub(ip[k].xh[a], ip[k].xl[a], c[a], dh, dl);
                    ip[k].ndh[a] = dup(-dh);
                    ip[k].ndl[a] = dup(-dl);
                }
            if (uni) run_tile(F, CN{}, T_{});
            else run_tile(F, CN{}, F_{});
        } else if (mid) {
            // the tile's positions relative to w, once for the warp (c - w
            // exact on the grid): each lane takes float4 quads lane and
            // lane + 32 of each axis; each i relative to w
#pragma unroll
            for (int k = 0; k < NI; ++k)
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    ip[k].ndh[a] = dup(-__fadd_rn(__fsub_rn(ip[k].xh[a], wc[a]),
                                                  ip[k].xl[a]));
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float cwa = c[a] - wc[a];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int q = 4 * (lane + 32 * h);
                    float4 v = *(const float4 *)(F + (F_DHX + a) * CT + q);
                    v.x = __fadd_rn(v.x, cwa);
                    v.y = __fadd_rn(v.y, cwa);
                    v.z = __fadd_rn(v.z, cwa);
                    v.w = __fadd_rn(v.w, cwa);
                    *(float4 *)(Wb + a * CT + q) = v;
                }
            }
            __syncwarp();
            if (uni) run_tile(F, CM{}, T_{});
            else run_tile(F, CM{}, F_{});
        } else {
            if (uni) run_tile(F, CF{}, T_{});
            else run_tile(F, CF{}, F_{});
        }
        __syncthreads();
        if (tid == 0 && t + CT_STAGES < nt) issue(t + CT_STAGES);
    }
    if (!ok) {
        // Copies of tiles tfail .. tfail + CT_STAGES - 1 may still be in
        // flight: wait for each (full bound, its pending parity) before the
        // shared memory goes away, then leave without writing results.
        if (tid == 0)
            for (int u = tfail; u < nt && u < tfail + CT_STAGES; ++u)
                mbar_wait_bounded(&bar[u % CT_STAGES],
                                  (uint32_t)((u / CT_STAGES) & 1), L.err);
        return;
    }
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        const uint64_t s = ibase + 32 * k;
        if (s >= L.ni) continue;
        if (gridDim.y == 1) {
            const uint32_t o = L.perm[s];
#pragma unroll
            for (int c = 0; c < NO; ++c)
                L.out[c][o] = (double)sum[k][c] - (double)corr[k][c];
        } else {
#pragma unroll
            for (int c = 0; c < NO; ++c)
                L.partial[((uint64_t)blockIdx.y * NO + c) * L.ni + s] =
                    (double)sum[k][c] - (double)corr[k][c];
        }
    }
}

// Sum the grid j-split partials in a fixed order and scatter to the
// caller's order; nothing is written if a sweep CTA reported an error.
template <int NO>
__global__ void ct_finalize(const CtLaunch L, int gsplit)
{
    if (*(volatile unsigned *)L.err) return;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
         s < L.ni; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o = L.perm[s];
#pragma unroll
        for (int c = 0; c < NO; ++c) {
            double a = L.partial[(uint64_t)c * L.ni + s];
            for (int y = 1; y < gsplit; ++y)
                a += L.partial[((uint64_t)y * NO + c) * L.ni + s];
            L.out[c][o] = a;
        }
    }
}

// ---------------------------------------------------------------------------
// Host side: workspace layout and the launch sequence.
// ---------------------------------------------------------------------------
struct CtLayout {
    size_t box, key_a, key_b, val_b, counts, perm_i, perm_j, irec, tiles,
        partial, total;
};

static size_t up256(size_t x) { return (x + 255) / 256 * 256; }

static CtLayout ct_layout(int k, uint64_t ni, uint64_t nj, bool same,
                          int gsplit)
{
    const uint64_t nmax = ni > nj ? ni : nj;
    const uint64_t ntiles = (nj + CT - 1) / CT;
    const uint64_t nb = (nmax + RS_TILE - 1) / RS_TILE;
    CtLayout L;
    size_t o = 0;
    L.box = o;     o += 256;
    L.key_a = o;   o += up256(8 * nmax);
    L.key_b = o;   o += up256(8 * nmax);
    L.val_b = o;   o += up256(4 * nmax);
    L.counts = o;  o += up256(4 * 256 * nb);
    L.perm_i = o;  o += up256(4 * ni);
    L.perm_j = same ? L.perm_i : o;
    if (!same) o += up256(4 * nj);
    L.irec = o;    o += up256(48 * ni);
    L.tiles = o;   o += up256(4 * ntiles * (uint64_t)ct_block_floats(k));
    L.partial = o;
    if (gsplit > 1) o += up256(8 * (uint64_t)gsplit * n_out(k) * ni);
    L.total = o;
    return L;
}

size_t centred_workspace_bytes(int k, uint64_t ni, uint64_t nj, bool same,
                               int gsplit)
{
    return ct_layout(k, ni, nj, same, gsplit).total;
}

// Launch shapes of the centred sweep: i per thread, CTAs per SM, threads
// per CTA.
struct CtShape { int ni_per_thread, ctas_per_sm, threads; };
static const CtShape kCtShapes[] = {{1, 2, 256}, {2, 1, 256}, {1, 4, 128}};
constexpr int CT_SHAPES = 3;

int centred_shape_count() { return CT_SHAPES; }

// Grid j-split that balances the waves of a sweep of ni i against ntiles
// tiles: the smallest waves x tiles-per-chunk (ties to the smaller split).
int centred_choose_gsplit(uint64_t ni, uint64_t nj, int shape, int sms)
{
    const uint64_t ntiles = (nj + CT - 1) / CT;
    const CtShape S = kCtShapes[shape];
    const uint64_t ipc = (uint64_t)S.threads * S.ni_per_thread;
    const uint64_t gx = (ni + ipc - 1) / ipc;
    const double cap = (double)sms * S.ctas_per_sm;
    double best = 1e300;
    int bg = 1;
    for (int g = 1; g <= 64; g *= 2) {
        if ((uint64_t)g > ntiles) break;
        const uint64_t tpc = (ntiles + g - 1) / g;
        const uint64_t geff = (ntiles + tpc - 1) / tpc;
        const double waves = ceil((double)gx * geff / cap);
        // a small cost per chunk: the partial-sum traffic and pass
        const double t = waves * (double)tpc + (g > 1 ? 0.25 * g : 0.0);
        if (t < best * 0.999) {
            best = t;
            bg = g;
        }
    }
    return bg;
}

template <class Op, int NI, int NT, int MINB>
static cudaError_t ct_run(const CtLaunch &L, int gsplit, cudaStream_t st)
{
    const uint64_t gx = (L.ni + (uint64_t)NT * NI - 1) / ((uint64_t)NT * NI);
    constexpr size_t smem = ct_smem_bytes<Op, NT>();
    static std::atomic<int> attr{0};
    if (!attr.load()) {
        TG_CUDA_TRY(cudaFuncSetAttribute(
            ct_sweep<Op, NI, NT, MINB>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr.store(1);
    }
    ct_sweep<Op, NI, NT, MINB><<<dim3((unsigned)gx, (unsigned)gsplit), NT,
                                 smem, st>>>(L);
    g_launch_count += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || gsplit == 1) return e;
    uint64_t blocks = (L.ni + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    ct_finalize<Op::NO><<<(unsigned)blocks, 256, 0, st>>>(L, gsplit);
    g_launch_count += 1;
    return cudaGetLastError();
}

static unsigned grid_for(uint64_t n)
{
    uint64_t b = (n + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    return (unsigned)(b ? b : 1);
}

// One centred sweep on device arrays (fp64 SoA in libtupan.h order).  ws is
// a device workspace of centred_workspace_bytes(); shape a launch shape,
// gsplit the grid j-split.
cudaError_t launch_centred(int k, uint64_t ni, const void *const *ia,
                           uint64_t nj, const void *const *ja, bool same,
                           void *const *out, void *ws, int shape, int gsplit,
                           unsigned *err, cudaStream_t st)
{
    if (ni == 0) return cudaSuccess;
    if (!centred_supported(k) || ni > 0xffffffffull || nj > 0xffffffffull ||
        shape < 0 || shape >= CT_SHAPES)
        return cudaErrorInvalidValue;
    if (gsplit < 1) gsplit = 1;
    const uint64_t ntiles = (nj + CT - 1) / CT;
    uint32_t tpc = (uint32_t)((ntiles + gsplit - 1) / gsplit);
    if (tpc == 0) tpc = 1;
    const int geff = ntiles ? (int)((ntiles + tpc - 1) / tpc) : 1;
    const CtLayout Y = ct_layout(k, ni, nj, same, geff);
    char *base = (char *)ws;
    uint32_t *box = (uint32_t *)(base + Y.box);
    uint64_t *ka = (uint64_t *)(base + Y.key_a);
    uint64_t *kb = (uint64_t *)(base + Y.key_b);
    uint32_t *vb = (uint32_t *)(base + Y.val_b);
    uint32_t *counts = (uint32_t *)(base + Y.counts);
    uint32_t *perm_i = (uint32_t *)(base + Y.perm_i);
    uint32_t *perm_j = (uint32_t *)(base + Y.perm_j);
    float4 *irec = (float4 *)(base + Y.irec);
    float *tiles = (float *)(base + Y.tiles);
    CtAttrs AI, AJ;
    const int na = n_attr(k);
    for (int a = 0; a < 8; ++a) {
        AI.a[a] = a < na ? (const double *)ia[a] : nullptr;
        AJ.a[a] = a < na ? (const double *)ja[a] : nullptr;
    }

    // bounding box of both sets, Morton order of each
    TG_CUDA_TRY(cudaMemsetAsync(box, 0xff, 3 * sizeof(uint32_t), st));
    TG_CUDA_TRY(cudaMemsetAsync(box + 3, 0, 3 * sizeof(uint32_t), st));
    ct_bbox<<<grid_for(ni), 256, 0, st>>>(AI.a[1], AI.a[2], AI.a[3], ni, box);
    g_launch_count += 1;
    if (!same && nj) {
        ct_bbox<<<grid_for(nj), 256, 0, st>>>(AJ.a[1], AJ.a[2], AJ.a[3], nj,
                                              box);
        g_launch_count += 1;
    }
    ct_keys<<<grid_for(ni), 256, 0, st>>>(AI.a[1], AI.a[2], AI.a[3], ni, box,
                                          ka, perm_i);
    g_launch_count += 1;
    TG_CUDA_TRY(radix_sort(ka, perm_i, kb, vb, counts, (uint32_t)ni, st));
    if (!same && nj) {
        ct_keys<<<grid_for(nj), 256, 0, st>>>(AJ.a[1], AJ.a[2], AJ.a[3], nj,
                                              box, ka, perm_j);
        g_launch_count += 1;
        TG_CUDA_TRY(radix_sort(ka, perm_j, kb, vb, counts, (uint32_t)nj, st));
    }

    // tiles and i-records
    if (ntiles) {
        switch (k) {
        case K_PHI:
            ct_tiles<K_PHI><<<(unsigned)ntiles, CT, 0, st>>>(AJ, nj, perm_j, box,
                                                    tiles);
            break;
        case K_ACC:
            ct_tiles<K_ACC><<<(unsigned)ntiles, CT, 0, st>>>(AJ, nj, perm_j, box,
                                                    tiles);
            break;
        default:
            ct_tiles<K_ACC_JERK><<<(unsigned)ntiles, CT, 0, st>>>(AJ, nj, perm_j, box,
                                                    tiles);
            break;
        }
        g_launch_count += 1;
    }
    if (k == K_ACC_JERK)
        ct_pack_i<K_ACC_JERK><<<grid_for(ni), 256, 0, st>>>(AI, ni, perm_i, irec);
    else
        ct_pack_i<K_ACC><<<grid_for(ni), 256, 0, st>>>(AI, ni, perm_i, irec);
    g_launch_count += 1;
    TG_CUDA_TRY(cudaGetLastError());

    CtLaunch L;
    memset(&L, 0, sizeof(L));
    L.irec = irec;
    L.perm = perm_i;
    L.tiles = tiles;
    L.ni = ni;
    L.ntiles = (uint32_t)ntiles;
    L.tiles_per_chunk = tpc;
    for (int c = 0; c < MAX_OUT; ++c)
        L.out[c] = c < n_out(k) ? (double *)out[c] : nullptr;
    L.partial = (double *)(base + Y.partial);
    L.err = err;
    L.spin = pipe_spin_limit();
    L.mid = centred_mid_reach();
    L.box = box;
    switch (k * CT_SHAPES + shape) {
    case K_PHI * CT_SHAPES + 0: return ct_run<CtPhi, 1, 256, 2>(L, geff, st);
    case K_PHI * CT_SHAPES + 1: return ct_run<CtPhi, 2, 256, 1>(L, geff, st);
    case K_PHI * CT_SHAPES + 2: return ct_run<CtPhi, 1, 128, 4>(L, geff, st);
    case K_ACC * CT_SHAPES + 0: return ct_run<CtAcc, 1, 256, 2>(L, geff, st);
    case K_ACC * CT_SHAPES + 1: return ct_run<CtAcc, 2, 256, 1>(L, geff, st);
    case K_ACC * CT_SHAPES + 2: return ct_run<CtAcc, 1, 128, 4>(L, geff, st);
    case K_ACC_JERK * CT_SHAPES + 0:
        return ct_run<CtAccJerk, 1, 256, 2>(L, geff, st);
    case K_ACC_JERK * CT_SHAPES + 1:
        return ct_run<CtAccJerk, 2, 256, 1>(L, geff, st);
    default: return ct_run<CtAccJerk, 1, 128, 4>(L, geff, st);
    }
}

}  // namespace tg
