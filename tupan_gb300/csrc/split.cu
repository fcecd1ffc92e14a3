// SPLIT-mode sweeps: FP32 pair arithmetic on double-single positions with
// compensated accumulation, for inputs and outputs in double.
//
//  * Positions are split once per call into hi + lo floats (pack kernel), so
//    x_j - x_i is formed as (xh_j - xh_i) + (xl_j - xl_i): the difference of
//    two nearby positions keeps ~48 bits instead of FP32's 24.
//  * 1/sqrt(r^2 + eps^2) is the MUFU rsqrt alone (variants 9-11, the
//    default) or rsqrt plus one Newton step (variants 0-8).
//  * Each lane sums a run of pair terms in FP32, then folds the run into a
//    Kahan-compensated (sum, correction) pair; the final value is formed in
//    double.  j-split lanes of one i are combined with warp shuffles, grid
//    j-splits through a partial-sum buffer reduced in a fixed order.
//  * j-records are staged into shared memory by bulk asynchronous copies
//    (TMA, cp.async.bulk) into a two-stage ring guarded by mbarriers; i-data
//    stay in registers.
//
// Phi, Acc and AccJerk sweeps of at least 2^31 interactions take the
// centred kernels of csweep.cu instead (run_device_sweep in abi.cu decides).
//
// The j - i sign convention is used throughout (the reference forms i - j
// and subtracts); every output is the same quantity.

#include <string.h>

#include <type_traits>

#include "tg_common.cuh"
#include "tg_pn.cuh"
#include "tg_split_ops.cuh"
#include "tg_tma.cuh"

namespace tg {

// Post-Newtonian order and inverse powers of c for the PNAcc sweep.
struct PnParams {
    int order;
    float inv[8];   // inv[k] = 1/c^k, k = 1..7
};

// pnacc_kernel_common.h:8-70 with p2p_pnterms (pn_terms.h:473-567) in FP32:
// the reference's PN polynomials (tg_pn.cuh, instantiated in float) on the
// double-single position difference, softened 1/r from rsqrt.  The result
// is the PN correction alone, as in the reference; i - j as there.
struct PnAccS {
    static constexpr int NF = 3, NO = 3, MAXC = -1;
    static constexpr bool PN = true;
    using P = PosVelRec;
    __device__ static P load(const float4 *r) { return AccJerkS::load(r); }
    __device__ static void pair(const P &i, const P &j, float *o,
                                const PnParams &pn)
    {
        const float im = i.m, jm = j.m;
        const float dx = (i.xh - j.xh) + (i.xl - j.xl);
        const float dy = (i.yh - j.yh) + (i.yl - j.yl);
        const float dz = (i.zh - j.zh) + (i.zl - j.zl);
        const float h2 = i.e2 + j.e2;
        const float ux = i.vx - j.vx, uy = i.vy - j.vy, uz = i.vz - j.vz;
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float v2 = fmaf(uz, uz, fmaf(uy, uy, ux * ux));
        float inv_r = rsqrtf(r2 + h2);
        inv_r = (r2 > 0.f) ? inv_r : 0.f;      // self pairs contribute nothing
        const float inv_r2 = inv_r * inv_r;
        const float inv_r3 = inv_r2 * inv_r;
        const float nx = dx * inv_r, ny = dy * inv_r, nz = dz * inv_r;
        const float iv2 = fmaf(i.vz, i.vz, fmaf(i.vy, i.vy, i.vx * i.vx));
        const float jv2 = fmaf(j.vz, j.vz, fmaf(j.vy, j.vy, j.vx * j.vx));
        PnTerm<float> p2 = {0, 0}, p4 = {0, 0}, p5 = {0, 0}, p6 = {0, 0},
                      p7 = {0, 0};
        const int order = pn.order;
        if (order > 1) {
            const float niv = fmaf(nz, i.vz, fmaf(ny, i.vy, nx * i.vx));
            const float njv = fmaf(nz, j.vz, fmaf(ny, j.vy, nx * j.vx));
            const float njv2 = njv * njv;
            const float ivjv = fmaf(i.vz, j.vz, fmaf(i.vy, j.vy, i.vx * j.vx));
            p2 = pn2<float>(im, jm, inv_r, iv2, jv2, ivjv, niv, njv, njv2,
                            pn.inv[2]);
            if (order > 3) {
                const float im2 = im * im, jm2 = jm * jm, imjm = im * jm;
                const float jv4 = jv2 * jv2;
                const float ivjvivjv = ivjv * ivjv;
                const float nv = fmaf(nz, uz, fmaf(ny, uy, nx * ux));
                const float niv2 = niv * niv;
                const float nivnjv = niv * njv;
                p4 = pn4<float>(im, jm, im2, jm2, imjm, inv_r, inv_r2, iv2,
                                jv2, jv4, ivjv, ivjvivjv, nv, niv, njv, niv2,
                                njv2, nivnjv, pn.inv[4]);
                if (order > 4) {
                    p5 = pn5<float>(im, jm, inv_r, v2, nv, pn.inv[5]);
                    if (order > 5) {
                        const float nvnv = nv * nv;
                        p6 = pn6<float>(im, jm, im2, jm2, imjm, inv_r, inv_r2,
                                        v2, iv2, jv2, jv4, ivjv, ivjvivjv, nv,
                                        nvnv, niv, njv, niv2, njv2, nivnjv,
                                        pn.inv[6]);
                        if (order > 6) {
                            const float iv4 = iv2 * iv2;
                            p7 = pn7<float>(im, jm, im2, jm2, imjm, inv_r,
                                            inv_r2, v2, iv2, jv2, iv4, jv4,
                                            ivjv, nv, nvnv, niv, njv, niv2,
                                            njv2, nivnjv, pn.inv[7]);
                        }
                    }
                }
            }
        }
        const float pa = ((((p7.a + p6.a) + p5.a) + p4.a) + p2.a) * (jm * inv_r3);
        const float pb = ((((p7.b + p6.b) + p5.b) + p4.b) + p2.b) * (jm * inv_r2);
        o[0] = fmaf(pa, dx, fmaf(pb, ux, o[0]));
        o[1] = fmaf(pa, dy, fmaf(pb, uy, o[1]));
        o[2] = fmaf(pa, dz, fmaf(pb, uz, o[2]));
    }
    __device__ static void finish(double *, double) {}
};

// Whether an operator takes the PN parameters instead of eta.
template <class Op, class = void> struct TakesPn : std::false_type {};
template <class Op>
struct TakesPn<Op, std::void_t<decltype(Op::PN)>> : std::true_type {};

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
    const unsigned *n_dev;   // count read on the device (or null)
};

__global__ void pack_records(const PackArgs p, uint64_t n_max, float4 *out)
{
    const uint64_t n = p.n_dev ? (uint64_t)*p.n_dev : n_max;
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

cudaError_t launch_pack_dev(int kernel, uint64_t n, const unsigned *n_dev,
                            const void *const *attrs, float4 *out,
                            cudaStream_t st);

cudaError_t launch_pack(int kernel, uint64_t n, const void *const *attrs,
                        float4 *out, cudaStream_t st)
{
    return launch_pack_dev(kernel, n, nullptr, attrs, out, st);
}

// As launch_pack; with n_dev set, the count is read on the device (n is its
// upper bound and sizes the grid).
cudaError_t launch_pack_dev(int kernel, uint64_t n, const unsigned *n_dev,
                            const void *const *attrs, float4 *out,
                            cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    PackArgs p;
    p.n_dev = n_dev;
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
    uint32_t spin;        // main-loop wait limit (pipe_spin_limit())
    PnParams pn;          // PNAcc only
    const unsigned *ni_dev;   // i count read on the device (ni: its bound)
};

constexpr int SPLIT_TILE = 256;   // j-records per pipeline stage

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
    // the FP32 rounding of each run small next to the particle's |a|
    // (runs of 32 measured max |da|/|a| 1.09e-6 at N = 3000; 16 stay
    // inside 1e-6).
    constexpr int FOLD = (TJ / JS) < 16 ? (TJ / JS) : 16;
    static_assert(TJ % (JS * FOLD) == 0, "fold must divide the tile");
    constexpr int GROUPS = NT / JS;          // i-groups per CTA
    constexpr int IPC = GROUPS * NI;         // i-particles per CTA

    __shared__ __align__(128) float4 ring[2][TJ * NJF];
    __shared__ __align__(8) uint64_t bar[2];

    const int tid = threadIdx.x;
    const int js = tid % JS;
    const int grp = tid / JS;
    const uint64_t ni = L.ni_dev ? (uint64_t)*L.ni_dev : L.ni;
    // CTAs past a device-side count have no i: the whole CTA leaves before
    // any barrier or copy exists
    if ((uint64_t)blockIdx.x * IPC >= ni) return;
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
        if (i >= ni) i = ni - 1;
        ip[k] = Op::load(L.irec + i * NF);
    }

    float sum[NI][NO], corr[NI][NO], part[NI][NO];
#pragma unroll
    for (int k = 0; k < NI; ++k)
#pragma unroll
        for (int c = 0; c < NO; ++c) sum[k][c] = corr[k][c] = part[k][c] = 0.f;
    // packed variants keep the Kahan pairs of an i pair as float2
    float2 sum2[NP][NO], corr2[NP][NO];
#pragma unroll
    for (int q = 0; q < NP; ++q)
#pragma unroll
        for (int c = 0; c < NO; ++c)
            sum2[q][c] = corr2[q][c] = make_float2(0.f, 0.f);

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
    int tfail = 0;
    for (int t = 0; t < ntiles; ++t) {
        bool got = mbar_wait_bounded(&bar[t & 1], (uint32_t)((t >> 1) & 1),
                                     L.err, L.spin);
        if (!__syncthreads_and(got)) { ok = false; tfail = t; break; }
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
            auto run_tile = [&](auto pairfn) {
#pragma unroll 1
                for (int r0 = js; r0 < n; r0 += JS * FOLD) {
                    float2 p2[NP][NO];
#pragma unroll
                    for (int q = 0; q < NP; ++q)
#pragma unroll
                        for (int c = 0; c < NO; ++c)
                            p2[q][c] = make_float2(0.f, 0.f);
                    if (n == TJ) {
#pragma unroll
                        for (int u = 0; u < FOLD; ++u) {
                            const typename Op::P jp =
                                Op::load(tile + (r0 + u * JS) * NF);
#pragma unroll
                            for (int q = 0; q < NP; ++q) pairfn(q, jp, p2[q]);
                        }
                    } else {
#pragma unroll 1
                        for (int u = 0; u < FOLD && r0 + u * JS < n; ++u) {
                            const typename Op::P jp =
                                Op::load(tile + (r0 + u * JS) * NF);
#pragma unroll
                            for (int q = 0; q < NP; ++q) pairfn(q, jp, p2[q]);
                        }
                    }
                    // the run folds into the packed Kahan pairs of both i
#pragma unroll
                    for (int q = 0; q < NP; ++q)
#pragma unroll
                        for (int c = 0; c < NO; ++c) {
                            if (c == MAXC)
                                sum2[q][c] = make_float2(
                                    fmaxf(sum2[q][c].x, p2[q][c].x),
                                    fmaxf(sum2[q][c].y, p2[q][c].y));
                            else
                                kahan_add2(sum2[q][c], corr2[q][c], p2[q][c]);
                        }
                }
            };
            bool uniform = false;
            float e2t = 0.f;
            if constexpr (OpX2::HAS_H2) {
                // One softening for every record of the tile (the common
                // case): h2 = e2_i + e2_tile is formed once per tile.
                e2t = tile[1].w;
                bool same = true;
                for (int r = tid; r < n; r += NT)
                    same = same && (tile[r * NF + 1].w == e2t);
                uniform = __syncthreads_and(same);
            }
            if constexpr (OpX2::HAS_H2) {
                if (uniform) {
                    float2 h2t[NP];
#pragma unroll
                    for (int q = 0; q < NP; ++q)
                        h2t[q] = add2(ip2[q].e2, dup(e2t));
                    run_tile([&](int q, const typename Op::P &jp, float2 *a) {
                        OpX2::pair_h2(ip2[q], jp, a, h2t[q]);
                    });
                }
            }
            if (!uniform)
                run_tile([&](int q, const typename Op::P &jp, float2 *a) {
                    OpX2::pair(ip2[q], jp, a, L.eta);
                });
        } else if (n == TJ) {
#pragma unroll 1
            for (int r0 = 0; r0 < TJ; r0 += JS * FOLD) {
#pragma unroll
                for (int u = 0; u < FOLD; ++u) {
                    const typename Op::P jp =
                        Op::load(tile + (r0 + u * JS + js) * NF);
#pragma unroll
                    for (int k = 0; k < NI; ++k) {
                        if constexpr (TakesPn<Op>::value)
                            Op::pair(ip[k], jp, part[k], L.pn);
                        else
                            Op::pair(ip[k], jp, part[k], L.eta);
                    }
                }
                fold();
            }
        } else {
#pragma unroll 1
            for (int r = js; r < n; r += JS) {
                const typename Op::P jp = Op::load(tile + r * NF);
#pragma unroll
                for (int k = 0; k < NI; ++k) {
                    if constexpr (TakesPn<Op>::value)
                        Op::pair(ip[k], jp, part[k], L.pn);
                    else
                        Op::pair(ip[k], jp, part[k], L.eta);
                }
            }
            fold();
        }
        __syncthreads();
        if (tid == 0 && t + 2 < ntiles) issue(t + 2);
    }
    if (!ok) {
        // A copy did not complete in time.  The copies of tiles tfail and
        // tfail + 1 (where they exist) were issued and not yet consumed:
        // wait for each (full bound, its pending parity) before the shared
        // memory goes away, then leave without writing results (the host
        // reports the error word).
        if (tid == 0)
            for (int u = tfail; u < ntiles && u < tfail + 2; ++u)
                mbar_wait_bounded(&bar[u & 1], (uint32_t)((u >> 1) & 1), L.err);
        return;
    }

    if constexpr (X2) {
#pragma unroll
        for (int q = 0; q < NP; ++q)
#pragma unroll
            for (int c = 0; c < NO; ++c) {
                sum[2 * q][c] = sum2[q][c].x;
                sum[2 * q + 1][c] = sum2[q][c].y;
                corr[2 * q][c] = corr2[q][c].x;
                corr[2 * q + 1][c] = corr2[q][c].y;
            }
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
        if (js == 0 && i < ni) {
            if (gridDim.y == 1) {
                Op::finish(v, L.eta_d);
#pragma unroll
                for (int c = 0; c < NO; ++c) L.out[c][i] = v[c];
            } else {
#pragma unroll
                for (int c = 0; c < NO; ++c)
                    L.partial[((uint64_t)blockIdx.y * NO + c) * ni + i] = v[c];
            }
        }
    }
}

// Reduce grid j-split partials in a fixed order and apply the finish step.
template <class Op>
__global__ void split_finalize(const SplitLaunch L, int gsplit)
{
    constexpr int NO = Op::NO, MAXC = Op::MAXC;
    // a sweep CTA that reported an error left its partials unwritten
    if (*(volatile unsigned *)L.err) return;
    const uint64_t ni = L.ni_dev ? (uint64_t)*L.ni_dev : L.ni;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
         i < ni; i += (uint64_t)gridDim.x * blockDim.x) {
        double v[NO];
#pragma unroll
        for (int c = 0; c < NO; ++c) {
            double a = L.partial[(uint64_t)c * ni + i];
            for (int y = 1; y < gsplit; ++y) {
                double b = L.partial[((uint64_t)y * NO + c) * ni + i];
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
    {2, 1, 256},   // as 5, 1/sqrt without the Newton step
    {4, 1, 256},   // as 7, 1/sqrt without the Newton step
    {2, 1, 256},   // as 0, 1/sqrt without the Newton step
};
constexpr int N_VARIANTS = sizeof(kVariants) / sizeof(kVariants[0]);

int split_variant_count() { return N_VARIANTS; }

void split_variant_info(int v, int *ni_per_thread, int *jsplit, int *threads)
{
    *ni_per_thread = kVariants[v].ni_per_thread;
    *jsplit = kVariants[v].jsplit;
    *threads = kVariants[v].threads;
}

// Variants 9 to 11 take 1/sqrt from the MUFU approximation alone (every
// SPLIT operator has that form).
template <class Op> struct RawOf { using type = Op; };
template <> struct RawOf<PhiS> { using type = PhiSN<false>; };
template <> struct RawOf<AccS> { using type = AccSN<false>; };
template <> struct RawOf<AccJerkS> { using type = AccJerkSN<false>; };
template <> struct RawOf<TstepS> { using type = TstepSN<false>; };
template <> struct RawOf<SnapS> { using type = SnapSN<false>; };

bool split_has_raw(int kernel)
{
    return kernel == K_PHI || kernel == K_ACC || kernel == K_ACC_JERK ||
           kernel == K_TSTEP || kernel == K_SNAP_CRACKLE;
}

// Kernels with a packed-pair (f32x2) operator: variants 5 to 10 use it.
bool split_has_x2(int kernel)
{
    return kernel == K_PHI || kernel == K_ACC || kernel == K_ACC_JERK ||
           kernel == K_TSTEP || kernel == K_SNAP_CRACKLE;
}

bool split_supported(int kernel)
{
    return kernel == K_PHI || kernel == K_ACC || kernel == K_ACC_JERK ||
           kernel == K_TSTEP || kernel == K_SNAP_CRACKLE || kernel == K_PNACC;
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
    case 9:
    case 10:
    case 11: {
        using R = typename RawOf<Op>::type;
        if constexpr (!std::is_void<typename X2Of<R>::type>::value) {
            if (variant == 9) return run_variant<R, 2, 1, 256, 2, true>(L, gsplit, st);
            if (variant == 10) return run_variant<R, 4, 1, 256, 1, true>(L, gsplit, st);
        }
        return run_variant<R, 2, 1, 256, 2>(L, gsplit, st);
    }
    default: return cudaErrorInvalidValue;
    }
}

// irec/jrec: packed records (launch_pack); out: NO double arrays;
// partial: gsplit x NO x ni doubles when gsplit > 1.
cudaError_t launch_split_pn(int kernel, const float4 *irec,
                            const float4 *jrec, uint64_t ni, uint64_t nj,
                            void *const *out, double *partial, int variant,
                            int gsplit, double eta, const double *pn,
                            unsigned *err, cudaStream_t st);

cudaError_t launch_split(int kernel, const float4 *irec, const float4 *jrec,
                         uint64_t ni, uint64_t nj, void *const *out,
                         double *partial, int variant, int gsplit, double eta,
                         unsigned *err, cudaStream_t st)
{
    return launch_split_pn(kernel, irec, jrec, ni, nj, out, partial, variant,
                           gsplit, eta, nullptr, err, st);
}

cudaError_t launch_split_dev(int kernel, const float4 *irec,
                             const float4 *jrec, uint64_t ni,
                             const unsigned *ni_dev, uint64_t nj,
                             void *const *out, double *partial, int variant,
                             int gsplit, double eta, const double *pn,
                             unsigned *err, cudaStream_t st);

// As launch_split; pn: PN order then 1/c .. 1/c^7 (PNAcc; else unused).
cudaError_t launch_split_pn(int kernel, const float4 *irec,
                            const float4 *jrec, uint64_t ni, uint64_t nj,
                            void *const *out, double *partial, int variant,
                            int gsplit, double eta, const double *pn,
                            unsigned *err, cudaStream_t st)
{
    return launch_split_dev(kernel, irec, jrec, ni, nullptr, nj, out, partial,
                            variant, gsplit, eta, pn, err, st);
}

// As launch_split_pn; with ni_dev set, the i count is read on the device
// when the sweep runs (ni is its upper bound and sizes the grid; CTAs past
// the count leave at once).
cudaError_t launch_split_dev(int kernel, const float4 *irec,
                             const float4 *jrec, uint64_t ni,
                             const unsigned *ni_dev, uint64_t nj,
                             void *const *out, double *partial, int variant,
                             int gsplit, double eta, const double *pn,
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
    L.spin = pipe_spin_limit();
    L.ni_dev = ni_dev;
    memset(&L.pn, 0, sizeof(L.pn));
    if (pn) {
        L.pn.order = (int)pn[0];
        for (int q = 1; q < 8; ++q) L.pn.inv[q] = (float)pn[q];
    }
    switch (kernel) {
    case K_PHI: return run_op<PhiS>(L, variant, gsplit, st);
    case K_ACC: return run_op<AccS>(L, variant, gsplit, st);
    case K_ACC_JERK: return run_op<AccJerkS>(L, variant, gsplit, st);
    case K_TSTEP: return run_op<TstepS>(L, variant, gsplit, st);
    case K_SNAP_CRACKLE: return run_op<SnapS>(L, variant, gsplit, st);
    case K_PNACC: return run_op<PnAccS>(L, variant, gsplit, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tg
