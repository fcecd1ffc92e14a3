// Ensemble driver: many independent N-body systems of mixed size advanced
// together on one GPU, each with its own shared adaptive Hermite-4 step
// (tupan's "ahermite4": hermite.py:390-410 with the quantisation of
// integrator/__init__.py:59-78), each system's step held in device memory.
//
// Every force evaluation of the whole ensemble is ONE launch of a
// persistent batched SPLIT sweep (k_e_sweep) whose CTAs take (system,
// i-block) work items of the unfinished systems from an atomic queue,
// largest systems first.  The CTA that computed an i-block's forces runs
// the step's next per-particle stage on that block (state copy, predictor,
// corrector) and packs the FP32 records the next sweep reads; only the
// step size, a minimum over the whole system, waits for the system's last
// item.  A step is a fixed sequence of five launches and `batch` steps are
// captured in a CUDA graph and replayed.  Systems with hard binaries take
// tens of thousands of small shared steps, so several hundred systems stay
// active through most of a run: the sweep's throughput with a few hundred
// mid-size systems (small CTAs, few barriers per item) sets the run time,
// and the step latency once only a few systems remain sets its tail.
// A persistent mode (k_e_run) instead gives each CTA a whole system for
// many steps per launch.
// Energies are fp64: an in-order fp64 Phi per system (same arithmetic and j
// order as phi_kernel.c) and fp64 sums in fixed order.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <type_traits>
#include <numeric>
#include <vector>

#include "tg_common.cuh"
#include "tg_split_ops.cuh"
#include "tg_tma.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))


using namespace tg;

namespace {

struct SysCtl {
    double t, tau;
    unsigned long long min_bits;
    long long nsteps;
};

struct EArrays {
    double *m, *e2, *r[3], *v[3], *r0[3], *v0[3], *f0[6], *f1[6], *dt[2];
    double *phi;
    unsigned *sys;          // system of each particle
};

__device__ __forceinline__ double e_base_tstep(double t, double t_end,
                                               double eta)
{
    double dt = fmin(fabs(t_end) - fabs(t), fabs(eta));
    dt = fmax(dt, fabs(t_end) * (2.0 * 2.220446049250313e-16));
    return copysign(dt, eta);
}

__device__ __forceinline__ double e_block_tstep(double min_ts, double t,
                                                double tau)
{
    long long power = quantised_power(min_ts);
    double min_bts = ldexp(1.0, (int)power);
    double t_next = t + min_bts;
    for (int k = 0; k < 2100 && fmod(t_next, min_bts) != 0.0; ++k)
        min_bts /= 2.0;
    min_bts = copysign(min_bts, tau);
    if (fabs(min_bts) > fabs(tau)) min_bts = tau;
    return min_bts;
}

// The systems still short of t_end, in processing order (largest first),
// and the batched sweep's work items in the same order: each active system
// split into i-blocks, (system, ib | ie << 16) per item, so a large system
// is spread over several CTAs.  The block is the shape's full i-block while
// the active systems outnumber the sweep's CTAs (fewer items, less
// reloading of j-records), and shrinks to a half and a quarter of it (not
// below 32 i) as systems finish, so the last few systems still use many
// SMs.  One CTA: the per-system step start (activity, base step; t_end is
// read from device memory, so a captured graph replays with the value of
// the current evolve call), then a stable compaction.
constexpr int COMPACT_NT = 1024;

__device__ unsigned block_exclusive_scan(unsigned v, unsigned *wsum,
                                         unsigned *total)
{
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    unsigned before = 0, all = 0;
    for (int q = 0; q < COMPACT_NT / 32; ++q) {
        before += q < w ? wsum[q] : 0;
        all += wsum[q];
    }
    __syncthreads();
    *total = all;
    return before + x - v;
}

__global__ void __launch_bounds__(COMPACT_NT)
k_e_begin(SysCtl *c, int *active, const unsigned *order, const uint64_t *off,
          unsigned ns, const double *t_end_p, double eta, unsigned ctas,
          unsigned ib_full, unsigned *alist, unsigned *acount, uint2 *items, unsigned *icount,
          unsigned *sys_items, unsigned *queues)
{
    // the work counters of the step's four sweeps (a kernel write instead
    // of memset nodes in the step graph)
    if (threadIdx.x < 4) queues[threadIdx.x] = 0;
    __shared__ unsigned wsum[COMPACT_NT / 32];
    __shared__ unsigned n_active;
    const int t = threadIdx.x;
    const double t_end = *t_end_p;
    if (t == 0) n_active = 0;
    __syncthreads();
    unsigned mine = 0;
    for (unsigned s = t; s < ns; s += COMPACT_NT) {
        const bool on = fabs(c[s].t) < t_end;
        active[s] = on ? 1 : 0;
        c[s].tau = on ? e_base_tstep(c[s].t, t_end, eta) : 0.0;
        mine += on ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((t & 31) == 0) atomicAdd(&n_active, mine);
    __syncthreads();
    const unsigned na = n_active;
    unsigned IB = na >= ctas ? ib_full : (na >= ctas / 4 ? ib_full / 2
                                                         : ib_full / 4);
    IB = IB < 32u ? 32u : IB;
    unsigned sbase = 0, ibase = 0;
    for (unsigned c0 = 0; c0 < ns; c0 += COMPACT_NT) {
        const unsigned k = c0 + t;
        const unsigned s = k < ns ? order[k] : 0;
        const bool on = k < ns && active[s];
        const unsigned n = on ? (unsigned)(off[s + 1] - off[s]) : 0;
        const unsigned nb = on ? (n + IB - 1) / IB : 0;
        unsigned stot, itot;
        const unsigned spos = block_exclusive_scan(on ? 1u : 0u, wsum, &stot);
        const unsigned ipos = block_exclusive_scan(nb, wsum, &itot);
        if (on) {
            alist[sbase + spos] = s;
            sys_items[s] = nb;
            for (unsigned q = 0; q < nb; ++q) {
                const unsigned ib = q * IB, ie = ib + IB < n ? ib + IB : n;
                items[ibase + ipos + q] = make_uint2(s, ib | (ie << 16));
            }
        }
        sbase += stot;
        ibase += itot;
    }
    if (t == 0) {
        *acount = sbase;
        *icount = ibase;
    }
}

// Packed record of particle i (the layout of split.cu's pack_records for 3
// float4: {xh yh zh m} {xl yl zl e2} {vx vy vz 0}), from the current state.
__device__ __forceinline__ void e_pack_rec(const EArrays &A, float4 *r,
                                           uint64_t i)
{
    float xh, xl, yh, yl, zh, zl;
    split2(A.r[0][i], xh, xl);
    split2(A.r[1][i], yh, yl);
    split2(A.r[2][i], zh, zl);
    r[0] = make_float4(xh, yh, zh, (float)A.m[i]);
    r[1] = make_float4(xl, yl, zl, (float)A.e2[i]);
    r[2] = make_float4((float)A.v[0][i], (float)A.v[1][i], (float)A.v[2][i],
                       0.f);
}

__device__ __forceinline__ void e_pack_one(const EArrays &A, float4 *out,
                                           uint64_t i)
{
    e_pack_rec(A, out + i * 3, i);
}

// Records of every particle (before the first step of an evolve call).
__global__ void k_e_pack_all(EArrays A, uint64_t n, float4 *out)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        e_pack_one(A, out, i);
}

// ---------------------------------------------------------------------------
// Per-system epilogues, run by the CTA that completes a system's last work
// item of a sweep (the other items' outputs are read through L2).
// ---------------------------------------------------------------------------
enum Epilogue { EPI_NONE = 0, EPI_STEP_SIZE, EPI_PREDICT, EPI_CORRECT,
                EPI_CORRECT_END };

// The step's per-particle stages on one i-block [b, e) of a system, run by
// the CTA that computed the block's forces right after it (a particle's
// update needs only its own forces).  Records go to a buffer the running
// sweep does not read, so items of the same system still loading theirs
// see the old state.

// the copy of the state at the start of the step
__device__ void epi_copy(const EArrays &A, uint64_t b, uint64_t e)
{
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x)
        for (int d = 0; d < 3; ++d) {
            A.r0[d][i] = A.r[d][i];
            A.v0[d][i] = A.v[d][i];
        }
}

// min |dt_a| over the whole system -> power-of-two step (integrator/
// __init__.py:59-78): run by the CTA that completes the system's last item
// (the other items' outputs are read through L2).
__device__ void epi_step_size(const EArrays &A, SysCtl *c, uint64_t s,
                              uint64_t b, uint64_t e)
{
    __shared__ double red[32];
    const int t = threadIdx.x;
    double m = INFINITY;
    for (uint64_t i = b + t; i < e; i += blockDim.x)
        m = fmin(m, fabs(__ldcg(&A.dt[0][i])));
    for (int o = 16; o > 0; o >>= 1)
        m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((t & 31) == 0) red[t >> 5] = m;
    __syncthreads();
    if (t == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) m = fmin(m, red[q]);
        c[s].tau = e_block_tstep(m, c[s].t, c[s].tau);
    }
    __syncthreads();
}

// H4.epredict (hermite.py:83-88) of particle i.
__device__ __forceinline__ void predict_one(const EArrays &A, double tau,
                                            uint64_t i)
{
    for (int d = 0; d < 3; ++d) {
        const double a = A.f0[d][i], j = A.f0[3 + d][i], v = A.v[d][i];
        A.r[d][i] = A.r[d][i] + ((j * tau / 3 + a) * tau / 2 + v) * tau;
        A.v[d][i] = v + (j * tau / 2 + a) * tau;
    }
}

// H4.ecorrect (hermite.py:96-119) of particle i.
__device__ __forceinline__ void correct_one(const EArrays &A, double tau,
                                            uint64_t i)
{
    for (int d = 0; d < 3; ++d) {
        const double a0 = A.f0[d][i], a1 = A.f1[d][i];
        const double j0 = A.f0[3 + d][i], j1 = A.f1[3 + d][i];
        const double v0 = A.v0[d][i], r0 = A.r0[d][i];
        const double v1 = (((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + v0);
        A.v[d][i] = v1;
        A.r[d][i] = (((a0 - a1) * tau / 6 + (v0 + v1)) * tau / 2 + r0);
    }
}

// ---------------------------------------------------------------------------
// Batched SPLIT sweep over the (system, i-block) work items of the active
// systems, one persistent launch per force evaluation.  CTAs take items
// from an atomic queue (largest systems first), stage the system's packed
// records in shared memory with one bulk copy, and give each i (or packed i
// pair) `lanes` threads that split the j loop and combine through shuffles.
// The CTA that completes the last item of a system runs the step's next
// per-system stage (the epilogue), so a Hermite step is five launches.
// ---------------------------------------------------------------------------
// AccJerk and Tstep with 1/sqrt from rsqrtf alone (the split sweeps'
// default forms)
using AccJerkFast = AccJerkSN<false>;
using TstepFast = TstepSN<false>;

constexpr int RUN_NT = 256;               // persistent mode: threads per CTA
constexpr int BATCH_MAXN = 512;           // largest system held in smem

// Launch shape of the batched sweep: threads per CTA (128 with four CTAs per
// SM, or 256 with two), the i-block of a work item while the active systems
// fill the grid (halved and quartered, not below 32, as they finish), and
// whether a CTA copies its next item's records while it computes the
// current one (two record buffers, 48 KiB of shared memory per CTA).  The
// default is the fastest of the twelve shapes on 4096 systems of 3-512
// (t_end = 1/64 after 1/512 of warm-up, GB300): 128 threads, i-block 128,
// no prefetch, 0.621 s; with prefetch 0.644 s; 256 threads 0.70-0.98 s.
// The copy of a system's records is short next to its item's sweep, so
// hiding it does not pay for the second buffer's occupancy.
struct EShape {
    int nt = 128;
    int ib = 128;
    int prefetch = 0;
};
EShape g_ens_default;                     // shape of new ensembles

inline int shape_minb(const EShape &s) { return s.nt == 256 ? 2 : 4; }
inline bool shape_valid(int nt, int ib, int prefetch)
{
    return (nt == 128 || nt == 256) &&
           (ib == 32 || ib == 64 || ib == 128 || ib == 256 || ib == 512) &&
           (prefetch == 0 || prefetch == 1);
}

struct BatchLaunch {
    const float4 *rec;        // packed records of all systems
    const uint64_t *off;      // n_sys + 1 offsets
    const uint2 *items;       // (system, ib | ie << 16) per item
    const unsigned *n_items;  // item count (device)
    unsigned *queue;          // work counter (zeroed before the launch)
    unsigned *sys_done;       // items finished per system (self-resetting)
    const unsigned *sys_items;// items per system this step
    double *out[MAX_OUT];
    float eta;
    double eta_d;
    unsigned *err;
    uint32_t spin;            // main-loop wait limit (pipe_spin_limit())
    int epi;
    EArrays A;
    SysCtl *ctl;
    float4 *rec_out;          // records written by the epilogues
};

// One system's i-range [ib, ib + ni) against all of its j (records in
// shared memory); outputs to out[c][b + i].
template <class Op, bool X2, int NT>
__device__ __forceinline__ void batched_block(double *const *out, float eta,
                                              double eta_d, const float4 *rec,
                                              uint64_t b, int n, int ib, int ni)
{
    constexpr int NF = Op::NF, NO = Op::NO, MAXC = Op::MAXC;
    constexpr int NI = X2 ? 2 : 1;               // i per thread
    const int tid = threadIdx.x;
    const int units = (ni + NI - 1) / NI;        // i (pairs) of the block
    int lanes = 1;
    while (lanes < 32 && lanes * 2 * units <= NT) lanes *= 2;
    const int groups = NT / lanes;
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
                if (j0 + 15 * lanes < n) {
                    // a whole run: unrolled, so independent pairs interleave
#pragma unroll
                    for (int u = 0; u < 16; ++u)
                        OpX2::pair(ip2, Op::load(rec + (j0 + u * lanes) * NF),
                                   p2, eta);
                } else {
                    for (int j = j0; j < n; j += lanes)
                        OpX2::pair(ip2, Op::load(rec + j * NF), p2, eta);
                }
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
                if (j0 + 15 * lanes < n) {
#pragma unroll
                    for (int u = 0; u < 16; ++u)
                        Op::pair(ip, Op::load(rec + (j0 + u * lanes) * NF),
                                 part[0], eta);
                } else {
                    for (int j = j0; j < n; j += lanes)
                        Op::pair(ip, Op::load(rec + j * NF), part[0], eta);
                }
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
                Op::finish(v, eta_d);
#pragma unroll
                for (int c = 0; c < NO; ++c) out[c][b + iv[k]] = v[c];
            }
        }
    }
}

// Validates work item w and, when it is one, starts the bulk copy of its
// system's records into dst (thread 0 only).  An invalid item is left for
// the loop, which reports it.
template <int NF>
__device__ __forceinline__ bool e_issue(const BatchLaunch &L, unsigned w,
                                        unsigned n_items, float4 *dst,
                                        uint64_t *bar)
{
    if (w >= n_items) return false;
    const unsigned sys = L.items[w].x;
    const uint64_t b = L.off[sys];
    const int n = (int)(L.off[sys + 1] - b);
    const int ib = (int)(L.items[w].y & 0xffffu);
    const int ie = (int)(L.items[w].y >> 16);
    if (n > BATCH_MAXN || ie > n || ib >= ie) return false;
    const uint32_t bytes = (uint32_t)(n * NF * sizeof(float4));
    mbar_arrive_expect_tx(bar, bytes);
    bulk_g2s(dst, L.rec + b * NF, bytes, bar);
    return true;
}

template <class Op, int NT, int MINB, bool PREFETCH>
__global__ void __launch_bounds__(NT, MINB)
k_e_sweep(const BatchLaunch L)
{
    constexpr int NF = Op::NF;
    constexpr bool X2 = !std::is_void<typename X2Of<Op>::type>::value;
    constexpr int NBUF = PREFETCH ? 2 : 1;
    constexpr int BUF = BATCH_MAXN * NF;          // float4 per record buffer
    extern __shared__ __align__(128) float4 e_rec[];
    __shared__ __align__(8) uint64_t bar[NBUF];
    __shared__ unsigned item[NBUF];
    __shared__ int last;
    const int tid = threadIdx.x;
    const unsigned n_items = *L.n_items;
    // thread 0: buffers with a copy in flight; bit q of phase: the parity
    // of buffer q's next completion
    unsigned pending = 0, phase = 0;
    if (tid == 0) {
        for (int q = 0; q < NBUF; ++q) mbar_init(&bar[q], 1);
        mbar_init_fence();
        item[0] = atomicAdd(L.queue, 1u);
        if (PREFETCH && e_issue<NF>(L, item[0], n_items, e_rec, &bar[0]))
            pending = 1u;
    }
    __syncthreads();
    for (int cur = 0;; cur = PREFETCH ? cur ^ 1 : 0) {
        const unsigned w = item[cur];
        if (w >= n_items) break;
        const unsigned sys = L.items[w].x;
        const uint64_t b = L.off[sys];
        const int n = (int)(L.off[sys + 1] - b);
        const int ib = (int)(L.items[w].y & 0xffffu);
        const int ie = (int)(L.items[w].y >> 16);
        if (n > BATCH_MAXN || ie > n || ib >= ie) {
            // no copy was started for it; a prefetch is started only after
            // this check, so none is in flight either
            if (tid == 0) atomicOr(L.err, (unsigned)DERR_BAD_LAUNCH);
            break;
        }
        float4 *rec = e_rec + cur * BUF;
        if (tid == 0) {
            if (PREFETCH) {
                // the next item's copy runs while this one computes; its
                // buffer was last read before the previous item's closing
                // barrier
                const unsigned nx = atomicAdd(L.queue, 1u);
                item[cur ^ 1] = nx;
                if (e_issue<NF>(L, nx, n_items, e_rec + (cur ^ 1) * BUF,
                                &bar[cur ^ 1]))
                    pending |= 1u << (cur ^ 1);
            } else if (e_issue<NF>(L, w, n_items, rec, &bar[0])) {
                pending |= 1u;
            }
        }
        const bool got = mbar_wait_bounded(&bar[cur], (phase >> cur) & 1u,
                                           L.err, L.spin);
        if (!__syncthreads_and(got)) {
            // a copy did not complete in time: wait (bounded) once more for
            // every copy in flight before the shared memory goes away
            if (tid == 0)
                for (int q = 0; q < NBUF; ++q)
                    if (pending & (1u << q))
                        mbar_wait_bounded(&bar[q], (phase >> q) & 1u, L.err);
            break;
        }
        phase ^= 1u << cur;
        pending &= ~(1u << cur);
        const uint64_t bi = b + ib, ei = b + ie;
        // Tstep sweeps (the one operator with a max output) end in the
        // step size; AccJerk sweeps in the predictor or corrector
        constexpr bool TSTEP_SWEEP = Op::MAXC >= 0;
        batched_block<Op, X2, NT>(L.out, L.eta, L.eta_d, rec, b, n, ib,
                                  ie - ib);
        // this block's outputs are written (CTA scope), for a stage here
        if (TSTEP_SWEEP || L.epi != EPI_NONE) __syncthreads();
        if constexpr (TSTEP_SWEEP) {
            if (L.epi == EPI_STEP_SIZE) {
                epi_copy(L.A, bi, ei);
                // publish this item's Tstep outputs, then count it; the
                // CTA that completes the system takes the system's minimum
                __threadfence();
                __syncthreads();
                if (tid == 0)
                    last = atomicAdd(&L.sys_done[sys], 1u) + 1u ==
                           L.sys_items[sys];
                __syncthreads();
                if (last) {
                    __threadfence();
                    epi_step_size(L.A, L.ctl, sys, b, b + n);
                    if (tid == 0) L.sys_done[sys] = 0;
                }
            }
        } else {
            // the block's predictor or corrector, spread over the CTA;
            // records go to the buffer the next sweep reads
            const double tau = L.ctl[sys].tau;
            if (L.epi == EPI_PREDICT) {
                for (uint64_t i = bi + tid; i < ei; i += NT) {
                    predict_one(L.A, tau, i);
                    e_pack_one(L.A, L.rec_out, i);
                }
            } else if (L.epi == EPI_CORRECT || L.epi == EPI_CORRECT_END) {
                for (uint64_t i = bi + tid; i < ei; i += NT) {
                    correct_one(L.A, tau, i);
                    e_pack_one(L.A, L.rec_out, i);
                }
                // the system's time moves once, by its first item
                if (L.epi == EPI_CORRECT_END && ib == 0 && tid == 0) {
                    L.ctl[sys].t += tau;
                    L.ctl[sys].nsteps += 1;
                }
            }
        }
        // every thread read this item before the copy barrier above; the
        // closing barrier ends this item's reads of its record buffer
        // before a copy into it starts
        if (!PREFETCH && tid == 0) item[0] = atomicAdd(L.queue, 1u);
        __syncthreads();
    }
}

template <class Op, int NT, int MINB, bool PREFETCH>
size_t e_sweep_smem()
{
    return (size_t)(PREFETCH ? 2 : 1) * BATCH_MAXN * Op::NF * sizeof(float4);
}

// Shared-memory limits of every instantiation (above the 48 KiB default for
// the double-buffered ones); once per process.
cudaError_t e_sweep_attributes()
{
    static std::atomic<int> done{0};
    if (done.load()) return cudaSuccess;
    cudaError_t e = cudaSuccess;
#define TG_E_ATTR(OP, NT, MINB, PF)                                           \
    if (e == cudaSuccess)                                                     \
        e = cudaFuncSetAttribute(k_e_sweep<OP, NT, MINB, PF>,                 \
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 (int)e_sweep_smem<OP, NT, MINB, PF>());
    TG_E_ATTR(TstepFast, 128, 4, false)
    TG_E_ATTR(TstepFast, 128, 4, true)
    TG_E_ATTR(TstepFast, 256, 2, false)
    TG_E_ATTR(TstepFast, 256, 2, true)
    TG_E_ATTR(AccJerkFast, 128, 4, false)
    TG_E_ATTR(AccJerkFast, 128, 4, true)
    TG_E_ATTR(AccJerkFast, 256, 2, false)
    TG_E_ATTR(AccJerkFast, 256, 2, true)
#undef TG_E_ATTR
    if (e == cudaSuccess) done.store(1);
    return e;
}

template <class Op>
void e_launch(const EShape &sh, unsigned grid, cudaStream_t st,
              const BatchLaunch &L)
{
    if (sh.nt == 256) {
        if (sh.prefetch)
            k_e_sweep<Op, 256, 2, true><<<grid, 256,
                e_sweep_smem<Op, 256, 2, true>(), st>>>(L);
        else
            k_e_sweep<Op, 256, 2, false><<<grid, 256,
                e_sweep_smem<Op, 256, 2, false>(), st>>>(L);
    } else {
        if (sh.prefetch)
            k_e_sweep<Op, 128, 4, true><<<grid, 128,
                e_sweep_smem<Op, 128, 4, true>(), st>>>(L);
        else
            k_e_sweep<Op, 128, 4, false><<<grid, 128,
                e_sweep_smem<Op, 128, 4, false>(), st>>>(L);
    }
}

// The per-particle stage of an AccJerk sweep as a launch of its own over
// the same work items (the sweep then runs without it): kind EPI_PREDICT,
// EPI_CORRECT or EPI_CORRECT_END.  The sweep's warps keep to FP32 work and
// one barrier less per item; the stage's fp64 loads and stores run
// coalesced over all SMs (an option: slower overall, see
// tupan_gb300_ensemble_set_stage).
__global__ void __launch_bounds__(128)
k_e_stage(const EArrays A, SysCtl *ctl, const uint64_t *off,
          const uint2 *items, const unsigned *n_items, float4 *rec_out,
          int kind)
{
    const unsigned n_it = *n_items;
    for (unsigned w = blockIdx.x; w < n_it; w += gridDim.x) {
        const unsigned sys = items[w].x;
        const uint64_t b = off[sys];
        const int n = (int)(off[sys + 1] - b);
        const int ib = (int)(items[w].y & 0xffffu);
        const int ie = (int)(items[w].y >> 16);
        if (ie > n || ib >= ie) continue;    // the sweep reports it
        const double tau = ctl[sys].tau;
        for (int q = ib + (int)threadIdx.x; q < ie; q += (int)blockDim.x) {
            const uint64_t i = b + (uint64_t)q;
            if (kind == EPI_PREDICT) predict_one(A, tau, i);
            else correct_one(A, tau, i);
            e_pack_one(A, rec_out, i);
        }
        // the system's time moves once, by its first item
        if (kind == EPI_CORRECT_END && ib == 0 && threadIdx.x == 0) {
            ctl[sys].t += tau;
            ctl[sys].nsteps += 1;
        }
    }
}

// ---------------------------------------------------------------------------
// Persistent mode: each CTA takes a whole system from a queue (largest
// first) and steps it on its own, with the system's packed records resident
// in shared memory and __syncthreads between the stages, for up to
// `max_steps` steps or until t_end; then it takes the next system.  No CTA
// waits on another.  The stages and their arithmetic are those of the
// batched mode (Tstep -> step size, AccJerk -> predict, AccJerk -> correct,
// AccJerk -> correct); only the order of the j sums differs.
// ---------------------------------------------------------------------------
struct RunLaunch {
    EArrays A;
    SysCtl *ctl;
    const uint64_t *off;
    const unsigned *order;
    unsigned ns;
    unsigned *queue;
    const double *t_end_p;
    double eta;
    int max_steps;
    unsigned *err;
};

__global__ void __launch_bounds__(RUN_NT, 2)
k_e_run(const RunLaunch R)
{
    __shared__ __align__(16) float4 rec[BATCH_MAXN * 3];
    __shared__ double red[RUN_NT / 32];
    __shared__ unsigned item;
    const int tid = threadIdx.x;
    const double t_end = *R.t_end_p;
    const EArrays &A = R.A;
    for (;;) {
        if (tid == 0) item = atomicAdd(R.queue, 1u);
        __syncthreads();
        const unsigned w = item;
        __syncthreads();               // `item` is rewritten next round
        if (w >= R.ns) break;
        const unsigned s = R.order[w];
        const uint64_t b = R.off[s];
        const int n = (int)(R.off[s + 1] - b);
        if (n > BATCH_MAXN) {
            if (tid == 0) atomicOr(R.err, (unsigned)DERR_BAD_LAUNCH);
            continue;
        }
        double t = R.ctl[s].t;
        long long steps = R.ctl[s].nsteps;
        if (n < 1 || !(fabs(t) < t_end)) continue;
        for (int i = tid; i < n; i += RUN_NT) e_pack_rec(A, rec + 3 * i, b + i);
        __syncthreads();
        for (int k = 0; k < R.max_steps && fabs(t) < t_end; ++k) {
            // step size: Tstep sweep, min |dt_a| over the system, quantised
            const double tau0 = e_base_tstep(t, t_end, R.eta);
            batched_block<TstepFast, true, RUN_NT>(A.dt, (float)R.eta, R.eta, rec, b, n,
                                        0, n);
            __syncthreads();
            double m = INFINITY;
            for (int i = tid; i < n; i += RUN_NT)
                m = fmin(m, fabs(A.dt[0][b + i]));
            for (int o = 16; o > 0; o >>= 1)
                m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((tid & 31) == 0) red[tid >> 5] = m;
            __syncthreads();
            if (tid == 0) {
                for (int q = 1; q < RUN_NT / 32; ++q) m = fmin(m, red[q]);
                red[0] = e_block_tstep(m, t, tau0);
            }
            __syncthreads();
            const double tau = red[0];
            for (int i = tid; i < n; i += RUN_NT)
                for (int d = 0; d < 3; ++d) {
                    A.r0[d][b + i] = A.r[d][b + i];
                    A.v0[d][b + i] = A.v[d][b + i];
                }
            // P(EC)^2: forces at the start, predict, two corrections
            batched_block<AccJerkFast, true, RUN_NT>(A.f0, 0.f, 0.0, rec, b, n, 0, n);
            __syncthreads();
            for (int i = tid; i < n; i += RUN_NT) {
                predict_one(A, tau, b + i);
                e_pack_rec(A, rec + 3 * i, b + i);
            }
            __syncthreads();
            for (int pass = 0; pass < 2; ++pass) {
                batched_block<AccJerkFast, true, RUN_NT>(A.f1, 0.f, 0.0, rec, b, n, 0, n);
                __syncthreads();
                for (int i = tid; i < n; i += RUN_NT) {
                    correct_one(A, tau, b + i);
                    e_pack_rec(A, rec + 3 * i, b + i);
                }
                __syncthreads();
            }
            t += tau;
            steps += 1;
        }
        if (tid == 0) {
            R.ctl[s].t = t;
            R.ctl[s].nsteps = steps;
        }
        __syncthreads();
    }
}

// fp64 potential of each system in j order (phi_kernel.c:20-33 arithmetic)
// and the system's kinetic and potential energy in a fixed reduction order.
__global__ void k_e_energy(EArrays A, const uint64_t *off, double *ke,
                           double *pe)
{
    const unsigned s = blockIdx.x;
    const uint64_t b = off[s], e = off[s + 1];
    __shared__ double sk[256], sp[256];
    double kk = 0.0, pp = 0.0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        double phi = 0.0;
        for (uint64_t j = b; j < e; ++j) {
            const double dx = A.r[0][i] - A.r[0][j];
            const double dy = A.r[1][i] - A.r[1][j];
            const double dz = A.r[2][i] - A.r[2][j];
            const double h2 = A.e2[i] + A.e2[j];
            const double r2 = dx * dx + dy * dy + dz * dz;
            double q = 1.0 / (r2 + h2);
            q = (r2 > 0.0) ? q : 0.0;
            phi -= A.m[j] * sqrt(q);
        }
        const double vx = A.v[0][i], vy = A.v[1][i], vz = A.v[2][i];
        kk += 0.5 * A.m[i] * (vx * vx + vy * vy + vz * vz);
        pp += A.m[i] * phi;
    }
    sk[threadIdx.x] = kk;
    sp[threadIdx.x] = pp;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sk[threadIdx.x] += sk[threadIdx.x + w];
            sp[threadIdx.x] += sp[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ke[s] = sk[0];
        pe[s] = 0.5 * sp[0];
    }
}

struct Ensemble {
    uint64_t n = 0;
    unsigned ns = 0;
    double eta = 0.0;
    int sms = 152;
    cudaStream_t stream = nullptr;
    double *pool = nullptr;
    EArrays A;
    uint64_t *off = nullptr;
    unsigned *order = nullptr;
    int *active = nullptr;
    unsigned *alist = nullptr;      // active systems, largest first
    unsigned *acount = nullptr;
    uint2 *items = nullptr;         // their i-blocks, same order
    unsigned *icount = nullptr;
    unsigned *sys_items = nullptr;  // items per system this step
    unsigned *sys_done = nullptr;   // items finished per system
    SysCtl *ctl = nullptr;
    unsigned *queue = nullptr;      // work counters of the four sweeps
    unsigned *err = nullptr;
    float4 *pack = nullptr;         // three record buffers of n x 3 float4
    double *ke = nullptr, *pe = nullptr;
    double t_end = 0.0;
    double *d_tend = nullptr;       // t_end of the current evolve call
    cudaGraphExec_t graph = nullptr;
    int graph_batch = -1;
    unsigned long long launches_per_batch = 0;
    int mode = 0;                   // 0 batched steps, 1 persistent systems
    int steps_per_launch = 1024;    // persistent: cap per system and launch
    unsigned switch_below = 0;      // persistent -> batched below this many
    EShape shape;                   // batched sweep launch shape
    int split_stage = 0;            // AccJerk stages as launches of their own
};

// One force evaluation of every active system from the current records,
// followed per system by the epilogue `epi`.
cudaError_t e_sweep(Ensemble *E, int kernel, double *const *out, double eta,
                    int epi, int read_buf, int write_buf, int queue)
{
    BatchLaunch L;
    memset(&L, 0, sizeof(L));
    L.rec = E->pack + (size_t)read_buf * E->n * 3;
    L.off = E->off;
    L.items = E->items;
    L.n_items = E->icount;
    L.queue = E->queue + queue;
    L.sys_done = E->sys_done;
    L.sys_items = E->sys_items;
    for (int c = 0; c < n_out(kernel); ++c) L.out[c] = out[c];
    L.eta = (float)eta;
    L.eta_d = eta;
    L.err = E->err;
    L.spin = pipe_spin_limit();   // read when a step is launched or captured
    L.epi = epi;
    L.A = E->A;
    L.ctl = E->ctl;
    L.rec_out = E->pack + (size_t)write_buf * E->n * 3;
    // persistent CTAs; a system of up to 512 particles is at most 16 items
    const uint64_t max_items = (uint64_t)E->ns * 16;
    const uint64_t ctas = (uint64_t)E->sms * shape_minb(E->shape);
    const unsigned grid = (unsigned)(ctas < max_items ? ctas : max_items);
    if (kernel == K_TSTEP)
        e_launch<TstepFast>(E->shape, grid, E->stream, L);
    else
        e_launch<AccJerkFast>(E->shape, grid, E->stream, L);
    g_launch_count += 1;
    return cudaGetLastError();
}

// The per-particle stage `kind` of the current work items, records to
// buffer write_buf.
cudaError_t e_stage(Ensemble *E, int kind, int write_buf)
{
    const uint64_t max_items = (uint64_t)E->ns * 16;
    const uint64_t cap = (uint64_t)E->sms * 8;
    const unsigned grid = (unsigned)(max_items < cap ? max_items : cap);
    k_e_stage<<<grid, 128, 0, E->stream>>>(E->A, E->ctl, E->off, E->items,
                                           E->icount,
                                           E->pack + (size_t)write_buf * E->n * 3,
                                           kind);
    g_launch_count += 1;
    return cudaGetLastError();
}

// One Hermite-4 step of every unfinished system (hermite.py:390-410 with
// epec(2)): the step start and compaction, then four sweeps whose
// epilogues set the step size, predict, and correct twice.  Records rotate
// through three buffers (state A -> predicted B -> corrected C -> final A)
// so that no sweep writes the buffer it reads, and every step starts from
// buffer 0.
cudaError_t e_step(Ensemble *E)
{
    cudaStream_t st = E->stream;
    k_e_begin<<<1, COMPACT_NT, 0, st>>>(E->ctl, E->active, E->order, E->off,
                                        E->ns, E->d_tend, E->eta,
                                        (unsigned)(E->sms * shape_minb(E->shape)),
                                        (unsigned)E->shape.ib, E->alist,
                                        E->acount, E->items, E->icount,
                                        E->sys_items, E->queue);
    g_launch_count += 1;
    cudaError_t e = e_sweep(E, K_TSTEP, E->A.dt, E->eta, EPI_STEP_SIZE, 0, 0, 0);
    const int epis[3] = {EPI_PREDICT, EPI_CORRECT, EPI_CORRECT_END};
    double *const *outs[3] = {E->A.f0, E->A.f1, E->A.f1};
    for (int q = 0; q < 3 && e == cudaSuccess; ++q) {
        const int rb = q, wb = (q + 1) % 3;
        e = e_sweep(E, K_ACC_JERK, outs[q], 0.0,
                    E->split_stage ? EPI_NONE : epis[q], rb, wb, q + 1);
        if (e == cudaSuccess && E->split_stage) e = e_stage(E, epis[q], wb);
    }
    return e;
}

}  // namespace

// ===========================================================================
// C-ABI (no counterpart in the reference, which integrates one system).
// ===========================================================================

// n_sys systems; sys_off[n_sys + 1] host offsets into the concatenated HOST
// arrays m, e2, r, v (sizes 1 .. 512 each).  Forces are SPLIT-mode.
TG_EXPORT int tupan_gb300_ensemble_destroy(void *handle);

TG_EXPORT int tupan_gb300_ensemble_create(unsigned n_sys,
                                          const uint64_t *sys_off, double eta,
                                          const double *m, const double *e2,
                                          const double *rx, const double *ry,
                                          const double *rz, const double *vx,
                                          const double *vy, const double *vz,
                                          void **handle)
{
    if (!handle || n_sys == 0) return ST_BAD_ARGUMENT;
    const uint64_t n = sys_off[n_sys];
    for (unsigned s = 0; s < n_sys; ++s)
        if (sys_off[s + 1] < sys_off[s] || sys_off[s + 1] - sys_off[s] > 512)
            return ST_TOO_LARGE;
    Ensemble *E = new Ensemble();
    CreateGuard guard{E, tupan_gb300_ensemble_destroy};
    E->n = n;
    E->ns = n_sys;
    E->eta = eta;
    E->shape = g_ens_default;
    if (e_sweep_attributes() != cudaSuccess) return ST_CUDA;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&E->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) !=
        cudaSuccess)
        return ST_CUDA;
    const int narr = 2 + 12 + 12 + 2 + 1;
    if (cudaMalloc((void **)&E->pool, (size_t)narr * n * sizeof(double)) !=
        cudaSuccess)
        return ST_CUDA;
    cudaMemset(E->pool, 0, (size_t)narr * n * sizeof(double));
    double *p = E->pool;
    auto take = [&]() { double *q = p; p += n; return q; };
    EArrays &A = E->A;
    A.m = take();
    A.e2 = take();
    for (int d = 0; d < 3; ++d) A.r[d] = take();
    for (int d = 0; d < 3; ++d) A.v[d] = take();
    for (int d = 0; d < 3; ++d) A.r0[d] = take();
    for (int d = 0; d < 3; ++d) A.v0[d] = take();
    for (int q = 0; q < 6; ++q) A.f0[q] = take();
    for (int q = 0; q < 6; ++q) A.f1[q] = take();
    A.dt[0] = take();
    A.dt[1] = take();
    A.phi = take();
    std::vector<unsigned> sys(n);
    for (unsigned s = 0; s < n_sys; ++s)
        for (uint64_t i = sys_off[s]; i < sys_off[s + 1]; ++i) sys[i] = s;
    std::vector<unsigned> order(n_sys);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) {
        return sys_off[a + 1] - sys_off[a] > sys_off[b + 1] - sys_off[b];
    });
    if (cudaMalloc((void **)&A.sys, n * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->off, (n_sys + 1) * sizeof(uint64_t)) != cudaSuccess ||
        cudaMalloc((void **)&E->order, n_sys * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->active, n_sys * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&E->ctl, n_sys * sizeof(SysCtl)) != cudaSuccess ||
        cudaMalloc((void **)&E->queue, 4 * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->err, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->pack, 3 * n * 3 * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void **)&E->ke, n_sys * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&E->pe, n_sys * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&E->alist, n_sys * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->acount, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->items, (size_t)n_sys * 16 * sizeof(uint2)) !=
            cudaSuccess ||
        cudaMalloc((void **)&E->icount, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->sys_items, n_sys * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->sys_done, n_sys * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->d_tend, sizeof(double)) != cudaSuccess)
        return ST_CUDA;
    cudaMemset(E->acount, 0, sizeof(unsigned));
    cudaMemset(E->icount, 0, sizeof(unsigned));
    cudaMemset(E->sys_items, 0, n_sys * sizeof(unsigned));
    cudaMemset(E->sys_done, 0, n_sys * sizeof(unsigned));
    cudaMemcpy(A.sys, sys.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice);
    cudaMemcpy(E->off, sys_off, (n_sys + 1) * sizeof(uint64_t),
               cudaMemcpyHostToDevice);
    cudaMemcpy(E->order, order.data(), n_sys * sizeof(unsigned),
               cudaMemcpyHostToDevice);
    cudaMemset(E->ctl, 0, n_sys * sizeof(SysCtl));
    cudaMemset(E->err, 0, sizeof(unsigned));
    const double *src[8] = {m, e2, rx, ry, rz, vx, vy, vz};
    double *dst[8] = {A.m, A.e2, A.r[0], A.r[1], A.r[2], A.v[0], A.v[1], A.v[2]};
    for (int k = 0; k < 8; ++k)
        if (cudaMemcpy(dst[k], src[k], n * sizeof(double),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return ST_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return ST_CUDA;
    *handle = E;
    guard.keep();
    return ST_OK;
}

// Persistent launches until every system reaches t_end or fewer than
// E->switch_below systems are left.
static int evolve_persistent(Ensemble *E, double t_end)
{
    std::vector<SysCtl> c(E->ns);
    long long last_steps = -1;
    for (;;) {
        if (cudaMemcpy(c.data(), E->ctl, E->ns * sizeof(SysCtl),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
        unsigned left = 0;
        long long steps = 0;
        for (unsigned s = 0; s < E->ns; ++s) {
            if (fabs(c[s].t) < t_end) ++left;
            steps += c[s].nsteps;
        }
        if (left == 0 || left < E->switch_below) return ST_OK;
        if (steps == last_steps) return ST_DEVICE;
        last_steps = steps;
        RunLaunch R;
        R.A = E->A;
        R.ctl = E->ctl;
        R.off = E->off;
        R.order = E->order;
        R.ns = E->ns;
        R.queue = E->queue;
        R.t_end_p = E->d_tend;
        R.eta = E->eta;
        R.max_steps = E->steps_per_launch;
        R.err = E->err;
        const unsigned grid = (unsigned)std::min<uint64_t>(
            (uint64_t)E->sms * 2, (uint64_t)left);
        if (cudaMemsetAsync(E->queue, 0, sizeof(unsigned), E->stream) !=
            cudaSuccess)
            return ST_CUDA;
        k_e_run<<<grid, RUN_NT, 0, E->stream>>>(R);
        g_launch_count += 1;
        if (cudaGetLastError() != cudaSuccess ||
            cudaStreamSynchronize(E->stream) != cudaSuccess)
            return ST_CUDA;
    }
}

// Steps every system until it reaches t_end: persistent launches (mode 1)
// while at least `switch_below` systems are left, then batched steps (a
// graph of `batch` steps per host check).  Returns the largest step count
// over the systems.
TG_EXPORT int tupan_gb300_ensemble_evolve(void *handle, double t_end, int batch,
                                          long long *max_steps_out)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E) return ST_BAD_ARGUMENT;
    if (batch < 1) batch = 1;
    E->t_end = t_end;
    if (cudaMemcpy(E->d_tend, &t_end, sizeof(double), cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return ST_CUDA;
    if (E->mode == 1) {
        const int rc = evolve_persistent(E, t_end);
        if (rc != ST_OK) return rc;
    }
    // records of the current state for the first step's sweeps
    k_e_pack_all<<<(unsigned)E->sms * 8, 256, 0, E->stream>>>(E->A, E->n,
                                                               E->pack);
    g_launch_count += 1;
    if (E->graph && E->graph_batch != batch) {
        cudaGraphExecDestroy(E->graph);
        E->graph = nullptr;
    }
    if (!E->graph) {
        // one uncaptured step first: launches are validated outside capture
        if (e_step(E) != cudaSuccess) return ST_CUDA;
        if (cudaStreamSynchronize(E->stream) != cudaSuccess) return ST_CUDA;
        unsigned long long before = g_launch_count.load();
        cudaGraph_t g;
        if (cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            return ST_CUDA;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < batch && e == cudaSuccess; ++k) e = e_step(E);
        cudaError_t e2 = cudaStreamEndCapture(E->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) return ST_CUDA;
        if (cudaGraphInstantiate(&E->graph, g, 0) != cudaSuccess) return ST_CUDA;
        cudaGraphDestroy(g);
        E->graph_batch = batch;
        E->launches_per_batch = g_launch_count.load() - before;
        g_launch_count -= E->launches_per_batch;
    }
    std::vector<SysCtl> c(E->ns);
    long long last_steps = -1;
    for (;;) {
        if (cudaMemcpy(c.data(), E->ctl, E->ns * sizeof(SysCtl),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
        bool all = true;
        long long steps = 0;
        for (unsigned s = 0; s < E->ns; ++s) {
            if (fabs(c[s].t) < t_end) all = false;
            steps += c[s].nsteps;
        }
        if (all) break;
        // every replay advances each unfinished system by `batch` steps;
        // no progress means the device state is not what the graph expects
        if (steps == last_steps) return ST_DEVICE;
        last_steps = steps;
        if (cudaGraphLaunch(E->graph, E->stream) != cudaSuccess) return ST_CUDA;
        g_launch_count += E->launches_per_batch;
        if (cudaStreamSynchronize(E->stream) != cudaSuccess) return ST_CUDA;
    }
    long long mx = 0;
    for (unsigned s = 0; s < E->ns; ++s) mx = c[s].nsteps > mx ? c[s].nsteps : mx;
    if (max_steps_out) *max_steps_out = mx;
    unsigned h = 0;
    cudaMemcpy(&h, E->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return h ? ST_DEVICE : ST_OK;
}

// Launch shape of the batched sweep (threads per CTA 128 or 256, full
// i-block 32..512, prefetch 0/1) of one ensemble, or with handle NULL the
// default of ensembles created later.  A captured step graph is rebuilt.
TG_EXPORT int tupan_gb300_ensemble_set_shape(void *handle, int nt, int ib,
                                             int prefetch)
{
    if (!shape_valid(nt, ib, prefetch)) return ST_BAD_ARGUMENT;
    EShape sh;
    sh.nt = nt;
    sh.ib = ib;
    sh.prefetch = prefetch;
    Ensemble *E = (Ensemble *)handle;
    if (!E) {
        g_ens_default = sh;
        return ST_OK;
    }
    if (cudaStreamSynchronize(E->stream) != cudaSuccess) return ST_CUDA;
    E->shape = sh;
    if (E->graph) {
        cudaGraphExecDestroy(E->graph);
        E->graph = nullptr;
        E->graph_batch = -1;
    }
    return ST_OK;
}

// split 1: each AccJerk sweep's per-particle stage (predictor, corrector)
// runs as a launch of its own after the sweep; 0 (default): inside the
// sweep, by the CTA that computed each work item.  Measured on 4096
// systems to t_end = 1: 50.4 s split, 44.3 s inside (the three extra
// launches per step and the stage's own pass over the state cost more than
// the sweep's barrier saves).  A captured step graph is rebuilt.
TG_EXPORT int tupan_gb300_ensemble_set_stage(void *handle, int split)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E || split < 0 || split > 1) return ST_BAD_ARGUMENT;
    if (cudaStreamSynchronize(E->stream) != cudaSuccess) return ST_CUDA;
    E->split_stage = split;
    if (E->graph) {
        cudaGraphExecDestroy(E->graph);
        E->graph = nullptr;
        E->graph_batch = -1;
    }
    return ST_OK;
}

// The shape an ensemble (or, handle NULL, a new one) uses.
TG_EXPORT int tupan_gb300_ensemble_get_shape(void *handle, int *nt, int *ib,
                                             int *prefetch)
{
    const Ensemble *E = (const Ensemble *)handle;
    const EShape &sh = E ? E->shape : g_ens_default;
    if (nt) *nt = sh.nt;
    if (ib) *ib = sh.ib;
    if (prefetch) *prefetch = sh.prefetch;
    return ST_OK;
}

// mode 0: every step of every system in batched launches; mode 1: one CTA
// per system for up to steps_per_launch steps per launch, the last
// switch_below - 1 systems in batched mode (0: persistent to the end).
TG_EXPORT int tupan_gb300_ensemble_set_mode(void *handle, int mode,
                                            int steps_per_launch,
                                            int switch_below)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E || mode < 0 || mode > 1 || steps_per_launch < 1 || switch_below < 0)
        return ST_BAD_ARGUMENT;
    E->mode = mode;
    E->steps_per_launch = steps_per_launch;
    E->switch_below = (unsigned)switch_below;
    return ST_OK;
}

// fp64 kinetic and potential energy of every system (HOST arrays of n_sys).
TG_EXPORT int tupan_gb300_ensemble_energy(void *handle, double *ke, double *pe)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E) return ST_BAD_ARGUMENT;
    k_e_energy<<<E->ns, 256, 0, E->stream>>>(E->A, E->off, E->ke, E->pe);
    g_launch_count += 1;
    if (cudaMemcpyAsync(ke, E->ke, E->ns * sizeof(double),
                        cudaMemcpyDeviceToHost, E->stream) != cudaSuccess ||
        cudaMemcpyAsync(pe, E->pe, E->ns * sizeof(double),
                        cudaMemcpyDeviceToHost, E->stream) != cudaSuccess ||
        cudaStreamSynchronize(E->stream) != cudaSuccess)
        return ST_CUDA;
    return ST_OK;
}

// Times, step counts and state (HOST arrays; any pointer may be NULL).
TG_EXPORT int tupan_gb300_ensemble_get(void *handle, double *t,
                                       long long *nsteps, double *rx,
                                       double *ry, double *rz, double *vx,
                                       double *vy, double *vz)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E) return ST_BAD_ARGUMENT;
    std::vector<SysCtl> c(E->ns);
    cudaMemcpy(c.data(), E->ctl, E->ns * sizeof(SysCtl), cudaMemcpyDeviceToHost);
    for (unsigned s = 0; s < E->ns; ++s) {
        if (t) t[s] = c[s].t;
        if (nsteps) nsteps[s] = c[s].nsteps;
    }
    double *dst[6] = {rx, ry, rz, vx, vy, vz};
    double *src[6] = {E->A.r[0], E->A.r[1], E->A.r[2],
                      E->A.v[0], E->A.v[1], E->A.v[2]};
    for (int k = 0; k < 6; ++k)
        if (dst[k] && cudaMemcpy(dst[k], src[k], E->n * sizeof(double),
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
    return ST_OK;
}

TG_EXPORT int tupan_gb300_ensemble_destroy(void *handle)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E) return ST_BAD_ARGUMENT;
    cudaStreamSynchronize(E->stream);
    if (E->graph) cudaGraphExecDestroy(E->graph);
    cudaFree(E->pool);
    cudaFree(E->A.sys);
    cudaFree(E->off);
    cudaFree(E->order);
    cudaFree(E->alist);
    cudaFree(E->acount);
    cudaFree(E->items);
    cudaFree(E->icount);
    cudaFree(E->sys_items);
    cudaFree(E->sys_done);
    cudaFree(E->d_tend);
    cudaFree(E->active);
    cudaFree(E->ctl);
    cudaFree(E->queue);
    cudaFree(E->err);
    cudaFree(E->pack);
    cudaFree(E->ke);
    cudaFree(E->pe);
    if (E->stream) cudaStreamDestroy(E->stream);
    delete E;
    return ST_OK;
}
