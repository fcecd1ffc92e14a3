// Device-resident Hermite integrator with individual power-of-two block time
// steps (orders 4, 6, 8).
//
// tupan's Hermite integrator advances all particles with one shared step
// (tupan/integrator/hermite.py:390-410).  Here each particle i keeps its own
// time t_i and step dt_i, a power of two quantised with tupan's rule
// (tupan/integrator/__init__.py:59-78) at the block time it is set.  One block
// step:
//   1. t = min_i (t_i + dt_i); the active set is {i : t_i + dt_i == t};
//   2. every particle is predicted to t (Taylor series of r, v, a, j in fp64);
//   3. twice: forces of the active particles against all predicted ones
//      (acc_jerk, and snap_crackle for orders 6 and 8), Hermite correction of
//      the active particles with their own dt_i (the corrector formulas of
//      hermite.py:96-283), and the corrected state written into the predicted
//      set;
//   4. the active particles take the corrected state and the last forces as
//      their new derivatives, and a new dt_i from the Tstep kernel against all
//      particles, quantised at t with dt_max as the cap.
// The active i-sets (1 .. N particles) go through the same sweep launchers as
// everything else, so small sets use the j-split variants.  All fp64 updates
// are compiled without contraction; with EXACT forces a run is bit-identical
// to the numpy restatement of the scheme used by the tests.
//
// Launching.  The size of the active set is decided on the GPU each step.
// By default the steps run as one CUDA graph per batch of steps with no host
// round trip: a WHILE node repeats the block step while the block time is
// below t_end (at most a step budget per launch); inside it, after the
// active set is selected, a SWITCH node picks one of the bodies captured per
// block level -- level L holds active counts in (2^(L-1), 2^L] -- whose
// sweeps have the launch shape chosen for 2^L particles and read the exact
// count on the device (CTAs past it leave at once).  The host-synchronised
// path (read the count back, then launch for it) stays available.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "tg_common.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace tg {
template <typename R>
cudaError_t launch_exact(const Sweep &s, cudaStream_t st, long long budget,
                         unsigned *err);
cudaError_t launch_pack(int kernel, uint64_t n, const void *const *attrs,
                        float4 *out, cudaStream_t st);
cudaError_t launch_split(int kernel, const float4 *irec, const float4 *jrec,
                         uint64_t ni, uint64_t nj, void *const *out,
                         double *partial, int variant, int gsplit, double eta,
                         unsigned *err, cudaStream_t st);
cudaError_t launch_pack_dev(int kernel, uint64_t n, const unsigned *n_dev,
                            const void *const *attrs, float4 *out,
                            cudaStream_t st);
cudaError_t launch_split_dev(int kernel, const float4 *irec,
                             const float4 *jrec, uint64_t ni,
                             const unsigned *ni_dev, uint64_t nj,
                             void *const *out, double *partial, int variant,
                             int gsplit, double eta, const double *pn,
                             unsigned *err, cudaStream_t st);
void choose_split_public(int kernel, uint64_t ni, uint64_t nj, int *variant,
                         int *gsplit);
}  // namespace tg

using namespace tg;

namespace {

constexpr int MAX_LEVELS = 40;   // active-count levels of the graph path

struct BlockCtl {
    unsigned long long t_next_bits;   // min (t_i + dt_i), ordered bits
    unsigned int count;               // active particles
    unsigned int stalled;             // a step did not advance the block time
    // graph path: state kept on the device between steps
    double t_last;                    // block time of the last step
    double t_end;
    long long nsteps, active_sum;
    long long steps_left;             // step budget of the current launch
    unsigned long long launches;      // kernels run by the graph's steps
    int level;                        // level chosen for the current step
    int pad2;
    unsigned long long level_launches[MAX_LEVELS + 1];   // per level body
};

// Per-particle state (SoA, fp64, N each).
struct BState {
    double *m, *e2;
    double *r[3], *v[3];
    double *d[12];        // a(3) j(3) s(3) c(3) at t_i
    double *t, *dt;
    double *rp[3], *vp[3], *pd[6];    // predicted r, v, a, j at block time
    unsigned *idx;                    // active particle indices
    // compact active arrays
    double *cm, *ce2, *cr[3], *cv[3];
    double *cf[12];       // forces of the last evaluation: a j s c
    double *cdt[2];       // Tstep outputs
};

__device__ __forceinline__ double d_block_tstep(double min_ts, double t,
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

#define GRID_LOOP(i, n)                                                       \
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;       \
         i < (n); i += (uint64_t)gridDim.x * blockDim.x)

__global__ void k_reset(BlockCtl *c)
{
    c->t_next_bits = 0x7ff0000000000000ull;
    c->count = 0;
}

// t = min (t_i + dt_i): non-negative doubles order like their bit patterns.
__global__ void k_next_time(BState S, uint64_t n, BlockCtl *c)
{
    unsigned long long best = 0x7ff0000000000000ull;
    GRID_LOOP(i, n)
    {
        unsigned long long b =
            (unsigned long long)__double_as_longlong(S.t[i] + S.dt[i]);
        best = b < best ? b : best;
    }
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, best, off);
        best = o < best ? o : best;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(&c->t_next_bits, best);
}

// Active-set compaction (warp-aggregated atomics; the order of the active
// list does not change any result: each active particle is independent).
__global__ void k_select(BState S, uint64_t n, BlockCtl *c)
{
    const double tn = __longlong_as_double((long long)c->t_next_bits);
    GRID_LOOP(i, n)
    {
        const bool act = (S.t[i] + S.dt[i] == tn);
        const unsigned mask = __ballot_sync(__activemask(), act);
        if (!mask) continue;
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(mask) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&c->count, __popc(mask));
        base = __shfl_sync(__activemask(), base, leader);
        if (act) S.idx[base + __popc(mask & ((1u << lane) - 1))] = (unsigned)i;
    }
}

// Prediction of every particle to the block time (Taylor series in fp64).
template <int ORDER>
__global__ void k_predict_all(BState S, uint64_t n, const BlockCtl *c)
{
    const double tn = __longlong_as_double((long long)c->t_next_bits);
    GRID_LOOP(i, n)
    {
        const double h = tn - S.t[i];
        for (int d = 0; d < 3; ++d) {
            const double r = S.r[d][i], v = S.v[d][i];
            const double a = S.d[d][i], j = S.d[3 + d][i];
            if (ORDER == 4) {
                S.rp[d][i] = r + h * (v + h * (a + h * j / 3) / 2);
                S.vp[d][i] = v + h * (a + h * j / 2);
                S.pd[d][i] = a + h * j;
                S.pd[3 + d][i] = j;
            } else {
                const double s = S.d[6 + d][i], cr = S.d[9 + d][i];
                S.rp[d][i] = r + h * (v + h * (a + h * (j + h * (s + h * cr / 5) / 4) / 3) / 2);
                S.vp[d][i] = v + h * (a + h * (j + h * (s + h * cr / 4) / 3) / 2);
                S.pd[d][i] = a + h * (j + h * (s + h * cr / 3) / 2);
                S.pd[3 + d][i] = j + h * (s + h * cr / 2);
            }
        }
    }
}

// Compact i-arrays of the active particles from the predicted set.
__global__ void k_gather(BState S, const BlockCtl *c)
{
    const uint64_t na = c->count;
    GRID_LOOP(k, na)
    {
        const unsigned i = S.idx[k];
        S.cm[k] = S.m[i];
        S.ce2[k] = S.e2[i];
        for (int d = 0; d < 3; ++d) {
            S.cr[d][k] = S.rp[d][i];
            S.cv[d][k] = S.vp[d][i];
        }
    }
}

// Hermite correction of the active particles over their own dt_i; the
// corrected r, v go into the compact arrays and into the predicted set, and
// the new a, j into the predicted derivatives.
template <int ORDER>
__global__ void k_correct_active(BState S, const BlockCtl *c)
{
    const uint64_t na = c->count;
    GRID_LOOP(k, na)
    {
        const unsigned i = S.idx[k];
        const double tau = S.dt[i];
        for (int d = 0; d < 3; ++d) {
            const double a0 = S.d[d][i], a1 = S.cf[d][k];
            const double j0 = S.d[3 + d][i], j1 = S.cf[3 + d][k];
            const double v0 = S.v[d][i], r0 = S.r[d][i];
            double v1, r1;
            if (ORDER == 4) {
                v1 = ((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + v0;
                r1 = ((a0 - a1) * tau / 6 + (v0 + v1)) * tau / 2 + r0;
            } else if (ORDER == 6) {
                const double s0 = S.d[6 + d][i], s1 = S.cf[6 + d][k];
                v1 = (((s0 + s1) * tau / 12 + (j0 - j1)) * tau / 5 + (a0 + a1)) * tau / 2 + v0;
                r1 = (((j0 + j1) * tau / 12 + (a0 - a1)) * tau / 5 + (v0 + v1)) * tau / 2 + r0;
            } else {
                const double s0 = S.d[6 + d][i], s1 = S.cf[6 + d][k];
                const double c0 = S.d[9 + d][i], c1 = S.cf[9 + d][k];
                v1 = ((((c0 - c1) * tau / 20 + (s0 + s1)) * tau / 3 + 3 * (j0 - j1)) * tau / 14 + (a0 + a1)) * tau / 2 + v0;
                r1 = ((((s0 - s1) * tau / 20 + (j0 + j1)) * tau / 3 + 3 * (a0 - a1)) * tau / 14 + (v0 + v1)) * tau / 2 + r0;
            }
            S.cr[d][k] = r1;
            S.cv[d][k] = v1;
            S.rp[d][i] = r1;
            S.vp[d][i] = v1;
            S.pd[d][i] = a1;
            S.pd[3 + d][i] = j1;
        }
    }
}

// Commit the active particles at the block time.
template <int ORDER>
__global__ void k_commit(BState S, const BlockCtl *c)
{
    const uint64_t na = c->count;
    const double tn = __longlong_as_double((long long)c->t_next_bits);
    GRID_LOOP(k, na)
    {
        const unsigned i = S.idx[k];
        for (int d = 0; d < 3; ++d) {
            S.r[d][i] = S.cr[d][k];
            S.v[d][i] = S.cv[d][k];
        }
        const int nd = ORDER == 4 ? 6 : 12;
        for (int q = 0; q < nd; ++q) S.d[q][i] = S.cf[q][k];
        S.t[i] = tn;
    }
}

__global__ void k_new_dt(BState S, const BlockCtl *c, double dt_max)
{
    const uint64_t na = c->count;
    const double tn = __longlong_as_double((long long)c->t_next_bits);
    GRID_LOOP(k, na)
    {
        const unsigned i = S.idx[k];
        S.dt[i] = d_block_tstep(fabs(S.cdt[0][k]), tn, dt_max);
    }
}

// Level of an active count: L with count in (2^(L-1), 2^L]; 0 for 1.
__device__ __forceinline__ int count_level(unsigned count)
{
    return count <= 1u ? 0 : 32 - __clz(count - 1u);
}

// Graph path: choose the level body of this step (none for an empty set).
__global__ void k_level(BlockCtl *c, cudaGraphConditionalHandle hs, int nb)
{
    if (threadIdx.x != 0) return;
    const unsigned count = c->count;
    const int lv = count ? count_level(count) : nb;
    c->level = lv;
    cudaGraphSetConditional(hs, (unsigned)(lv < nb ? lv : nb));
}

// Graph path: close the step (statistics, block time) and decide whether the
// WHILE node runs another: the block time advanced, is still below t_end and
// the launch's step budget is not spent.  `pre` kernels ran before the level
// body and this one.
__global__ void k_step_end(BlockCtl *c, cudaGraphConditionalHandle hw,
                           int nb, unsigned long long pre)
{
    if (threadIdx.x != 0) return;
    const double tn = __longlong_as_double((long long)c->t_next_bits);
    const unsigned count = c->count;
    bool progress = false;
    if (count > 0 && tn > c->t_last) {
        progress = true;
        c->nsteps += 1;
        c->active_sum += count;
        c->t_last = tn;
    }
    if (!progress) c->stalled = 1;
    c->launches += pre + (c->level < nb ? c->level_launches[c->level] : 0ull);
    c->steps_left -= 1;
    const bool more = progress && c->t_last < c->t_end && c->steps_left > 0;
    cudaGraphSetConditional(hw, more ? 1u : 0u);
}

// Graph path: arm a launch (end time, step budget, and the host's view of
// the block time and counters, which the host-synchronised path may have
// advanced).
__global__ void k_arm(BlockCtl *c, double t_end, long long steps,
                      double t_last, long long nsteps, long long active_sum)
{
    if (threadIdx.x != 0) return;
    c->t_end = t_end;
    c->steps_left = steps;
    c->stalled = 0;
    c->t_last = t_last;
    c->nsteps = nsteps;
    c->active_sum = active_sum;
}

__global__ void k_init_dt(BState S, uint64_t n, double dt_max)
{
    GRID_LOOP(i, n)
    {
        S.dt[i] = d_block_tstep(fabs(S.cdt[0][i]), 0.0, dt_max);
        S.t[i] = 0.0;
    }
}

struct Block {
    uint64_t n = 0;
    int order = 4;
    int mode = MODE_EXACT;
    int sms = 152;
    double eta = 0.0, dt_max = 0.0;
    double t = 0.0;
    long long nsteps = 0;
    long long active_sum = 0;
    cudaStream_t stream = nullptr;
    BlockCtl *ctl = nullptr;
    unsigned *err = nullptr;
    double *pool = nullptr;
    BState S;
    float4 *pack_i = nullptr, *pack_j = nullptr;
    double *partial = nullptr;
    // graph path
    int use_graphs = 1;           // 1: graph path, 0: host-synchronised
    bool graph_failed = false;    // building the graph failed: host path
    cudaGraphExec_t exec = nullptr;
    int nlevels = 0;
    const unsigned *count_dev = nullptr;   // &ctl->count while capturing
    unsigned long long host_launches = 0;  // ctl->launches already counted
};

unsigned grid_for(uint64_t n, int sms)
{
    uint64_t b = (n + 255) / 256;
    uint64_t cap = (uint64_t)sms * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// One sweep of ni (compact or full) i-particles against all predicted j.
cudaError_t bsweep(Block *b, int kernel, uint64_t ni, const double *const *ia,
                   const double *const *ja, double *const *out, double eta)
{
    if (ni == 0) return cudaSuccess;
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = kernel;
    s.mode = b->mode;
    s.ni = ni;
    s.nj = b->n;
    for (int a = 0; a < n_attr(kernel); ++a) {
        s.ip[a] = ia[a];
        s.jp[a] = ja[a];
    }
    for (int o = 0; o < n_out(kernel); ++o) s.out[o] = out[o];
    s.scal[0] = eta;
    // while a level body is captured, ni is the level's bound and the count
    // is read on the device
    s.ni_dev = b->count_dev;
    if (b->mode == MODE_EXACT)
        return launch_exact<double>(s, b->stream, 1LL << 20, b->err);
    cudaError_t e = launch_pack_dev(kernel, ni, b->count_dev, s.ip, b->pack_i,
                                    b->stream);
    if (e == cudaSuccess) e = launch_pack(kernel, b->n, s.jp, b->pack_j, b->stream);
    if (e != cudaSuccess) return e;
    int variant, gsplit;
    choose_split_public(kernel, ni, b->n, &variant, &gsplit);
    return launch_split_dev(kernel, b->pack_i, b->pack_j, ni, b->count_dev,
                            b->n, s.out, b->partial, variant, gsplit, eta,
                            nullptr, b->err, b->stream);
}

// Forces of the ni i-particles given by (m, e2, r, v) arrays against the
// predicted set, into S.cf (a, j and for orders 6/8 s, c).
cudaError_t bforces(Block *b, uint64_t ni, const double *im, const double *ie2,
                    double *const *ir, double *const *iv, double *const *out)
{
    BState &S = b->S;
    const double *ia[14] = {im, ir[0], ir[1], ir[2], ie2, iv[0], iv[1], iv[2],
                            out[0], out[1], out[2], out[3], out[4], out[5]};
    const double *ja[14] = {S.m, S.rp[0], S.rp[1], S.rp[2], S.e2,
                            S.vp[0], S.vp[1], S.vp[2], S.pd[0], S.pd[1],
                            S.pd[2], S.pd[3], S.pd[4], S.pd[5]};
    cudaError_t e = bsweep(b, K_ACC_JERK, ni, ia, ja, out, 0.0);
    if (e != cudaSuccess || b->order < 6) return e;
    return bsweep(b, K_SNAP_CRACKLE, ni, ia, ja, out + 6, 0.0);
}

template <int ORDER>
cudaError_t step_body(Block *b, uint64_t na);

template <int ORDER>
int block_step(Block *b)
{
    BState &S = b->S;
    cudaStream_t st = b->stream;
    const unsigned g = grid_for(b->n, b->sms);
    k_reset<<<1, 1, 0, st>>>(b->ctl);
    k_next_time<<<g, 256, 0, st>>>(S, b->n, b->ctl);
    k_select<<<g, 256, 0, st>>>(S, b->n, b->ctl);
    k_predict_all<ORDER><<<g, 256, 0, st>>>(S, b->n, b->ctl);
    k_gather<<<g, 256, 0, st>>>(S, b->ctl);
    g_launch_count += 5;
    BlockCtl c;
    if (cudaMemcpyAsync(&c, b->ctl, sizeof(c), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ST_CUDA;
    const uint64_t na = c.count;
    if (step_body<ORDER>(b, na) != cudaSuccess) return ST_CUDA;
    double tn;
    memcpy(&tn, &c.t_next_bits, sizeof(tn));
    b->t = tn;
    b->nsteps += 1;
    b->active_sum += (long long)na;
    return ST_OK;
}

// The forces, corrections, commit and new steps of one block step for an
// active set of at most `na` particles (count read on the device when
// count_dev is set).
template <int ORDER>
cudaError_t step_body(Block *b, uint64_t na)
{
    BState &S = b->S;
    cudaStream_t st = b->stream;
    const unsigned ga = grid_for(na, b->sms);
    for (int pass = 0; pass < 2; ++pass) {
        cudaError_t e = bforces(b, na, S.cm, S.ce2, S.cr, S.cv, S.cf);
        if (e != cudaSuccess) return e;
        k_correct_active<ORDER><<<ga, 256, 0, st>>>(S, b->ctl);
        g_launch_count += 1;
    }
    k_commit<ORDER><<<ga, 256, 0, st>>>(S, b->ctl);
    g_launch_count += 1;
    const double *ia[8] = {S.cm, S.cr[0], S.cr[1], S.cr[2], S.ce2,
                           S.cv[0], S.cv[1], S.cv[2]};
    const double *ja[8] = {S.m, S.rp[0], S.rp[1], S.rp[2], S.e2,
                           S.vp[0], S.vp[1], S.vp[2]};
    cudaError_t e = bsweep(b, K_TSTEP, na, ia, ja, S.cdt, b->eta);
    if (e != cudaSuccess) return e;
    k_new_dt<<<ga, 256, 0, st>>>(S, b->ctl, b->dt_max);
    g_launch_count += 1;
    return cudaGetLastError();
}

// Builds the graph path: WHILE { select; SWITCH(level) { body }; end }.
// Host work only (capture into graphs); nothing runs.
template <int ORDER>
cudaError_t build_graph(Block *b)
{
    BState &S = b->S;
    cudaStream_t st = b->stream;
    const unsigned g = grid_for(b->n, b->sms);
    int nb = 1;
    while ((1ull << (nb - 1)) < b->n && nb < MAX_LEVELS) ++nb;
    b->nlevels = nb;
    cudaGraph_t G = nullptr;
    TG_CUDA_TRY(cudaGraphCreate(&G, 0));
    cudaGraphConditionalHandle hw, hs;
    cudaError_t e = cudaGraphConditionalHandleCreate(&hw, G, 1,
                                                     cudaGraphCondAssignDefault);
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wn;
    if (e == cudaSuccess) e = cudaGraphAddNode(&wn, G, nullptr, nullptr, 0, &wp);
    if (e != cudaSuccess) { cudaGraphDestroy(G); return e; }
    cudaGraph_t W = wp.conditional.phGraph_out[0];

    const unsigned long long c0 = g_launch_count.load();
    e = cudaStreamBeginCaptureToGraph(st, W, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { cudaGraphDestroy(G); return e; }
    k_reset<<<1, 1, 0, st>>>(b->ctl);
    k_next_time<<<g, 256, 0, st>>>(S, b->n, b->ctl);
    k_select<<<g, 256, 0, st>>>(S, b->n, b->ctl);
    k_predict_all<ORDER><<<g, 256, 0, st>>>(S, b->n, b->ctl);
    k_gather<<<g, 256, 0, st>>>(S, b->ctl);
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hs, cg, 0, 0);
    cudaGraphNodeParams sp = {};
    sp.type = cudaGraphNodeTypeConditional;
    sp.conditional.handle = hs;
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = (unsigned)nb;
    cudaGraphNode_t sn;
    if (e == cudaSuccess) {
        k_level<<<1, 32, 0, st>>>(b->ctl, hs, nb);
        e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd);
    }
    if (e == cudaSuccess) e = cudaGraphAddNode(&sn, cg, deps, nullptr, nd, &sp);
    if (e == cudaSuccess)
        e = cudaStreamUpdateCaptureDependencies(st, &sn, nullptr, 1,
                                                cudaStreamSetCaptureDependencies);
    // reset, next_time, select, predict, gather, level, step_end
    const unsigned long long pre = 7;
    if (e == cudaSuccess)
        k_step_end<<<1, 32, 0, st>>>(b->ctl, hw, nb, pre);
    cudaGraph_t Wout = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(st, &Wout);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGetLastError();
    // one body per level, its sweeps shaped for the level's largest count
    unsigned long long per_level[MAX_LEVELS + 1];
    memset(per_level, 0, sizeof(per_level));
    b->count_dev = &b->ctl->count;
    for (int lv = 0; lv < nb && e == cudaSuccess; ++lv) {
        uint64_t na = 1ull << lv;
        if (na > b->n) na = b->n;
        const unsigned long long l0 = g_launch_count.load();
        e = cudaStreamBeginCaptureToGraph(st, sp.conditional.phGraph_out[lv],
                                          nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) break;
        cudaError_t eb = step_body<ORDER>(b, na);
        cudaGraph_t bout = nullptr;
        e = cudaStreamEndCapture(st, &bout);
        if (e == cudaSuccess) e = eb;
        per_level[lv] = g_launch_count.load() - l0;
    }
    b->count_dev = nullptr;
    g_launch_count -= g_launch_count.load() - c0;   // nothing ran yet
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, G, 0);
    cudaGraphDestroy(G);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e;
    }
    // the per-level launch counts let the device count the kernels it runs
    e = cudaMemcpyAsync(b->ctl->level_launches, per_level, sizeof(per_level),
                        cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// Graph-path evolution: launches of up to `batch` steps until the block time
// reaches t_end or max_steps steps are taken.
int evolve_graph(Block *b, double t_end, long long max_steps)
{
    cudaStream_t st = b->stream;
    long long taken = 0;
    for (;;) {
        if (!(b->t < t_end) || (max_steps > 0 && taken >= max_steps)) break;
        long long budget = 4096;
        if (max_steps > 0 && max_steps - taken < budget)
            budget = max_steps - taken;
        k_arm<<<1, 32, 0, st>>>(b->ctl, t_end, budget, b->t, b->nsteps,
                                b->active_sum);
        g_launch_count += 1;
        if (cudaGraphLaunch(b->exec, st) != cudaSuccess) return ST_CUDA;
        BlockCtl c;
        if (cudaMemcpyAsync(&c, b->ctl, sizeof(c), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return ST_CUDA;
        g_launch_count += c.launches - b->host_launches;
        b->host_launches = c.launches;
        taken += c.nsteps - b->nsteps;
        b->nsteps = c.nsteps;
        b->active_sum = c.active_sum;
        // the block time must advance (a zero or non-finite step would loop)
        if (c.stalled && !(c.t_last > b->t)) return ST_DEVICE;
        b->t = c.t_last;
        if (c.stalled) return ST_DEVICE;
    }
    return ST_OK;
}

}  // namespace

// ===========================================================================
// C-ABI of the block-step driver (no counterpart in the reference: tupan's
// Hermite integrator has only a shared step).
// ===========================================================================

// Creates a system from HOST arrays and initialises forces and steps at t=0.
// order 4, 6 or 8; mode 0 EXACT / 1 SPLIT; dt_max caps every step.
TG_EXPORT int tupan_gb300_block_destroy(void *handle);

TG_EXPORT int tupan_gb300_block_create(uint64_t n, int order, int mode,
                                       double eta, double dt_max,
                                       const double *m, const double *e2,
                                       const double *rx, const double *ry,
                                       const double *rz, const double *vx,
                                       const double *vy, const double *vz,
                                       void **handle)
{
    if (!handle || n == 0 || n > 0xffffffffull ||
        (order != 4 && order != 6 && order != 8) || !(dt_max > 0))
        return ST_BAD_ARGUMENT;
    Block *b = new Block();
    CreateGuard guard{b, tupan_gb300_block_destroy};
    b->n = n;
    b->order = order;
    b->mode = mode == MODE_SPLIT ? MODE_SPLIT : MODE_EXACT;
    b->eta = eta;
    b->dt_max = dt_max;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) !=
        cudaSuccess)
        return ST_CUDA;
    // m e2 r3 v3 d12 t dt rp3 vp3 pd6 | cm ce2 cr3 cv3 cf12 cdt2 = 56 arrays
    const int narr = 56;
    if (cudaMalloc((void **)&b->pool, (size_t)narr * n * sizeof(double)) !=
        cudaSuccess)
        return ST_CUDA;
    cudaMemset(b->pool, 0, (size_t)narr * n * sizeof(double));
    double *p = b->pool;
    auto take = [&]() { double *q = p; p += n; return q; };
    BState &S = b->S;
    S.m = take();
    S.e2 = take();
    for (int d = 0; d < 3; ++d) S.r[d] = take();
    for (int d = 0; d < 3; ++d) S.v[d] = take();
    for (int q = 0; q < 12; ++q) S.d[q] = take();
    S.t = take();
    S.dt = take();
    for (int d = 0; d < 3; ++d) S.rp[d] = take();
    for (int d = 0; d < 3; ++d) S.vp[d] = take();
    for (int q = 0; q < 6; ++q) S.pd[q] = take();
    S.cm = take();
    S.ce2 = take();
    for (int d = 0; d < 3; ++d) S.cr[d] = take();
    for (int d = 0; d < 3; ++d) S.cv[d] = take();
    for (int q = 0; q < 12; ++q) S.cf[q] = take();
    for (int q = 0; q < 2; ++q) S.cdt[q] = take();
    if (cudaMalloc((void **)&S.idx, n * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&b->ctl, sizeof(BlockCtl)) != cudaSuccess ||
        cudaMalloc((void **)&b->err, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&b->pack_i, n * 5 * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void **)&b->pack_j, n * 5 * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void **)&b->partial, (size_t)64 * 7 * n * sizeof(double)) !=
            cudaSuccess)
        return ST_CUDA;
    cudaMemset(b->err, 0, sizeof(unsigned));
    cudaMemset(b->ctl, 0, sizeof(BlockCtl));
    const double *src[8] = {m, e2, rx, ry, rz, vx, vy, vz};
    double *dst[8] = {S.m, S.e2, S.r[0], S.r[1], S.r[2], S.v[0], S.v[1], S.v[2]};
    for (int k = 0; k < 8; ++k)
        if (cudaMemcpy(dst[k], src[k], n * sizeof(double),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return ST_CUDA;
    // t = 0: forces and steps of all particles (the predicted set is the
    // initial state itself).
    for (int d = 0; d < 3; ++d) {
        cudaMemcpy(S.rp[d], S.r[d], n * sizeof(double), cudaMemcpyDeviceToDevice);
        cudaMemcpy(S.vp[d], S.v[d], n * sizeof(double), cudaMemcpyDeviceToDevice);
    }
    {
        // acc/jerk of everything, then snap/crackle with those a, j on both
        // the i and the j side
        const double *ia[14] = {S.m, S.r[0], S.r[1], S.r[2], S.e2, S.v[0],
                                S.v[1], S.v[2], S.d[0], S.d[1], S.d[2],
                                S.d[3], S.d[4], S.d[5]};
        if (bsweep(b, K_ACC_JERK, n, ia, ia, S.d, 0.0) != cudaSuccess)
            return ST_CUDA;
        if (order >= 6 &&
            bsweep(b, K_SNAP_CRACKLE, n, ia, ia, S.d + 6, 0.0) != cudaSuccess)
            return ST_CUDA;
    }
    for (int q = 0; q < 6; ++q)
        cudaMemcpyAsync(S.pd[q], S.d[q], n * sizeof(double),
                        cudaMemcpyDeviceToDevice, b->stream);
    {
        const double *ia[8] = {S.m, S.r[0], S.r[1], S.r[2], S.e2,
                               S.v[0], S.v[1], S.v[2]};
        if (bsweep(b, K_TSTEP, n, ia, ia, S.cdt, eta) != cudaSuccess)
            return ST_CUDA;
    }
    k_init_dt<<<grid_for(n, b->sms), 256, 0, b->stream>>>(S, n, dt_max);
    g_launch_count += 1;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return ST_CUDA;
    *handle = b;
    guard.keep();
    return ST_OK;
}

// Block steps until the block time reaches t_end (or max_steps steps).
// Returns the time, the number of block steps and the active particles
// summed over them.
TG_EXPORT int tupan_gb300_block_evolve(void *handle, double t_end,
                                       long long max_steps, double *t_out,
                                       long long *steps_out,
                                       long long *active_out)
{
    Block *b = (Block *)handle;
    if (!b) return ST_BAD_ARGUMENT;
    if (b->use_graphs && !b->graph_failed && !b->exec) {
        const cudaError_t e = b->order == 4 ? build_graph<4>(b)
                            : b->order == 6 ? build_graph<6>(b)
                                            : build_graph<8>(b);
        if (e != cudaSuccess) {
            // conditional graph nodes unavailable: the host-synchronised
            // path runs instead (tupan_gb300_block_launch_mode reports it)
            b->graph_failed = true;
            cudaGetLastError();
        }
    }
    if (b->use_graphs && b->exec) {
        const int rc = evolve_graph(b, t_end, max_steps);
        if (rc) return rc;
        if (cudaStreamSynchronize(b->stream) != cudaSuccess) return ST_CUDA;
        unsigned herr = 0;
        cudaMemcpy(&herr, b->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
        if (t_out) *t_out = b->t;
        if (steps_out) *steps_out = b->nsteps;
        if (active_out) *active_out = b->active_sum;
        return herr ? ST_DEVICE : ST_OK;
    }
    long long k = 0;
    while (b->t < t_end && (max_steps <= 0 || k < max_steps)) {
        const double t_before = b->t;
        int rc = b->order == 4 ? block_step<4>(b)
               : b->order == 6 ? block_step<6>(b) : block_step<8>(b);
        if (rc) return rc;
        // the block time must advance (a zero or non-finite step would
        // loop forever)
        if (!(b->t > t_before)) return ST_DEVICE;
        ++k;
    }
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return ST_CUDA;
    unsigned herr = 0;
    cudaMemcpy(&herr, b->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (t_out) *t_out = b->t;
    if (steps_out) *steps_out = b->nsteps;
    if (active_out) *active_out = b->active_sum;
    return herr ? ST_DEVICE : ST_OK;
}

// State at each particle's own time t_i, and t_i and dt_i (HOST arrays).
TG_EXPORT int tupan_gb300_block_get_state(void *handle, double *rx, double *ry,
                                          double *rz, double *vx, double *vy,
                                          double *vz, double *t, double *dt)
{
    Block *b = (Block *)handle;
    if (!b) return ST_BAD_ARGUMENT;
    BState &S = b->S;
    double *dst[8] = {rx, ry, rz, vx, vy, vz, t, dt};
    double *src[8] = {S.r[0], S.r[1], S.r[2], S.v[0], S.v[1], S.v[2], S.t, S.dt};
    for (int q = 0; q < 8; ++q)
        if (dst[q] && cudaMemcpy(dst[q], src[q], b->n * sizeof(double),
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
    return ST_OK;
}

// How block steps are launched: 1 (default) one CUDA graph per batch of
// steps, the active-set size decided and used on the device (WHILE over
// steps, SWITCH over active-count levels); 0 host-synchronised (the count is
// read back each step).  Returns the previous setting.
TG_EXPORT int tupan_gb300_block_set_graphs(void *handle, int on)
{
    Block *b = (Block *)handle;
    if (!b) return -1;
    const int old = b->use_graphs;
    b->use_graphs = on ? 1 : 0;
    return old;
}

// The launch path the last evolve used or will use: 1 graphs, 0
// host-synchronised (also when building the graph failed).
TG_EXPORT int tupan_gb300_block_launch_mode(void *handle)
{
    Block *b = (Block *)handle;
    if (!b) return -1;
    return (b->use_graphs && !b->graph_failed) ? 1 : 0;
}

TG_EXPORT int tupan_gb300_block_destroy(void *handle)
{
    Block *b = (Block *)handle;
    if (!b) return ST_BAD_ARGUMENT;
    cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    cudaFree(b->pool);
    cudaFree(b->S.idx);
    cudaFree(b->ctl);
    cudaFree(b->err);
    cudaFree(b->pack_i);
    cudaFree(b->pack_j);
    cudaFree(b->partial);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return ST_OK;
}
