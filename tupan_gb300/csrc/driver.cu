// Device-resident Hermite driver: shared adaptive (power-of-two) steps of
// order 2/4/6/8 with the particles kept in HBM between steps.
//
// One step is tupan's Hermite.do_step (tupan/integrator/hermite.py:390-410):
// Tstep sweep -> min |dt| -> block quantisation (integrator/__init__.py:
// 59-78) -> copy of the state -> forces on the copy -> predictor -> two
// corrector passes, each after a force sweep on the predicted state.  The
// step size lives in device memory, so a step is a fixed sequence of
// launches that can be replayed from a CUDA graph without host round trips;
// steps past t_end are no-ops (the control block's `done` flag).
//
// The predictor/corrector and quantisation kernels are compiled with
// -fmad=false and evaluate each update in the reference's order, so with
// EXACT-mode forces a run is bit-identical to tupan's own integrator on its C
// backend; with SPLIT-mode forces only the pairwise sums change.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

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
void choose_split_public(int kernel, uint64_t ni, uint64_t nj, int *variant,
                         int *gsplit);
}  // namespace tg

using namespace tg;

namespace {

// Control block of one system (device memory).
struct StepCtl {
    double t;          // current time (type(ps).t_curr)
    double t_end;
    double eta;
    double tau;        // step of the current iteration
    unsigned long long min_ts_bits;   // min |dt_a| as ordered bits
    int done;          // 1 once |t| >= t_end: further steps are no-ops
    int pad;
    long long nsteps;
};

__device__ __forceinline__ double d_base_tstep(double t, double t_end,
                                               double eta)
{
    // integrator/__init__.py:48-57
    double dt = fmin(fabs(t_end) - fabs(t), fabs(eta));
    dt = fmax(dt, fabs(t_end) * (2.0 * 2.220446049250313e-16));
    return copysign(dt, eta);
}

__device__ __forceinline__ double d_block_tstep(double min_ts, double t,
                                                double tau)
{
    // integrator/__init__.py:59-78 (power = int(log2(min_ts) - 1): C++'s
    // conversion truncates toward zero like Python's int(); the logarithm
    // is exact at powers of two, see quantised_power).
    long long power = quantised_power(min_ts);
    double min_bts = ldexp(1.0, (int)power);
    double t_next = t + min_bts;
    for (int k = 0; k < 2100 && fmod(t_next, min_bts) != 0.0; ++k)
        min_bts /= 2.0;
    min_bts = copysign(min_bts, tau);
    if (fabs(min_bts) > fabs(tau)) min_bts = tau;
    return min_bts;
}

__global__ void k_begin_step(StepCtl *c)
{
    if (threadIdx.x || blockIdx.x) return;
    if (fabs(c->t) >= c->t_end) {
        c->done = 1;
        c->tau = 0.0;
        return;
    }
    c->done = 0;
    c->tau = d_base_tstep(c->t, c->t_end, c->eta);
    c->min_ts_bits = 0x7ff0000000000000ull;   // +inf
}

// min |dt_a| over particles; non-negative doubles order like their bits.
__global__ void k_min_abs(const double *x, uint64_t n, StepCtl *c)
{
    if (c->done) return;
    unsigned long long best = 0x7ff0000000000000ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        unsigned long long b = (unsigned long long)__double_as_longlong(fabs(x[i]));
        best = b < best ? b : best;
    }
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, best, off);
        best = o < best ? o : best;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(&c->min_ts_bits, best);
}

__global__ void k_block_tstep(StepCtl *c)
{
    if (threadIdx.x || blockIdx.x || c->done) return;
    double min_ts = __longlong_as_double((long long)c->min_ts_bits);
    c->tau = d_block_tstep(min_ts, c->t, c->tau);
}

__global__ void k_end_step(StepCtl *c, double *tau_log, long long cap)
{
    if (threadIdx.x || blockIdx.x || c->done) return;
    if (tau_log && c->nsteps < cap) tau_log[c->nsteps] = c->tau;
    c->t += c->tau;
    c->nsteps += 1;
}

struct Arrays {
    double *m, *e2;
    double *r[3], *v[3];        // current state (ps / ps1)
    double *r0[3], *v0[3];      // copy at the start of the step (ps0)
    double *f0[12], *f1[12];    // a(3) j(3) s(3) c(3) of ps0 and ps1
    double *dt[2];              // tstep outputs (tstep, tstepij)
};

__global__ void k_copy_state(Arrays A, uint64_t n, const StepCtl *c)
{
    if (c->done) return;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < 3; ++d) {
            A.r0[d][i] = A.r[d][i];
            A.v0[d][i] = A.v[d][i];
        }
}

// Hn.epredict position/velocity updates (hermite.py:33-38, :83-88,
// :136-157, :210-235).
template <int ORDER>
__global__ void k_predict(Arrays A, uint64_t n, const StepCtl *c)
{
    if (c->done) return;
    const double tau = c->tau;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < 3; ++d) {
            const double a = A.f0[d][i];
            const double v = A.v[d][i];
            double rr, vv;
            if (ORDER == 2) {
                rr = (a * tau / 2 + v) * tau;
                vv = a * tau;
            } else if (ORDER == 4) {
                const double j = A.f0[3 + d][i];
                rr = ((j * tau / 3 + a) * tau / 2 + v) * tau;
                vv = (j * tau / 2 + a) * tau;
            } else if (ORDER == 6) {
                const double j = A.f0[3 + d][i], s = A.f0[6 + d][i];
                rr = (((s * tau / 4 + j) * tau / 3 + a) * tau / 2 + v) * tau;
                vv = ((s * tau / 3 + j) * tau / 2 + a) * tau;
            } else {
                const double j = A.f0[3 + d][i], s = A.f0[6 + d][i],
                             cr = A.f0[9 + d][i];
                rr = ((((cr * tau / 5 + s) * tau / 4 + j) * tau / 3 + a) *
                          tau / 2 + v) * tau;
                vv = (((cr * tau / 4 + s) * tau / 3 + j) * tau / 2 + a) * tau;
            }
            A.r[d][i] = A.r[d][i] + rr;
            A.v[d][i] = v + vv;
        }
}

// Hn.ecorrect (hermite.py:46-57, :96-119, :162-195, :238-283): velocities
// first, positions from the corrected velocities.
template <int ORDER>
__global__ void k_correct(Arrays A, uint64_t n, const StepCtl *c)
{
    if (c->done) return;
    const double tau = c->tau;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < 3; ++d) {
            const double a0 = A.f0[d][i], a1 = A.f1[d][i];
            const double v0 = A.v0[d][i], r0 = A.r0[d][i];
            double v1, r1;
            if (ORDER == 2) {
                v1 = ((a0 + a1) * tau / 2 + v0);
                r1 = ((v0 + v1) * tau / 2 + r0);
            } else if (ORDER == 4) {
                const double j0 = A.f0[3 + d][i], j1 = A.f1[3 + d][i];
                v1 = (((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + v0);
                r1 = (((a0 - a1) * tau / 6 + (v0 + v1)) * tau / 2 + r0);
            } else if (ORDER == 6) {
                const double j0 = A.f0[3 + d][i], j1 = A.f1[3 + d][i];
                const double s0 = A.f0[6 + d][i], s1 = A.f1[6 + d][i];
                v1 = ((((s0 + s1) * tau / 12 + (j0 - j1)) * tau / 5 +
                       (a0 + a1)) * tau / 2 + v0);
                r1 = ((((j0 + j1) * tau / 12 + (a0 - a1)) * tau / 5 +
                       (v0 + v1)) * tau / 2 + r0);
            } else {
                const double j0 = A.f0[3 + d][i], j1 = A.f1[3 + d][i];
                const double s0 = A.f0[6 + d][i], s1 = A.f1[6 + d][i];
                const double c0 = A.f0[9 + d][i], c1 = A.f1[9 + d][i];
                v1 = (((((c0 - c1) * tau / 20 + (s0 + s1)) * tau / 3 +
                        3 * (j0 - j1)) * tau / 14 + (a0 + a1)) * tau / 2 +
                      v0);
                r1 = (((((s0 - s1) * tau / 20 + (j0 + j1)) * tau / 3 +
                        3 * (a0 - a1)) * tau / 14 + (v0 + v1)) * tau / 2 +
                      r0);
            }
            A.v[d][i] = v1;
            A.r[d][i] = r1;
        }
}

// Kinetic energy 0.5 sum m v^2 and potential 0.5 sum m phi, fp64; block
// partials written to part[2 * block], reduced on the host in block order.
__global__ void k_energy(const double *m, const double *const *v3,
                         const double *phi, uint64_t n, double *part)
{
    __shared__ double sk[256], sp[256];
    double ke = 0.0, pe = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        double vx = v3[0][i], vy = v3[1][i], vz = v3[2][i];
        ke += 0.5 * m[i] * (vx * vx + vy * vy + vz * vz);
        pe += m[i] * phi[i];
    }
    sk[threadIdx.x] = ke;
    sp[threadIdx.x] = pe;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sk[threadIdx.x] += sk[threadIdx.x + s];
            sp[threadIdx.x] += sp[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sk[0];
        part[2 * blockIdx.x + 1] = sp[0];
    }
}

struct Hermite {
    uint64_t n = 0;
    int order = 4;
    int adaptive = 1;
    int mode = MODE_EXACT;
    int sms = 152;
    cudaStream_t stream = nullptr;
    StepCtl *ctl = nullptr;
    unsigned *err = nullptr;
    double *pool = nullptr;
    Arrays A;
    double *tau_log = nullptr;
    long long tau_cap = 0;
    void *pack = nullptr;
    size_t pack_bytes = 0;
    double *partial = nullptr;
    size_t partial_bytes = 0;
    double *phi = nullptr;
    double *epart = nullptr;
    double **v3 = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_batch = -1;
    unsigned long long launches_per_batch = 0;
    long long kepler_budget = 1LL << 20;
    double eta = 0.0;
};

int grow(void **p, size_t *have, size_t need)
{
    if (need <= *have) return 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    if (cudaMalloc(p, need) != cudaSuccess) return 1;
    *have = need;
    return 0;
}

unsigned grid_for(uint64_t n, int sms)
{
    uint64_t b = (n + 255) / 256;
    uint64_t cap = (uint64_t)sms * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// One pairwise sweep of all particles against all (i and j are the same
// arrays), in the system's mode.  Workspace must already be sized.
cudaError_t sweep(Hermite *h, int kernel, const double *const *attrs,
                  double *const *out, double eta)
{
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = kernel;
    s.mode = h->mode;
    s.ni = s.nj = h->n;
    for (int a = 0; a < n_attr(kernel); ++a) s.ip[a] = s.jp[a] = attrs[a];
    for (int o = 0; o < n_out(kernel); ++o) s.out[o] = out[o];
    s.scal[0] = eta;
    if (h->mode == MODE_EXACT)
        return launch_exact<double>(s, h->stream, h->kepler_budget, h->err);
    cudaError_t e = launch_pack(kernel, h->n, s.ip, (float4 *)h->pack,
                                h->stream);
    if (e != cudaSuccess) return e;
    int variant, gsplit;
    choose_split_public(kernel, h->n, h->n, &variant, &gsplit);
    return launch_split(kernel, (const float4 *)h->pack,
                        (const float4 *)h->pack, h->n, h->n, s.out, h->partial,
                        variant, gsplit, eta, h->err, h->stream);
}

int size_workspace(Hermite *h)
{
    // largest packed record (snap: 5 float4) and partials for 64 splits
    if (grow(&h->pack, &h->pack_bytes, (size_t)h->n * 5 * 16 + 256)) return 1;
    if (grow((void **)&h->partial, &h->partial_bytes,
             (size_t)64 * 7 * h->n * sizeof(double)))
        return 1;
    return 0;
}

cudaError_t forces(Hermite *h, double *const *rr, double *const *vv,
                   double *const *f)
{
    const double *at[14] = {h->A.m, rr[0], rr[1], rr[2], h->A.e2,
                            vv[0], vv[1], vv[2], f[0], f[1], f[2],
                            f[3], f[4], f[5]};
    cudaError_t e;
    if (h->order == 2) return sweep(h, K_ACC, at, f, 0.0);
    e = sweep(h, K_ACC_JERK, at, f, 0.0);
    if (e != cudaSuccess || h->order < 6) return e;
    return sweep(h, K_SNAP_CRACKLE, at, f + 6, 0.0);
}

template <int ORDER>
cudaError_t step_order(Hermite *h)
{
    const unsigned g = grid_for(h->n, h->sms);
    cudaStream_t st = h->stream;
    k_begin_step<<<1, 32, 0, st>>>(h->ctl);
    if (h->adaptive) {
        const double *at[8] = {h->A.m, h->A.r[0], h->A.r[1], h->A.r[2],
                               h->A.e2, h->A.v[0], h->A.v[1], h->A.v[2]};
        cudaError_t e = sweep(h, K_TSTEP, at, h->A.dt, h->eta);
        if (e != cudaSuccess) return e;
        k_min_abs<<<g, 256, 0, st>>>(h->A.dt[0], h->n, h->ctl);
        k_block_tstep<<<1, 32, 0, st>>>(h->ctl);
    }
    k_copy_state<<<g, 256, 0, st>>>(h->A, h->n, h->ctl);
    cudaError_t e = forces(h, h->A.r0, h->A.v0, h->A.f0);
    if (e != cudaSuccess) return e;
    k_predict<ORDER><<<g, 256, 0, st>>>(h->A, h->n, h->ctl);
    for (int pass = 0; pass < 2; ++pass) {
        e = forces(h, h->A.r, h->A.v, h->A.f1);
        if (e != cudaSuccess) return e;
        k_correct<ORDER><<<g, 256, 0, st>>>(h->A, h->n, h->ctl);
    }
    k_end_step<<<1, 32, 0, st>>>(h->ctl, h->tau_log, h->tau_cap);
    g_launch_count += h->adaptive ? 8 : 6;
    return cudaGetLastError();
}

cudaError_t one_step(Hermite *h)
{
    switch (h->order) {
    case 2: return step_order<2>(h);
    case 4: return step_order<4>(h);
    case 6: return step_order<6>(h);
    default: return step_order<8>(h);
    }
}

}  // namespace

// ===========================================================================
// C-ABI of the device-resident Hermite driver (no counterpart in the
// reference, whose integrators keep particles in host numpy arrays).
// ===========================================================================

// Creates a system of n particles from HOST arrays.  order: 2, 4, 6 or 8;
// adaptive: 1 = tupan's "ahermiteN" (Tstep + power-of-two quantisation),
// 0 = "hermiteN" (step = eta); mode: 0 EXACT, 1 SPLIT forces.  tau_log_cap:
// number of step sizes to record (0: none).
TG_EXPORT int tupan_gb300_hermite_destroy(void *handle);

TG_EXPORT int tupan_gb300_hermite_create(
    uint64_t n, int order, int adaptive, int mode, double eta,
    const double *m, const double *e2, const double *rx, const double *ry,
    const double *rz, const double *vx, const double *vy, const double *vz,
    long long tau_log_cap, void **handle)
{
    if (!handle || n == 0 || (order != 2 && order != 4 && order != 6 &&
                              order != 8))
        return ST_BAD_ARGUMENT;
    Hermite *h = new Hermite();
    CreateGuard guard{h, tupan_gb300_hermite_destroy};
    h->n = n;
    h->order = order;
    h->adaptive = adaptive ? 1 : 0;
    h->mode = mode == MODE_SPLIT ? MODE_SPLIT : MODE_EXACT;
    h->eta = eta;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) !=
        cudaSuccess)
        return ST_CUDA;
    const int narr = 2 + 6 + 6 + 24 + 2 + 1;
    if (cudaMalloc((void **)&h->pool, (size_t)narr * n * sizeof(double)) !=
        cudaSuccess)
        return ST_CUDA;
    cudaMemset(h->pool, 0, (size_t)narr * n * sizeof(double));
    double *p = h->pool;
    auto take = [&]() { double *q = p; p += n; return q; };
    h->A.m = take();
    h->A.e2 = take();
    for (int d = 0; d < 3; ++d) h->A.r[d] = take();
    for (int d = 0; d < 3; ++d) h->A.v[d] = take();
    for (int d = 0; d < 3; ++d) h->A.r0[d] = take();
    for (int d = 0; d < 3; ++d) h->A.v0[d] = take();
    for (int k = 0; k < 12; ++k) h->A.f0[k] = take();
    for (int k = 0; k < 12; ++k) h->A.f1[k] = take();
    h->A.dt[0] = take();
    h->A.dt[1] = take();
    h->phi = take();
    const double *src[8] = {m, e2, rx, ry, rz, vx, vy, vz};
    double *dst[8] = {h->A.m, h->A.e2, h->A.r[0], h->A.r[1], h->A.r[2],
                      h->A.v[0], h->A.v[1], h->A.v[2]};
    for (int k = 0; k < 8; ++k)
        if (cudaMemcpy(dst[k], src[k], n * sizeof(double),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return ST_CUDA;
    if (cudaMalloc((void **)&h->ctl, sizeof(StepCtl)) != cudaSuccess)
        return ST_CUDA;
    StepCtl c;
    memset(&c, 0, sizeof(c));
    c.eta = eta;
    c.t_end = 0.0;
    cudaMemcpy(h->ctl, &c, sizeof(c), cudaMemcpyHostToDevice);
    cudaMalloc((void **)&h->err, sizeof(unsigned));
    cudaMemset(h->err, 0, sizeof(unsigned));
    if (tau_log_cap > 0) {
        cudaMalloc((void **)&h->tau_log, tau_log_cap * sizeof(double));
        h->tau_cap = tau_log_cap;
    }
    cudaMalloc((void **)&h->epart, 2 * 1024 * sizeof(double));
    cudaMalloc((void **)&h->v3, 3 * sizeof(double *));
    cudaMemcpy(h->v3, h->A.v, 3 * sizeof(double *), cudaMemcpyHostToDevice);
    if (size_workspace(h)) return ST_CUDA;
    int v, gs;
    choose_split_public(K_ACC_JERK, n, n, &v, &gs);   // initialise device state
    if (cudaDeviceSynchronize() != cudaSuccess) return ST_CUDA;
    *handle = h;
    guard.keep();
    return ST_OK;
}

// Advances until |t| >= t_end or max_steps steps were taken.  A CUDA graph
// of `batch` steps is replayed between host checks of the time (steps past
// t_end inside a batch do nothing).  Returns the time and the step count.
TG_EXPORT int tupan_gb300_hermite_evolve(void *handle, double t_end,
                                         long long max_steps, int batch,
                                         double *t_out, long long *steps_out)
{
    Hermite *h = (Hermite *)handle;
    if (!h) return ST_BAD_ARGUMENT;
    if (batch < 1) batch = 1;
    cudaMemcpy(&h->ctl->t_end, &t_end, sizeof(double), cudaMemcpyHostToDevice);
    // build (or rebuild) the graph of `batch` steps; split-sweep choices are
    // made once here (workspace is already sized, nothing allocates).
    if (h->graph && h->graph_batch != batch) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (!h->graph) {
        cudaGraph_t g;
        unsigned long long before = g_launch_count.load();
        if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            return ST_CUDA;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < batch && e == cudaSuccess; ++k) e = one_step(h);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) return ST_CUDA;
        if (cudaGraphInstantiate(&h->graph, g, 0) != cudaSuccess) return ST_CUDA;
        cudaGraphDestroy(g);
        h->graph_batch = batch;
        h->launches_per_batch = g_launch_count.load() - before;
        g_launch_count -= h->launches_per_batch;   // counted when replayed
    }
    StepCtl c;
    long long start = -1;
    double t_prev = NAN;
    for (;;) {
        cudaMemcpy(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost);
        if (start < 0) start = c.nsteps;
        if (fabs(c.t) >= t_end || (max_steps > 0 && c.nsteps - start >= max_steps))
            break;
        // a step that does not advance time (a zero or non-finite step
        // size) would loop forever: report it instead
        if (!isfinite(c.t) || c.t == t_prev) return ST_DEVICE;
        t_prev = c.t;
        long long left = max_steps > 0 ? max_steps - (c.nsteps - start) : batch;
        if (left < batch) {
            // finish with single uncaptured steps so max_steps is exact
            for (long long k = 0; k < left; ++k)
                if (one_step(h) != cudaSuccess) return ST_CUDA;
        } else {
            if (cudaGraphLaunch(h->graph, h->stream) != cudaSuccess)
                return ST_CUDA;
            g_launch_count += h->launches_per_batch;
        }
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) return ST_CUDA;
    }
    unsigned herr = 0;
    cudaMemcpy(&herr, h->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (t_out) *t_out = c.t;
    if (steps_out) *steps_out = c.nsteps;
    return herr ? ST_DEVICE : ST_OK;
}

// Copies the state back to HOST arrays.
TG_EXPORT int tupan_gb300_hermite_get_state(void *handle, double *rx,
                                            double *ry, double *rz,
                                            double *vx, double *vy,
                                            double *vz)
{
    Hermite *h = (Hermite *)handle;
    if (!h) return ST_BAD_ARGUMENT;
    double *dst[6] = {rx, ry, rz, vx, vy, vz};
    double *src[6] = {h->A.r[0], h->A.r[1], h->A.r[2],
                      h->A.v[0], h->A.v[1], h->A.v[2]};
    for (int k = 0; k < 6; ++k)
        if (cudaMemcpy(dst[k], src[k], h->n * sizeof(double),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
    return ST_OK;
}

// Recorded step sizes (up to cap); returns how many were copied.
TG_EXPORT long long tupan_gb300_hermite_tau_log(void *handle, double *out,
                                                long long cap)
{
    Hermite *h = (Hermite *)handle;
    if (!h || !h->tau_log) return 0;
    StepCtl c;
    cudaMemcpy(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost);
    long long k = c.nsteps < h->tau_cap ? c.nsteps : h->tau_cap;
    if (k > cap) k = cap;
    cudaMemcpy(out, h->tau_log, k * sizeof(double), cudaMemcpyDeviceToHost);
    return k;
}

// Total kinetic and potential energy (body.py:260-321).  The diagnostic is
// FP64 whatever the integration mode: the potential comes from an EXACT Phi
// sweep and the sums are fp64 on the device.
TG_EXPORT int tupan_gb300_hermite_energy(void *handle, double *ke, double *pe)
{
    Hermite *h = (Hermite *)handle;
    if (!h) return ST_BAD_ARGUMENT;
    const double *at[5] = {h->A.m, h->A.r[0], h->A.r[1], h->A.r[2], h->A.e2};
    double *out[1] = {h->phi};
    const int mode = h->mode;
    h->mode = MODE_EXACT;
    cudaError_t se = sweep(h, K_PHI, at, out, 0.0);
    h->mode = mode;
    if (se != cudaSuccess) return ST_CUDA;
    const int blocks = 1024;
    k_energy<<<blocks, 256, 0, h->stream>>>(h->A.m, h->v3, h->phi, h->n,
                                            h->epart);
    g_launch_count += 1;
    std::vector<double> part(2 * blocks);
    if (cudaMemcpyAsync(part.data(), h->epart, part.size() * sizeof(double),
                        cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
        return ST_CUDA;
    double k = 0.0, p = 0.0;
    for (int b = 0; b < blocks; ++b) {
        k += part[2 * b];
        p += part[2 * b + 1];
    }
    *ke = k;
    *pe = 0.5 * p;
    return ST_OK;
}

TG_EXPORT int tupan_gb300_hermite_destroy(void *handle)
{
    Hermite *h = (Hermite *)handle;
    if (!h) return ST_BAD_ARGUMENT;
    cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    cudaFree(h->pool);
    cudaFree(h->ctl);
    cudaFree(h->err);
    if (h->tau_log) cudaFree(h->tau_log);
    cudaFree(h->pack);
    cudaFree(h->partial);
    cudaFree(h->epart);
    cudaFree(h->v3);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return ST_OK;
}
