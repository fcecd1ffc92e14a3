// Ensemble driver: many independent N-body systems of mixed size advanced
// together on one GPU, each with its own shared adaptive Hermite-4 step
// (tupan's "ahermite4": hermite.py:390-410 with the quantisation of
// integrator/__init__.py:59-78), each system's step held in device memory.
//
// Every force evaluation of the whole ensemble is ONE launch of the batched
// SPLIT sweep (split_sweep_batched: a persistent kernel whose CTAs take
// systems from an atomic work queue, largest first); the per-particle
// predictor/corrector and the per-system step control are elementwise
// kernels.  A step is a fixed launch sequence, so `batch` steps are captured
// in a CUDA graph and replayed; systems that reached t_end are skipped.
// Energies are fp64: an in-order fp64 Phi per system (same arithmetic and j
// order as phi_kernel.c) and fp64 sums in fixed order.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "tg_common.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace tg {
cudaError_t launch_pack(int kernel, uint64_t n, const void *const *attrs,
                        float4 *out, cudaStream_t st);
cudaError_t launch_split_batched(int kernel, const float4 *rec,
                                 const uint64_t *off, const unsigned *order,
                                 const int *active, unsigned n_sys,
                                 unsigned *queue, void *const *out, double eta,
                                 unsigned *err, int sms, cudaStream_t st);
}  // namespace tg

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
    long long power = (long long)(log2(min_ts) - 1.0);
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

__global__ void k_e_begin(SysCtl *c, int *active, unsigned ns, double t_end,
                          double eta)
{
    GRID_LOOP(s, ns)
    {
        if (fabs(c[s].t) >= t_end) {
            active[s] = 0;
            c[s].tau = 0.0;
            continue;
        }
        active[s] = 1;
        c[s].tau = e_base_tstep(c[s].t, t_end, eta);
        c[s].min_bits = 0x7ff0000000000000ull;
    }
}

__global__ void k_e_min(EArrays A, uint64_t n, SysCtl *c, const int *active)
{
    GRID_LOOP(i, n)
    {
        const unsigned s = A.sys[i];
        if (!active[s]) continue;
        atomicMin(&c[s].min_bits,
                  (unsigned long long)__double_as_longlong(fabs(A.dt[0][i])));
    }
}

__global__ void k_e_block(SysCtl *c, const int *active, unsigned ns)
{
    GRID_LOOP(s, ns)
    {
        if (!active[s]) continue;
        const double m = __longlong_as_double((long long)c[s].min_bits);
        c[s].tau = e_block_tstep(m, c[s].t, c[s].tau);
    }
}

__global__ void k_e_copy(EArrays A, uint64_t n, const int *active)
{
    GRID_LOOP(i, n)
    {
        if (!active[A.sys[i]]) continue;
        for (int d = 0; d < 3; ++d) {
            A.r0[d][i] = A.r[d][i];
            A.v0[d][i] = A.v[d][i];
        }
    }
}

// H4.epredict (hermite.py:83-88)
__global__ void k_e_predict(EArrays A, uint64_t n, const SysCtl *c,
                            const int *active)
{
    GRID_LOOP(i, n)
    {
        const unsigned s = A.sys[i];
        if (!active[s]) continue;
        const double tau = c[s].tau;
        for (int d = 0; d < 3; ++d) {
            const double a = A.f0[d][i], j = A.f0[3 + d][i], v = A.v[d][i];
            A.r[d][i] = A.r[d][i] + ((j * tau / 3 + a) * tau / 2 + v) * tau;
            A.v[d][i] = v + (j * tau / 2 + a) * tau;
        }
    }
}

// H4.ecorrect (hermite.py:96-119)
__global__ void k_e_correct(EArrays A, uint64_t n, const SysCtl *c,
                            const int *active)
{
    GRID_LOOP(i, n)
    {
        const unsigned s = A.sys[i];
        if (!active[s]) continue;
        const double tau = c[s].tau;
        for (int d = 0; d < 3; ++d) {
            const double a0 = A.f0[d][i], a1 = A.f1[d][i];
            const double j0 = A.f0[3 + d][i], j1 = A.f1[3 + d][i];
            const double v0 = A.v0[d][i], r0 = A.r0[d][i];
            const double v1 = (((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + v0);
            A.v[d][i] = v1;
            A.r[d][i] = (((a0 - a1) * tau / 6 + (v0 + v1)) * tau / 2 + r0);
        }
    }
}

__global__ void k_e_end(SysCtl *c, const int *active, unsigned ns)
{
    GRID_LOOP(s, ns)
    {
        if (!active[s]) continue;
        c[s].t += c[s].tau;
        c[s].nsteps += 1;
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
    SysCtl *ctl = nullptr;
    unsigned *queue = nullptr;
    unsigned *err = nullptr;
    float4 *pack = nullptr;
    double *ke = nullptr, *pe = nullptr;
    double t_end = 0.0;
    cudaGraphExec_t graph = nullptr;
    int graph_batch = -1;
    unsigned long long launches_per_batch = 0;
};

unsigned grid_for(uint64_t n, int sms)
{
    uint64_t b = (n + 255) / 256;
    uint64_t cap = (uint64_t)sms * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

cudaError_t e_forces(Ensemble *E, double *const *rr, double *const *vv,
                     double *const *out, int kernel, double eta)
{
    const void *at[8] = {E->A.m, rr[0], rr[1], rr[2], E->A.e2, vv[0], vv[1],
                         vv[2]};
    cudaError_t e = launch_pack(kernel, E->n, at, E->pack, E->stream);
    if (e != cudaSuccess) return e;
    return launch_split_batched(kernel, E->pack, E->off, E->order, E->active,
                                E->ns, E->queue, (void *const *)out, eta,
                                E->err, E->sms, E->stream);
}

cudaError_t e_step(Ensemble *E)
{
    cudaStream_t st = E->stream;
    const unsigned gp = grid_for(E->n, E->sms), gs = grid_for(E->ns, E->sms);
    k_e_begin<<<gs, 256, 0, st>>>(E->ctl, E->active, E->ns, E->t_end, E->eta);
    cudaError_t e = e_forces(E, E->A.r, E->A.v, E->A.dt, K_TSTEP, E->eta);
    if (e != cudaSuccess) return e;
    k_e_min<<<gp, 256, 0, st>>>(E->A, E->n, E->ctl, E->active);
    k_e_block<<<gs, 256, 0, st>>>(E->ctl, E->active, E->ns);
    k_e_copy<<<gp, 256, 0, st>>>(E->A, E->n, E->active);
    e = e_forces(E, E->A.r0, E->A.v0, E->A.f0, K_ACC_JERK, 0.0);
    if (e != cudaSuccess) return e;
    k_e_predict<<<gp, 256, 0, st>>>(E->A, E->n, E->ctl, E->active);
    for (int pass = 0; pass < 2; ++pass) {
        e = e_forces(E, E->A.r, E->A.v, E->A.f1, K_ACC_JERK, 0.0);
        if (e != cudaSuccess) return e;
        k_e_correct<<<gp, 256, 0, st>>>(E->A, E->n, E->ctl, E->active);
    }
    k_e_end<<<gs, 256, 0, st>>>(E->ctl, E->active, E->ns);
    g_launch_count += 8;
    return cudaGetLastError();
}

}  // namespace

// ===========================================================================
// C-ABI (no counterpart in the reference, which integrates one system).
// ===========================================================================

// n_sys systems; sys_off[n_sys + 1] host offsets into the concatenated HOST
// arrays m, e2, r, v (sizes 1 .. 512 each).  Forces are SPLIT-mode.
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
    E->n = n;
    E->ns = n_sys;
    E->eta = eta;
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
        cudaMalloc((void **)&E->queue, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->err, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&E->pack, n * 3 * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void **)&E->ke, n_sys * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&E->pe, n_sys * sizeof(double)) != cudaSuccess)
        return ST_CUDA;
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
    return ST_OK;
}

// Steps every system until it reaches t_end (a graph of `batch` steps per
// host check).  Returns the largest step count over the systems.
TG_EXPORT int tupan_gb300_ensemble_evolve(void *handle, double t_end, int batch,
                                          long long *max_steps_out)
{
    Ensemble *E = (Ensemble *)handle;
    if (!E) return ST_BAD_ARGUMENT;
    if (batch < 1) batch = 1;
    E->t_end = t_end;
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
    for (;;) {
        if (cudaMemcpy(c.data(), E->ctl, E->ns * sizeof(SysCtl),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
        bool all = true;
        for (unsigned s = 0; s < E->ns && all; ++s)
            if (fabs(c[s].t) < t_end) all = false;
        if (all) break;
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
    cudaFree(E->active);
    cudaFree(E->ctl);
    cudaFree(E->queue);
    cudaFree(E->err);
    cudaFree(E->pack);
    cudaFree(E->ke);
    cudaFree(E->pe);
    cudaStreamDestroy(E->stream);
    delete E;
    return ST_OK;
}
