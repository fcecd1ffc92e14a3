// Device-resident NREG driver: tupan's regularised-time integrators "nreg"
// and "anreg" (tupan/integrator/nreg.py) with the particles in HBM.
//
// A position half-update is one EXACT nreg_X sweep (m r, a and the pair
// potential u of every particle), r = (m r) / M and U = sum(u) / 2; a
// velocity update is one EXACT nreg_V sweep, v = (m v) / M, K = sum(m k) / 4M
// and W = K - E0.  The scalar recurrences between the updates (the step
// sizes h/W and h/U, S of nreg_step, the time) are the reference's and run
// on the host in double, as in the reference.  The sums are taken in numpy's
// order (pairwise: 8 running sums over blocks of at most 128 elements,
// halves above that), so with the EXACT sweeps, -fmad=false elementwise
// kernels and the same host arithmetic a run is bit-identical to the
// reference's NREG integrator on its C backend.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cfloat>
#include <vector>

#include "tg_common.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace tg {
template <typename R>
cudaError_t launch_exact(const Sweep &s, cudaStream_t st, long long budget,
                         unsigned *err);
}  // namespace tg

using namespace tg;

namespace {

enum Field {
    F_M = 0, F_RX, F_RY, F_RZ, F_E2, F_VX, F_VY, F_VZ,
    F_AX, F_AY, F_AZ, F_MRX, F_MRY, F_MRZ, F_U, F_MVX, F_MVY, F_MVZ, F_MK,
    F_PHI, F_TMP,
    NFIELD
};

struct Fields {
    double *f[NFIELD];
};

// numpy's pairwise summation of x[lo, lo + n) (the order of the reference's
// float64 .sum() calls).  Leaves of at most 128 elements are summed with
// eight running sums; the tree above them adds the two halves, the first
// rounded down to a multiple of 8.
__device__ double pw_leaf(const double *x, uint64_t lo, uint64_t n)
{
    if (n < 8) {
        double res = 0.0;
        for (uint64_t i = 0; i < n; ++i) res += x[lo + i];
        return res;
    }
    double r[8];
    for (int j = 0; j < 8; ++j) r[j] = x[lo + j];
    uint64_t i = 8;
    for (; i < n - (n % 8); i += 8)
        for (int j = 0; j < 8; ++j) r[j] += x[lo + i + j];
    double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; ++i) res += x[lo + i];
    return res;
}

constexpr int PW_NT = 256;
constexpr int PW_STACK = 64;

// One CTA: thread 0 walks the tree to list the leaves, all threads sum the
// leaves, thread 0 walks the tree again combining the leaf sums in order.
// leaf_lo/leaf_n/leaf_sum: scratch of at least n / 56 + 2 entries.
__global__ void __launch_bounds__(PW_NT)
k_pairwise_sum(const double *x, uint64_t n, uint64_t *leaf_lo,
               uint64_t *leaf_n, double *leaf_sum, double *out)
{
    __shared__ unsigned n_leaves;
    if (threadIdx.x == 0) {
        unsigned nl = 0;
        uint64_t st_lo[PW_STACK], st_n[PW_STACK];
        int sp = 0;
        st_lo[sp] = 0;
        st_n[sp] = n;
        ++sp;
        while (sp > 0) {
            --sp;
            const uint64_t lo = st_lo[sp], m = st_n[sp];
            if (m <= 128) {
                leaf_lo[nl] = lo;
                leaf_n[nl] = m;
                ++nl;
                continue;
            }
            uint64_t m2 = m / 2;
            m2 -= m2 % 8;
            // second half pushed first so the first half is listed first
            st_lo[sp] = lo + m2;
            st_n[sp] = m - m2;
            ++sp;
            st_lo[sp] = lo;
            st_n[sp] = m2;
            ++sp;
        }
        n_leaves = nl;
    }
    __syncthreads();
    for (unsigned k = threadIdx.x; k < n_leaves; k += PW_NT)
        leaf_sum[k] = pw_leaf(x, leaf_lo[k], leaf_n[k]);
    __syncthreads();
    if (threadIdx.x == 0) {
        // post-order combination: each node is its halves' sum
        uint64_t st_n[PW_STACK];
        int st_state[PW_STACK];
        double st_val[PW_STACK];
        int sp = 0;
        unsigned next_leaf = 0;
        double result = 0.0;
        st_n[sp] = n;
        st_state[sp] = 0;
        ++sp;
        while (sp > 0) {
            const int top = sp - 1;
            const uint64_t m = st_n[top];
            if (m <= 128) {
                const double v = leaf_sum[next_leaf++];
                --sp;
                if (sp == 0) {
                    result = v;
                } else if (st_state[sp - 1] == 1) {
                    st_val[sp - 1] = v;        // first half done
                } else {
                    st_val[sp - 1] = st_val[sp - 1] + v;   // second half
                    st_state[sp - 1] = 3;
                }
                continue;
            }
            uint64_t m2 = m / 2;
            m2 -= m2 % 8;
            if (st_state[top] == 0) {
                st_state[top] = 1;
                st_n[sp] = m2;
                st_state[sp] = 0;
                ++sp;
            } else if (st_state[top] == 1) {
                st_state[top] = 2;
                st_n[sp] = m - m2;
                st_state[sp] = 0;
                ++sp;
            } else {
                const double v = st_val[top];
                --sp;
                if (sp == 0) {
                    result = v;
                } else if (st_state[sp - 1] == 1) {
                    st_val[sp - 1] = v;
                } else {
                    st_val[sp - 1] = st_val[sp - 1] + v;
                    st_state[sp - 1] = 3;
                }
            }
        }
        *out = result;
    }
}

// x = num / mtot for three arrays.
__global__ void k_divide3(double *const *dst, const double *const *num,
                          uint64_t n, double mtot)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) dst[c][i] = num[c][i] / mtot;
}

// body.py:260-303 per particle: ke = 0.5 m (vx^2 + vy^2 + vz^2) into tmp,
// pe = m phi into phi.
__global__ void k_energy_terms(Fields F, uint64_t n)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const double vx = F.f[F_VX][i], vy = F.f[F_VY][i], vz = F.f[F_VZ][i];
        F.f[F_TMP][i] = 0.5 * F.f[F_M][i] * (vx * vx + vy * vy + vz * vz);
        F.f[F_PHI][i] = F.f[F_M][i] * F.f[F_PHI][i];
    }
}

struct Nreg {
    uint64_t n = 0;
    bool anreg = false;
    double eta = 0.0;
    double t = 0.0, W = 0.0, U = 0.0, S = 0.0, E0 = 0.0, mtot = 0.0;
    long long steps = 0;
    cudaStream_t stream = nullptr;
    double *pool = nullptr;
    Fields F;
    double **ptrs = nullptr;           // device: r, mr, v, mv (3 each)
    uint64_t *leaf_lo = nullptr, *leaf_n = nullptr;
    double *leaf_sum = nullptr, *sum = nullptr, *sum_host = nullptr;
    unsigned *err = nullptr;
    int sms = 152;
};

unsigned grid_for(const Nreg *N)
{
    uint64_t b = (N->n + 255) / 256;
    const uint64_t cap = (uint64_t)N->sms * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

int device_sum(Nreg *N, int field, double *out)
{
    k_pairwise_sum<<<1, PW_NT, 0, N->stream>>>(N->F.f[field], N->n, N->leaf_lo,
                                               N->leaf_n, N->leaf_sum, N->sum);
    g_launch_count += 1;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(N->sum_host, N->sum, sizeof(double),
                        cudaMemcpyDeviceToHost, N->stream) != cudaSuccess ||
        cudaStreamSynchronize(N->stream) != cudaSuccess)
        return ST_CUDA;
    *out = *N->sum_host;
    return ST_OK;
}

int sweep(Nreg *N, int kernel, double dt, const int *in, const int *outs)
{
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = kernel;
    s.mode = MODE_EXACT;
    s.ni = s.nj = N->n;
    for (int a = 0; a < n_attr(kernel); ++a)
        s.ip[a] = s.jp[a] = N->F.f[in[a]];
    for (int o = 0; o < n_out(kernel); ++o) s.out[o] = N->F.f[outs[o]];
    s.scal[0] = dt;
    return launch_exact<double>(s, N->stream, 0, N->err) == cudaSuccess
               ? ST_OK : ST_CUDA;
}

// nreg.py:22-34
int nreg_x(Nreg *N, double dt)
{
    const int in[8] = {F_M, F_RX, F_RY, F_RZ, F_E2, F_VX, F_VY, F_VZ};
    const int outs[7] = {F_MRX, F_MRY, F_MRZ, F_AX, F_AY, F_AZ, F_U};
    int rc = sweep(N, K_NREG_X, dt, in, outs);
    if (rc) return rc;
    k_divide3<<<grid_for(N), 256, 0, N->stream>>>(N->ptrs, N->ptrs + 3, N->n,
                                                  N->mtot);
    g_launch_count += 1;
    double su;
    rc = device_sum(N, F_U, &su);
    if (rc) return rc;
    N->U = 0.5 * su;
    N->t += dt;
    return ST_OK;
}

// nreg.py:46-57
int nreg_v(Nreg *N, double dt)
{
    const int in[7] = {F_M, F_VX, F_VY, F_VZ, F_AX, F_AY, F_AZ};
    const int outs[4] = {F_MVX, F_MVY, F_MVZ, F_MK};
    int rc = sweep(N, K_NREG_V, dt, in, outs);
    if (rc) return rc;
    k_divide3<<<grid_for(N), 256, 0, N->stream>>>(N->ptrs + 6, N->ptrs + 9,
                                                  N->n, N->mtot);
    g_launch_count += 1;
    double sk;
    rc = device_sum(N, F_MK, &sk);
    if (rc) return rc;
    const double K = 0.25 * sk / N->mtot;
    N->W = (K - N->E0);
    return ST_OK;
}

// nreg.py:77-86
int anreg_step(Nreg *N, double h)
{
    int rc = nreg_x(N, 0.5 * (h / N->W));
    if (!rc) rc = nreg_v(N, (h / N->U));
    if (!rc) rc = nreg_x(N, 0.5 * (h / N->W));
    return rc;
}

// nreg.py:89-98
int nreg_step(Nreg *N, double h)
{
    int rc = anreg_step(N, 0.5 * (h * N->S));
    if (rc) return rc;
    N->S = 1 / (2 / N->W - 1 / N->S);
    return anreg_step(N, 0.5 * (h * N->S));
}

double base_tstep(double t, double t_end, double eta)
{
    // tupan/integrator/__init__.py:48-57
    double dt = fmin(fabs(t_end) - fabs(t), fabs(eta));
    dt = fmax(dt, fabs(t_end) * (2 * DBL_EPSILON));
    return copysign(dt, eta);
}

void release(Nreg *N)
{
    if (N->stream) cudaStreamSynchronize(N->stream);
    cudaFree(N->pool);
    cudaFree(N->ptrs);
    cudaFree(N->leaf_lo);
    cudaFree(N->leaf_n);
    cudaFree(N->leaf_sum);
    cudaFree(N->sum);
    cudaFree(N->err);
    cudaFreeHost(N->sum_host);
    if (N->stream) cudaStreamDestroy(N->stream);
    delete N;
}

}  // namespace

// ===========================================================================
// C-ABI (no counterpart in the reference, whose NREG runs on host arrays).
// ===========================================================================

// anreg 0: "nreg", 1: "anreg".  Host arrays are copied in; the energies
// (E0 = K + U with U = sum(m phi) / 2 from an EXACT Phi sweep), W = U = S =
// -potential and the total mass are formed as NREG.initialize does.
TG_EXPORT int tupan_gb300_nreg_create(uint64_t n, int anreg, double eta,
                                      const double *m, const double *e2,
                                      const double *rx, const double *ry,
                                      const double *rz, const double *vx,
                                      const double *vy, const double *vz,
                                      void **handle)
{
    if (!handle || n == 0) return ST_BAD_ARGUMENT;
    Nreg *N = new Nreg();
    N->n = n;
    N->anreg = anreg != 0;
    N->eta = eta;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&N->sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t fb = n * sizeof(double);
    const size_t nleaf = n / 56 + 2;
    bool ok =
        cudaStreamCreateWithFlags(&N->stream, cudaStreamNonBlocking) == cudaSuccess &&
        cudaMalloc((void **)&N->pool, NFIELD * fb) == cudaSuccess &&
        cudaMalloc((void **)&N->ptrs, 12 * sizeof(double *)) == cudaSuccess &&
        cudaMalloc((void **)&N->leaf_lo, nleaf * sizeof(uint64_t)) == cudaSuccess &&
        cudaMalloc((void **)&N->leaf_n, nleaf * sizeof(uint64_t)) == cudaSuccess &&
        cudaMalloc((void **)&N->leaf_sum, nleaf * sizeof(double)) == cudaSuccess &&
        cudaMalloc((void **)&N->sum, sizeof(double)) == cudaSuccess &&
        cudaMalloc((void **)&N->err, sizeof(unsigned)) == cudaSuccess &&
        cudaMallocHost((void **)&N->sum_host, sizeof(double)) == cudaSuccess;
    if (!ok) {
        release(N);
        return ST_CUDA;
    }
    for (int f = 0; f < NFIELD; ++f) N->F.f[f] = N->pool + (size_t)f * n;
    cudaMemsetAsync(N->pool, 0, NFIELD * fb, N->stream);
    cudaMemsetAsync(N->err, 0, sizeof(unsigned), N->stream);
    double *ptrs[12] = {N->F.f[F_RX],  N->F.f[F_RY],  N->F.f[F_RZ],
                        N->F.f[F_MRX], N->F.f[F_MRY], N->F.f[F_MRZ],
                        N->F.f[F_VX],  N->F.f[F_VY],  N->F.f[F_VZ],
                        N->F.f[F_MVX], N->F.f[F_MVY], N->F.f[F_MVZ]};
    const double *src[8] = {m, rx, ry, rz, e2, vx, vy, vz};
    ok = cudaMemcpyAsync(N->ptrs, ptrs, sizeof(ptrs), cudaMemcpyHostToDevice,
                         N->stream) == cudaSuccess;
    for (int f = 0; f < 8 && ok; ++f)
        ok = cudaMemcpyAsync(N->F.f[f], src[f], fb, cudaMemcpyHostToDevice,
                             N->stream) == cudaSuccess;
    if (!ok) {
        release(N);
        return ST_CUDA;
    }
    // NREG.initialize (nreg.py:111-122)
    int rc = device_sum(N, F_M, &N->mtot);
    const int in5[5] = {F_M, F_RX, F_RY, F_RZ, F_E2};
    const int out1[1] = {F_PHI};
    if (!rc) rc = sweep(N, K_PHI, 0.0, in5, out1);
    if (!rc) {
        k_energy_terms<<<grid_for(N), 256, 0, N->stream>>>(N->F, N->n);
        g_launch_count += 1;
    }
    double ke = 0.0, pe = 0.0;
    if (!rc) rc = device_sum(N, F_TMP, &ke);
    if (!rc) rc = device_sum(N, F_PHI, &pe);
    if (rc) {
        release(N);
        return rc;
    }
    pe = 0.5 * pe;
    N->E0 = ke + pe;
    N->W = -pe;
    N->U = -pe;
    N->S = -pe;
    *handle = N;
    return ST_OK;
}

// Steps (NREG.do_step) until |t| >= t_end or max_steps (0: no limit) steps;
// t_log (host, may be NULL) receives the time after each step (at most
// log_cap).
TG_EXPORT int tupan_gb300_nreg_evolve(void *handle, double t_end,
                                      long long max_steps, double *t_out,
                                      long long *steps_out, double *t_log,
                                      long long log_cap)
{
    Nreg *N = (Nreg *)handle;
    if (!N) return ST_BAD_ARGUMENT;
    long long taken = 0;
    while (fabs(N->t) < t_end && (max_steps <= 0 || taken < max_steps)) {
        const double tau = base_tstep(N->t, t_end, N->eta);
        const int rc = N->anreg ? anreg_step(N, tau / 2) : nreg_step(N, tau);
        if (rc) return rc;
        if (t_log && taken < log_cap) t_log[taken] = N->t;
        ++taken;
        ++N->steps;
    }
    if (t_out) *t_out = N->t;
    if (steps_out) *steps_out = taken;
    return ST_OK;
}

// Positions and velocities (host arrays of n, any may be NULL) and the
// scalars {W, U, S, E0, t} (host, 5, may be NULL).
TG_EXPORT int tupan_gb300_nreg_get_state(void *handle, double *rx, double *ry,
                                         double *rz, double *vx, double *vy,
                                         double *vz, double *scalars)
{
    Nreg *N = (Nreg *)handle;
    if (!N) return ST_BAD_ARGUMENT;
    double *dst[6] = {rx, ry, rz, vx, vy, vz};
    const int src[6] = {F_RX, F_RY, F_RZ, F_VX, F_VY, F_VZ};
    for (int q = 0; q < 6; ++q)
        if (dst[q] && cudaMemcpyAsync(dst[q], N->F.f[src[q]],
                                      N->n * sizeof(double),
                                      cudaMemcpyDeviceToHost,
                                      N->stream) != cudaSuccess)
            return ST_CUDA;
    if (cudaStreamSynchronize(N->stream) != cudaSuccess) return ST_CUDA;
    if (scalars) {
        scalars[0] = N->W;
        scalars[1] = N->U;
        scalars[2] = N->S;
        scalars[3] = N->E0;
        scalars[4] = N->t;
    }
    return ST_OK;
}

TG_EXPORT int tupan_gb300_nreg_destroy(void *handle)
{
    Nreg *N = (Nreg *)handle;
    if (!N) return ST_BAD_ARGUMENT;
    release(N);
    return ST_OK;
}
