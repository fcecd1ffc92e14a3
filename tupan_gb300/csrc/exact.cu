// EXACT-mode sweeps: one i-particle per thread, j-particles streamed through
// shared memory in tiles and summed in source order.  With the pair
// arithmetic of tg_pairs.cuh and this file compiled with -fmad=false, every
// output is bit-identical to the reference C kernel (tupan/lib/src/*.c) on
// the same inputs, for REAL = double and REAL = float.
//
// Sakura and Kepler share the pair/solver code of tg_kepler.cuh; their
// leapfrog branch is bit-identical, their Kepler branch agrees to the
// accuracy of CUDA's transcendental functions.

#include "tg_common.cuh"
#include "tg_kepler.cuh"
#include "tg_pairs.cuh"
#include "tg_pn.cuh"

namespace tg {

constexpr int EXACT_THREADS = 128;
constexpr int EXACT_TILE = 128;

template <class Op, typename R>
__global__ void __launch_bounds__(EXACT_THREADS)
exact_sweep(const Sweep s)
{
    constexpr int NA = Op::NA;
    __shared__ R tile[NA][EXACT_TILE];
    const uint64_t ni = s.ni_dev ? (uint64_t)*s.ni_dev : s.ni, nj = s.nj;
    // blocks past a device-side count have no i (the whole block leaves)
    if ((uint64_t)blockIdx.x * EXACT_THREADS >= ni) return;
    const uint64_t i = (uint64_t)blockIdx.x * EXACT_THREADS + threadIdx.x;
    const uint64_t ic = i < ni ? i : ni - 1;
    R ip[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) ip[a] = ((const R *)s.ip[a])[ic];
    R o[Op::NO];
    Op::init(o);
    for (uint64_t j0 = 0; j0 < nj; j0 += EXACT_TILE) {
        const int n = (int)((nj - j0) < EXACT_TILE ? (nj - j0) : EXACT_TILE);
        __syncthreads();
        for (int t = threadIdx.x; t < NA * EXACT_TILE; t += EXACT_THREADS) {
            const int a = t / EXACT_TILE, jj = t % EXACT_TILE;
            if (jj < n) tile[a][jj] = ((const R *)s.jp[a])[j0 + jj];
        }
        __syncthreads();
        for (int jj = 0; jj < n; ++jj) {
            R jp[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a) jp[a] = tile[a][jj];
            Op::pair(ip, jp, o, s);
        }
    }
    if (i < ni) {
        Op::finish(ip, o, s);
#pragma unroll
        for (int c = 0; c < Op::NO; ++c) ((R *)s.out[c])[i] = o[c];
    }
}

// sakura_kernel.c:33-62: Sigma_j (m_j/M)(two-body step - initial state).
template <typename R>
__global__ void __launch_bounds__(EXACT_THREADS)
exact_sakura(const Sweep s, long long budget, unsigned *err)
{
    constexpr int NA = 8;
    __shared__ R tile[NA][EXACT_TILE];
    const uint64_t ni = s.ni, nj = s.nj;
    const uint64_t i = (uint64_t)blockIdx.x * EXACT_THREADS + threadIdx.x;
    const uint64_t ic = i < ni ? i : ni - 1;
    const R dt = R(s.scal[0]);
    const long long flag = s.iscal;
    R ip[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) ip[a] = ((const R *)s.ip[a])[ic];
    R o[6] = {0, 0, 0, 0, 0, 0};
    bool exhausted = false;
    for (uint64_t j0 = 0; j0 < nj; j0 += EXACT_TILE) {
        const int n = (int)((nj - j0) < EXACT_TILE ? (nj - j0) : EXACT_TILE);
        __syncthreads();
        for (int t = threadIdx.x; t < NA * EXACT_TILE; t += EXACT_THREADS) {
            const int a = t / EXACT_TILE, jj = t % EXACT_TILE;
            if (jj < n) tile[a][jj] = ((const R *)s.jp[a])[j0 + jj];
        }
        __syncthreads();
        for (int jj = 0; jj < n; ++jj) {
            R jp[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a) jp[a] = tile[a][jj];
            R p0[6], p1[6], m, e2;
            pair_state(ip, jp, p0, &m, &e2);
            KepCtx<R> c = {0, budget, 0, false, false, R(0)};
            evolve_pair(dt, flag, m, e2, p0, p1, c);
            exhausted |= c.exhausted;
            R mu = jp[0] / m;
#pragma unroll
            for (int q = 0; q < 6; ++q) o[q] += mu * (p1[q] - p0[q]);
        }
    }
    if (i < ni) {
#pragma unroll
        for (int q = 0; q < 6; ++q) ((R *)s.out[q])[i] = o[q];
        if (exhausted) atomicOr(err, (unsigned)DERR_KEPLER_BUDGET);
    }
}

// kepler_solver_kernel.c:5-49 with kepler_solver_kernel_common.h:8-80: two
// particles evolved in their centre-of-mass frame; outputs may alias inputs.
template <typename R>
__global__ void exact_kepler(const Sweep s, long long budget, unsigned *err)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    R a[8], b[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        a[k] = ((const R *)s.ip[k])[0];
        b[k] = ((const R *)s.ip[k])[1];
    }
    const R dt = R(s.scal[0]);
    KepCtx<R> ctx = {0, budget, 0, false, false, R(0)};
    R a1[6], b1[6];
    kepler_two_body(a, b, dt, a1, b1, ctx);
    for (int q = 0; q < 6; ++q) {
        ((R *)s.out[q])[0] = a1[q];
        ((R *)s.out[q])[1] = b1[q];
    }
    if (ctx.exhausted) atomicOr(err, (unsigned)DERR_KEPLER_BUDGET);
}

template <class Op, typename R>
static cudaError_t run_exact(const Sweep &s, cudaStream_t st)
{
    const unsigned blocks = (unsigned)((s.ni + EXACT_THREADS - 1) / EXACT_THREADS);
    exact_sweep<Op, R><<<blocks, EXACT_THREADS, 0, st>>>(s);
    g_launch_count += 1;
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_exact(const Sweep &s, cudaStream_t st, long long budget,
                         unsigned *err)
{
    if (s.kernel == K_KEPLER) {
        exact_kepler<R><<<1, 32, 0, st>>>(s, budget, err);
        g_launch_count += 1;
        return cudaGetLastError();
    }
    if (s.ni == 0) return cudaSuccess;
    switch (s.kernel) {
    case K_PHI: return run_exact<PhiPair<R>, R>(s, st);
    case K_ACC: return run_exact<AccPair<R>, R>(s, st);
    case K_ACC_JERK: return run_exact<AccJerkPair<R>, R>(s, st);
    case K_SNAP_CRACKLE: return run_exact<SnapCracklePair<R>, R>(s, st);
    case K_TSTEP: return run_exact<TstepPair<R>, R>(s, st);
    case K_PNACC: return run_exact<PnAccPair<R>, R>(s, st);
    case K_NREG_X: return run_exact<NregXPair<R>, R>(s, st);
    case K_NREG_V: return run_exact<NregVPair<R>, R>(s, st);
    case K_SAKURA: {
        const unsigned blocks =
            (unsigned)((s.ni + EXACT_THREADS - 1) / EXACT_THREADS);
        exact_sakura<R><<<blocks, EXACT_THREADS, 0, st>>>(s, budget, err);
        g_launch_count += 1;
        return cudaGetLastError();
    }
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_exact<double>(const Sweep &, cudaStream_t,
                                          long long, unsigned *);
template cudaError_t launch_exact<float>(const Sweep &, cudaStream_t,
                                         long long, unsigned *);

}  // namespace tg
