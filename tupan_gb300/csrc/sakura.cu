// Sakura sweep with the Kepler-branch pairs solved as a separate queue, and
// a standalone universal-Kepler pair solver with an optional learned start.
//
// tupan's sakura_kernel (sakura_kernel.c:33-62) evolves every (i, j) pair as
// a two-body problem over dt: about 99 % of pairs take the leapfrog branch
// (r^2 > (64 m / v^2)^2, sakura_kernel_common.h:111-117), the rest the
// iterative universal-variable solver.  Run inline, one Kepler pair stalls
// its whole warp.  Here, for the flags the Sakura integrator uses (-1, +1):
//   1. count, per i, the pairs that take the Kepler branch (cheap test);
//   2. exclusive scan of the counts;
//   3. sum the leapfrog pairs in j order and write the Kepler pairs' j
//      indices, in j order, into each i's segment of a queue;
//   4. solve the queue, one thread per pair (coherent work);
//   5. add each i's Kepler contributions, in j order, to its leapfrog sum.
// The leapfrog branch is bit-identical to the reference (compiled without
// contraction); the result differs from the reference's interleaved sum only
// by the order of the additions, and the Kepler branch by CUDA's
// transcendental functions.
//
// The pair solver is also the engine of the learned start: an MLP
// (4 -> 64 -> 64 -> 1, SiLU, bf16 weights, FP32 accumulation) predicts the
// ratio of the converged universal anomaly to the plain first guess; the
// plain Laguerre iteration then runs to the unchanged tolerance.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "tg_common.cuh"
#include "tg_kepler.cuh"
#include "tg_split_ops.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace tg {

cudaError_t launch_pack(int kernel, uint64_t n, const void *const *attrs,
                        float4 *out, cudaStream_t st);

// ---------------------------------------------------------------------------
// Learned start: parameters in device memory.
// ---------------------------------------------------------------------------
constexpr int MLP_IN = 4, MLP_H = 64;

struct MlpParams {
    const __nv_bfloat16 *w1;   // MLP_H x MLP_IN
    const float *b1;           // MLP_H
    const __nv_bfloat16 *w2;   // MLP_H x MLP_H
    const float *b2;           // MLP_H
    const __nv_bfloat16 *w3;   // MLP_H
    const float *b3;           // 1
    const float *norm;         // mean[4], 1/std[4] of the features
    float gate;                // learned start only where feature 3 exceeds it
};

__device__ __forceinline__ float silu(float x) { return x / (1.0f + __expf(-x)); }

// Features of a single-step solve, from the quantities of kep_setup, in
// FP32 (they only feed the network's guess): log r0, log |v0|, the cosine of
// the angle between r0 and v0, and the orbital phase of the step
// log(|dt| sqrt(m / r0^3)), formed from logarithms so that no power
// overflows.  kep_phase alone decides whether the network is evaluated.
__device__ __forceinline__ float kep_phase(const KepArg<double> &k)
{
    const float lr = __logf((float)k.r0);
    return __logf(fabsf((float)k.dt)) + 0.5f * (__logf((float)k.m) - 3.0f * lr);
}

__device__ __forceinline__ void kep_features(const KepArg<double> &k,
                                             const double *p, float *f)
{
    const float vx = (float)p[3], vy = (float)p[4], vz = (float)p[5];
    const float v = sqrtf(vx * vx + vy * vy + vz * vz);
    const float vs = v > 0.f ? v : 1e-30f;
    const float r = (float)k.r0;
    f[0] = __logf(r);
    f[1] = __logf(vs);
    f[2] = (float)k.rv0 / (r * vs);
    f[3] = kep_phase(k);
}

// Learned start of one solve: s0 scaled by exp(network); false (keep the
// plain guess) when the network's output is not finite.
__device__ __forceinline__ bool learned_start(double s0, double *start,
                                              float y)
{
    if (!isfinite(y)) return false;
    *start = s0 * (double)__expf(y);
    return true;
}

// Weights are shared by every thread of a block: staged once in shared memory
// (bf16), activations in registers, FP32 fused multiply-adds.
struct MlpSmem {
    __nv_bfloat16 w1[MLP_H * MLP_IN];
    __nv_bfloat16 w2[MLP_H * MLP_H];
    __nv_bfloat16 w3[MLP_H];
    float b1[MLP_H], b2[MLP_H], b3, norm[8];
};

__device__ void mlp_stage(MlpSmem &S, const MlpParams &P)
{
    for (int t = threadIdx.x; t < MLP_H * MLP_H; t += blockDim.x) {
        S.w2[t] = P.w2[t];
        if (t < MLP_H * MLP_IN) S.w1[t] = P.w1[t];
        if (t < MLP_H) {
            S.w3[t] = P.w3[t];
            S.b1[t] = P.b1[t];
            S.b2[t] = P.b2[t];
        }
        if (t < 8) S.norm[t] = P.norm[t];
        if (t == 0) S.b3 = P.b3[0];
    }
}

__device__ float mlp_eval(const MlpSmem &S, const float *x_raw)
{
    float x[MLP_IN];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k)
        x[k] = (x_raw[k] - S.norm[k]) * S.norm[4 + k];
    float h1[MLP_H];
#pragma unroll
    for (int o = 0; o < MLP_H; ++o) {
        float a = S.b1[o];
#pragma unroll
        for (int k = 0; k < MLP_IN; ++k)
            a = __fmaf_rn(__bfloat162float(S.w1[o * MLP_IN + k]), x[k], a);
        h1[o] = silu(a);
    }
    float y = S.b3;
    for (int o = 0; o < MLP_H; ++o) {
        float a = S.b2[o];
#pragma unroll
        for (int k = 0; k < MLP_H; ++k)
            a = __fmaf_rn(__bfloat162float(S.w2[o * MLP_H + k]), h1[k], a);
        y = __fmaf_rn(__bfloat162float(S.w3[o]), silu(a), y);
    }
    return y;
}

// ---------------------------------------------------------------------------
// Standalone pair solver: one universal_kepler_solver per pair (as the Kepler
// branch of twobody_solver calls it), optional learned start, optional record
// of (features, log(root / plain guess)) of each pair's first single-step
// solve for training.
// ---------------------------------------------------------------------------
struct PairSolve {
    uint64_t n;
    double dt;
    const double *m, *e2, *state;   // state: n x 6 (r, v)
    double *out;                    // n x 6
    int *iters;                     // Laguerre updates per pair (or null)
    float *rec_x, *rec_y;           // n x 4 features, n targets (or null)
    long long budget;
    int use_mlp;
    int form;                       // KeplerForm of the single-step solves
    MlpParams mlp;
};

__global__ void __launch_bounds__(128)
k_pair_solve(const PairSolve P, unsigned *err)
{
    __shared__ MlpSmem S;
    if (P.use_mlp) mlp_stage(S, P.mlp);
    __syncthreads();
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P.n) return;
    double p0[6], p1[6];
    for (int c = 0; c < 6; ++c) p0[c] = P.state[6 * q + c];
    const double m = P.m[q], e2 = P.e2[q];
    KepCtx<double> ctx = {0, P.budget, 0, false, false, 0.0};
    ctx.form = P.form;
    KepArg<double> ka;
    double s0;
    const bool moving = kep_setup(P.dt, m, e2, p0, &ka, &s0);
    if (moving && P.use_mlp && !P.rec_x && kep_phase(ka) > P.mlp.gate) {
        float f[MLP_IN];
        kep_features(ka, p0, f);
        ctx.use_start = learned_start(s0, &ctx.start, mlp_eval(S, f));
    }
    if (moving && P.rec_x) {
        float f[MLP_IN];
        kep_features(ka, p0, f);
        if (P.use_mlp && f[3] > P.mlp.gate)
            ctx.use_start = learned_start(s0, &ctx.start, mlp_eval(S, f));
        for (int k = 0; k < MLP_IN; ++k) P.rec_x[4 * q + k] = f[k];
        double root;
        int it = 0;
        const int st = kep_laguerre(s0, &root, ka, &it);
        P.rec_y[q] = (st == 0 && root / s0 > 0)
                         ? (float)log(root / s0) : __int_as_float(0x7fc00000);
    }
    kep_solve(P.dt, m, e2, p0, p1, ctx);
    for (int c = 0; c < 6; ++c) P.out[6 * q + c] = p1[c];
    if (P.iters) P.iters[q] = (int)ctx.iterations;
    if (ctx.exhausted) atomicOr(err, (unsigned)DERR_KEPLER_BUDGET);
}

// ---------------------------------------------------------------------------
// Queued Sakura sweep (flags -1 and +1).
// ---------------------------------------------------------------------------
constexpr int SK_THREADS = 128;
constexpr int SK_TILE = 128;

struct SakuraArgs {
    uint64_t ni, nj;
    const double *ip[8], *jp[8];
    double *out[6];
    double dt;
    long long flag;
    unsigned *cnt;          // ni (pass 1), then offsets (pass 2)
    unsigned *queue_j;      // Kepler pairs: j index
    unsigned *queue_i;      // Kepler pairs: i index
    double *contrib;        // 6 per queued pair
    int *iters;             // per queued pair (or null)
    long long budget;
    int use_mlp;
    int form;               // KeplerForm of the Kepler-branch solves
    MlpParams mlp;
};

// Drift applied before the two-body step for flag -1 (sakura_kernel_common.h
// :151-157); flag +1 evolves first and drifts after (:158-164).
__device__ __forceinline__ bool sk_kepler(const double *ip, const double *jp,
                                          double dt, long long flag,
                                          double *p0, double *pre, double *m,
                                          double *e2)
{
    pair_state(ip, jp, p0, m, e2);
    for (int c = 0; c < 6; ++c) pre[c] = p0[c];
    if (flag == -1) {
        pre[0] -= pre[3] * dt;
        pre[1] -= pre[4] * dt;
        pre[2] -= pre[5] * dt;
    }
    return !takes_leapfrog(*m, pre);
}

template <int PASS>
__global__ void __launch_bounds__(SK_THREADS)
k_sakura_pass(const SakuraArgs A)
{
    __shared__ double tile[8][SK_TILE];
    const uint64_t i = (uint64_t)blockIdx.x * SK_THREADS + threadIdx.x;
    const uint64_t ic = i < A.ni ? i : A.ni - 1;
    double ip[8];
    for (int a = 0; a < 8; ++a) ip[a] = A.ip[a][ic];
    const double dt = A.dt;
    const long long flag = A.flag;
    double o[6] = {0, 0, 0, 0, 0, 0};
    unsigned count = 0;
    const unsigned base = (PASS == 2 && i < A.ni) ? A.cnt[i] : 0;
    for (uint64_t j0 = 0; j0 < A.nj; j0 += SK_TILE) {
        const int n = (int)((A.nj - j0) < SK_TILE ? (A.nj - j0) : SK_TILE);
        __syncthreads();
        for (int t = threadIdx.x; t < 8 * SK_TILE; t += SK_THREADS) {
            const int a = t / SK_TILE, jj = t % SK_TILE;
            if (jj < n) tile[a][jj] = A.jp[a][j0 + jj];
        }
        __syncthreads();
        for (int jj = 0; jj < n; ++jj) {
            double jp[8];
            for (int a = 0; a < 8; ++a) jp[a] = tile[a][jj];
            double p0[6], pre[6], m, e2;
            const bool kep = sk_kepler(ip, jp, dt, flag, p0, pre, &m, &e2);
            if (PASS == 1) {
                count += kep ? 1u : 0u;
                continue;
            }
            if (kep) {
                if (i < A.ni) {
                    A.queue_j[base + count] = (unsigned)(j0 + jj);
                    A.queue_i[base + count] = (unsigned)i;
                }
                ++count;
                continue;
            }
            double p1[6];
            two_body_leapfrog(dt, m, e2, pre, p1);
            if (flag == 1) {
                p1[0] -= p1[3] * dt;
                p1[1] -= p1[4] * dt;
                p1[2] -= p1[5] * dt;
            }
            const double mu = jp[0] / m;
            for (int q = 0; q < 6; ++q) o[q] += mu * (p1[q] - p0[q]);
        }
    }
    if (i >= A.ni) return;
    if (PASS == 1) {
        A.cnt[i] = count;
    } else {
        for (int q = 0; q < 6; ++q) A.out[q][i] = o[q];
    }
}

// SPLIT mode of the two passes (flags -1 and +1): FP32 pair arithmetic on
// the packed double-single records.  In the leapfrog branch the pair's
// change over the step has a closed form: with the midpoint position
// b = r0 + flag v0 dt/2 and a = -m b / |b|^3 (softened), the velocity
// changes by a dt and the position by -flag a dt^2/2 (the algebra of
// sakura_kernel_common.h:45-91 with :151-164), so each pair is one
// acceleration evaluation formed directly as increments (no difference of
// nearly equal FP32 states).  The branch test is the reference's
// (r^2 > (64 m / v^2)^2, sakura_kernel_common.h:109-123) in FP32; both
// passes take the same decisions.  Kepler-branch pairs go to the same
// queue and fp64 solver as in EXACT mode.
constexpr int SKS_TILE = 256;

template <int PASS>
__global__ void __launch_bounds__(SK_THREADS)
k_sakura_split_pass(const SakuraArgs A, const float4 *irec, const float4 *jrec)
{
    __shared__ float4 tile[SKS_TILE * 3];
    const uint64_t i = (uint64_t)blockIdx.x * SK_THREADS + threadIdx.x;
    const uint64_t ic = i < A.ni ? i : A.ni - 1;
    const float4 ia = irec[3 * ic], ib = irec[3 * ic + 1], iv = irec[3 * ic + 2];
    const float fl = (float)A.flag;
    const float dt = (float)A.dt, hdt = 0.5f * dt, dt2h = 0.5f * dt * dt;
    double o[6] = {0, 0, 0, 0, 0, 0};
    float part[6] = {0, 0, 0, 0, 0, 0};
    int run = 0;
    unsigned count = 0;
    const unsigned base = (PASS == 2 && i < A.ni) ? A.cnt[i] : 0;
    for (uint64_t j0 = 0; j0 < A.nj; j0 += SKS_TILE) {
        const int n = (int)((A.nj - j0) < SKS_TILE ? (A.nj - j0) : SKS_TILE);
        __syncthreads();
        for (int t = threadIdx.x; t < 3 * n; t += SK_THREADS)
            tile[t] = jrec[3 * j0 + t];
        __syncthreads();
        for (int jj = 0; jj < n; ++jj) {
            const float4 ja = tile[3 * jj], jb = tile[3 * jj + 1],
                         jv = tile[3 * jj + 2];
            const float dx = (ia.x - ja.x) + (ib.x - jb.x);
            const float dy = (ia.y - ja.y) + (ib.y - jb.y);
            const float dz = (ia.z - ja.z) + (ib.z - jb.z);
            const float ux = iv.x - jv.x, uy = iv.y - jv.y, uz = iv.z - jv.z;
            const float m = ia.w + ja.w, e2 = ib.w + jb.w;
            // state the two-body step starts from: flag -1 drifts back first
            const float sh = fl < 0.f ? -dt : 0.f;
            const float px = fmaf(ux, sh, dx), py = fmaf(uy, sh, dy),
                        pz = fmaf(uz, sh, dz);
            const float r2p = fmaf(pz, pz, fmaf(py, py, px * px));
            const float v2 = fmaf(uz, uz, fmaf(uy, uy, ux * ux));
            const float R = 64.0f * (m / v2);
            if (!(r2p > R * R)) {           // Kepler branch
                if (PASS == 2 && i < A.ni) {
                    A.queue_j[base + count] = (unsigned)(j0 + jj);
                    A.queue_i[base + count] = (unsigned)i;
                }
                ++count;
                continue;
            }
            if (PASS == 1) continue;
            const float bx = fmaf(ux, fl * hdt, dx), by = fmaf(uy, fl * hdt, dy),
                        bz = fmaf(uz, fl * hdt, dz);
            const float r2b = fmaf(bz, bz, fmaf(by, by, bx * bx));
            float y = rsqrt_nr(r2b + e2);
            y = r2b > 0.f ? y : 0.f;
            const float jmk = -ja.w * (y * y) * y;      // -(m_j/m) m k
            const float av = jmk * dt, ar = -fl * jmk * dt2h;
            part[0] = fmaf(ar, bx, part[0]);
            part[1] = fmaf(ar, by, part[1]);
            part[2] = fmaf(ar, bz, part[2]);
            part[3] = fmaf(av, bx, part[3]);
            part[4] = fmaf(av, by, part[4]);
            part[5] = fmaf(av, bz, part[5]);
            if (++run == 16) {
                for (int q = 0; q < 6; ++q) {
                    o[q] += (double)part[q];
                    part[q] = 0.f;
                }
                run = 0;
            }
        }
    }
    if (i >= A.ni) return;
    if (PASS == 1) {
        A.cnt[i] = count;
    } else {
        for (int q = 0; q < 6; ++q) A.out[q][i] = o[q] + (double)part[q];
    }
}

// Exclusive scan of n counts in place (one block; returns the total).
__global__ void k_scan(unsigned *x, uint64_t n, unsigned long long *total)
{
    __shared__ unsigned long long carry;
    __shared__ unsigned long long part[1024];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t b = 0; b < n; b += blockDim.x) {
        const uint64_t i = b + threadIdx.x;
        unsigned long long v = i < n ? x[i] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            unsigned long long t =
                threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) x[i] = (unsigned)(carry + part[threadIdx.x] - v);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += part[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Step 4: one thread per queued pair.
__global__ void __launch_bounds__(128)
k_sakura_kepler(const SakuraArgs A, uint64_t nq, unsigned *err)
{
    __shared__ MlpSmem S;
    if (A.use_mlp) mlp_stage(S, A.mlp);
    __syncthreads();
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const uint64_t i = A.queue_i[q], j = A.queue_j[q];
    double ip[8], jp[8];
    for (int a = 0; a < 8; ++a) {
        ip[a] = A.ip[a][i];
        jp[a] = A.jp[a][j];
    }
    double p0[6], pre[6], m, e2, p1[6];
    sk_kepler(ip, jp, A.dt, A.flag, p0, pre, &m, &e2);
    KepCtx<double> ctx = {0, A.budget, 0, false, false, 0.0};
    ctx.form = A.form;
    if (A.use_mlp) {
        KepArg<double> ka;
        double s0;
        if (kep_setup(A.dt, m, e2, pre, &ka, &s0) &&
            kep_phase(ka) > A.mlp.gate) {
            float f[MLP_IN];
            kep_features(ka, pre, f);
            ctx.use_start = learned_start(s0, &ctx.start, mlp_eval(S, f));
        }
    }
    kep_solve(A.dt, m, e2, pre, p1, ctx);
    if (A.flag == 1) {
        p1[0] -= p1[3] * A.dt;
        p1[1] -= p1[4] * A.dt;
        p1[2] -= p1[5] * A.dt;
    }
    const double mu = jp[0] / m;
    for (int c = 0; c < 6; ++c) A.contrib[6 * q + c] = mu * (p1[c] - p0[c]);
    if (A.iters) A.iters[q] = (int)ctx.iterations;
    if (ctx.exhausted) atomicOr(err, (unsigned)DERR_KEPLER_BUDGET);
}

// Step 5: add each i's queued contributions in queue (= j) order.
__global__ void k_sakura_gather(const SakuraArgs A, uint64_t nq)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.ni) return;
    const uint64_t b = A.cnt[i];
    const uint64_t e = (i + 1 < A.ni) ? A.cnt[i + 1] : nq;
    double o[6];
    for (int c = 0; c < 6; ++c) o[c] = A.out[c][i];
    for (uint64_t q = b; q < e; ++q)
        for (int c = 0; c < 6; ++c) o[c] += A.contrib[6 * q + c];
    for (int c = 0; c < 6; ++c) A.out[c][i] = o[c];
}

}  // namespace tg

using namespace tg;

namespace {

struct SakuraWork {
    unsigned *cnt = nullptr;
    size_t cnt_cap = 0;
    unsigned *qi = nullptr, *qj = nullptr;
    double *contrib = nullptr;
    int *iters = nullptr;
    size_t q_cap = 0;
    unsigned long long *total = nullptr;
    unsigned *err = nullptr;
    float4 *rec = nullptr;            // SPLIT mode: packed i and j records
    size_t rec_cap = 0;
};

SakuraWork g_work;
MlpParams g_mlp;
bool g_have_mlp = false;
int g_kepler_form = KEP_REFERENCE;   // tupan_gb300_kepler_set_form

int grow_queue(size_t nq)
{
    if (nq <= g_work.q_cap) return 0;
    cudaFree(g_work.qi);
    cudaFree(g_work.qj);
    cudaFree(g_work.contrib);
    cudaFree(g_work.iters);
    size_t cap = nq + nq / 2 + 1024;
    if (cudaMalloc((void **)&g_work.qi, cap * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&g_work.qj, cap * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void **)&g_work.contrib, cap * 6 * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&g_work.iters, cap * sizeof(int)) != cudaSuccess)
        return 1;
    g_work.q_cap = cap;
    return 0;
}

}  // namespace

// ===========================================================================
// C-ABI (no counterpart in the reference).
// ===========================================================================

// Installs (or, with w1 == NULL, removes) the learned-start network: DEVICE
// pointers to bf16 weights w1 (64x4), w2 (64x64), w3 (64), fp32 biases b1,
// b2, b3 and the feature normalisation norm[8] = mean[4], 1/std[4].  The
// network is evaluated only for solves whose feature log(|dt| sqrt(m/r^3))
// exceeds `gate` (where the plain guess needs more than the minimum two
// updates); elsewhere the plain guess is kept.  The arrays must stay valid
// while the network is installed.
TG_EXPORT int tupan_gb300_kepler_set_mlp(const void *w1, const float *b1,
                                         const void *w2, const float *b2,
                                         const void *w3, const float *b3,
                                         const float *norm, float gate)
{
    if (!w1) {
        g_have_mlp = false;
        return ST_OK;
    }
    g_mlp.w1 = (const __nv_bfloat16 *)w1;
    g_mlp.b1 = b1;
    g_mlp.w2 = (const __nv_bfloat16 *)w2;
    g_mlp.b2 = b2;
    g_mlp.w3 = (const __nv_bfloat16 *)w3;
    g_mlp.b3 = b3;
    g_mlp.norm = norm;
    g_mlp.gate = gate;
    g_have_mlp = true;
    return ST_OK;
}

// Form of the universal-Kepler root solve used by the pair solver, the
// queued Sakura sweep and the device Sakura integrator: 0 the reference's
// structure (default), 1 the same arithmetic with one cos/sin (cosh/sinh)
// per Laguerre update (bit-identical), 2 FP32 Laguerre updates then FP64
// updates to the reference's 2^-42 tolerance (see tg_kepler.cuh).  The ten
// libtupan.h entry points always use form 0.  Returns the previous form, or
// -1 for an unknown one.
TG_EXPORT int tupan_gb300_kepler_set_form(int form)
{
    if (form < KEP_REFERENCE || form > KEP_MIXED) return -1;
    const int old = g_kepler_form;
    g_kepler_form = form;
    return old;
}

// Solves n independent pairs (DEVICE arrays: m, e2, state n x 6, out n x 6)
// over dt with universal_kepler_solver's full retry logic; iters, rec_x
// (n x 4) and rec_y (n) are optional.  use_mlp selects the learned start.
// Synchronous; returns a status code (3: a solve hit the budget).
TG_EXPORT int tupan_gb300_kepler_pairs(uint64_t n, double dt, const double *m,
                                       const double *e2, const double *state,
                                       double *out, int *iters, float *rec_x,
                                       float *rec_y, int use_mlp,
                                       long long budget, void *stream)
{
    if (use_mlp && !g_have_mlp) return ST_BAD_ARGUMENT;
    if (!g_work.err && cudaMalloc((void **)&g_work.err, sizeof(unsigned)) !=
                           cudaSuccess)
        return ST_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    cudaMemsetAsync(g_work.err, 0, sizeof(unsigned), st);
    PairSolve P;
    memset(&P, 0, sizeof(P));
    P.n = n;
    P.dt = dt;
    P.m = m;
    P.e2 = e2;
    P.state = state;
    P.out = out;
    P.iters = iters;
    P.rec_x = rec_x;
    P.rec_y = rec_y;
    P.budget = budget > 0 ? budget : (1LL << 20);
    P.use_mlp = use_mlp;
    P.form = g_kepler_form;
    P.mlp = g_mlp;
    if (n) {
        k_pair_solve<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(P, g_work.err);
        g_launch_count += 1;
    }
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, g_work.err, sizeof(unsigned),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ST_CUDA;
    return h ? ST_DEVICE : ST_OK;
}

// sakura_kernel (libtupan.h:203-229) on DEVICE arrays with the Kepler-branch
// pairs solved as a queue; flag must be -1 or +1 (the integrator's flags).
// i_attrs/j_attrs: 8 device pointers each (m r e2 v); outs: 6.  Optional
// iteration histogram: kepler_iters (host, 65 bins; bin k counts solves with
// k Laguerre updates, the last bin k >= 64).  Returns the number of queued
// (Kepler-branch) pairs in *n_kepler.  Synchronous.
TG_EXPORT int tupan_gb300_sakura_queue(uint64_t ni, const void *const *i_attrs,
                                       uint64_t nj, const void *const *j_attrs,
                                       double dt, int64_t flag,
                                       void *const *outs, int use_mlp,
                                       long long budget, void *stream,
                                       unsigned long long *n_kepler,
                                       long long *kepler_iters, int mode)
{
    if (flag != -1 && flag != 1) return ST_BAD_ARGUMENT;
    if (mode != MODE_EXACT && mode != MODE_SPLIT) return ST_BAD_ARGUMENT;
    if (use_mlp && !g_have_mlp) return ST_BAD_ARGUMENT;
    if (ni == 0) return ST_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (!g_work.err && (cudaMalloc((void **)&g_work.err, sizeof(unsigned)) !=
                            cudaSuccess))
        return ST_CUDA;
    if (!g_work.total &&
        cudaMalloc((void **)&g_work.total, sizeof(unsigned long long)) !=
            cudaSuccess)
        return ST_CUDA;
    if (ni > g_work.cnt_cap) {
        cudaFree(g_work.cnt);
        if (cudaMalloc((void **)&g_work.cnt, ni * sizeof(unsigned)) != cudaSuccess)
            return ST_CUDA;
        g_work.cnt_cap = ni;
    }
    SakuraArgs A;
    memset(&A, 0, sizeof(A));
    A.ni = ni;
    A.nj = nj;
    for (int a = 0; a < 8; ++a) {
        A.ip[a] = (const double *)i_attrs[a];
        A.jp[a] = (const double *)j_attrs[a];
    }
    for (int c = 0; c < 6; ++c) A.out[c] = (double *)outs[c];
    A.dt = dt;
    A.flag = flag;
    A.cnt = g_work.cnt;
    A.budget = budget > 0 ? budget : (1LL << 20);
    A.use_mlp = use_mlp;
    A.form = g_kepler_form;
    A.mlp = g_mlp;
    cudaMemsetAsync(g_work.err, 0, sizeof(unsigned), st);
    const unsigned blocks = (unsigned)((ni + SK_THREADS - 1) / SK_THREADS);
    const float4 *irec = nullptr, *jrec = nullptr;
    if (mode == MODE_SPLIT) {
        bool same = ni == nj;
        for (int a = 0; a < 8 && same; ++a) same = i_attrs[a] == j_attrs[a];
        const size_t need = (ni + (same ? 0 : nj)) * 3;
        if (need > g_work.rec_cap) {
            cudaFree(g_work.rec);
            g_work.rec = nullptr;
            g_work.rec_cap = 0;
            if (cudaMalloc((void **)&g_work.rec, need * sizeof(float4)) !=
                cudaSuccess)
                return ST_CUDA;
            g_work.rec_cap = need;
        }
        if (launch_pack(K_ACC_JERK, ni, i_attrs, g_work.rec, st) != cudaSuccess)
            return ST_CUDA;
        if (!same && launch_pack(K_ACC_JERK, nj, j_attrs, g_work.rec + ni * 3,
                                 st) != cudaSuccess)
            return ST_CUDA;
        irec = g_work.rec;
        jrec = same ? g_work.rec : g_work.rec + ni * 3;
    }
    if (mode == MODE_SPLIT)
        k_sakura_split_pass<1><<<blocks, SK_THREADS, 0, st>>>(A, irec, jrec);
    else
        k_sakura_pass<1><<<blocks, SK_THREADS, 0, st>>>(A);
    k_scan<<<1, 1024, 0, st>>>(g_work.cnt, ni, g_work.total);
    g_launch_count += 2;
    unsigned long long nq = 0;
    if (cudaMemcpyAsync(&nq, g_work.total, sizeof(nq), cudaMemcpyDeviceToHost,
                        st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ST_CUDA;
    if (grow_queue(nq ? nq : 1)) return ST_CUDA;
    A.queue_i = g_work.qi;
    A.queue_j = g_work.qj;
    A.contrib = g_work.contrib;
    A.iters = kepler_iters ? g_work.iters : nullptr;
    if (mode == MODE_SPLIT)
        k_sakura_split_pass<2><<<blocks, SK_THREADS, 0, st>>>(A, irec, jrec);
    else
        k_sakura_pass<2><<<blocks, SK_THREADS, 0, st>>>(A);
    g_launch_count += 1;
    if (nq) {
        k_sakura_kepler<<<(unsigned)((nq + 127) / 128), 128, 0, st>>>(
            A, nq, g_work.err);
        k_sakura_gather<<<(unsigned)((ni + 127) / 128), 128, 0, st>>>(A, nq);
        g_launch_count += 2;
    }
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, g_work.err, sizeof(unsigned),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ST_CUDA;
    if (n_kepler) *n_kepler = nq;
    if (kepler_iters) {
        for (int k = 0; k < 65; ++k) kepler_iters[k] = 0;
        if (nq) {
            int *hi = (int *)malloc(nq * sizeof(int));
            if (!hi) return ST_CUDA;
            cudaMemcpy(hi, g_work.iters, nq * sizeof(int), cudaMemcpyDeviceToHost);
            for (unsigned long long q = 0; q < nq; ++q)
                kepler_iters[hi[q] < 64 ? hi[q] : 64] += 1;
            free(hi);
        }
    }
    return h ? ST_DEVICE : ST_OK;
}

// ===========================================================================
// Device-resident Sakura integrator (sakura.py:22-50, fixed step): per step
// drift tau/2, queued Sakura sweeps with flag -1 then +1 at dt = tau/2, each
// followed by r += dr, v += dv, and a final drift tau/2.  State in HBM.
// ===========================================================================
namespace {

__global__ void k_drift(double *r0, double *r1, double *r2, const double *v0,
                        const double *v1, const double *v2, uint64_t n,
                        double tau)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        r0[i] = r0[i] + v0[i] * tau / 2;
        r1[i] = r1[i] + v1[i] * tau / 2;
        r2[i] = r2[i] + v2[i] * tau / 2;
    }
}

__global__ void k_kick(double *const *x, const double *const *d, uint64_t n)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        for (int c = 0; c < 6; ++c) x[c][i] = x[c][i] + d[c][i];
}

struct SakuraSys {
    uint64_t n = 0;
    double *pool = nullptr;          // m e2 r3 v3 d6
    double *a[8];                    // m r(3) e2 v(3), the kernels' order
    double *d[6];
    double **xd = nullptr, **dd = nullptr;   // device arrays of pointers
    cudaStream_t stream = nullptr;
    int use_mlp = 0;
    int mode = MODE_EXACT;           // Sakura sweeps: EXACT or SPLIT
    long long kepler_total = 0, steps = 0;
    long long hist[65] = {0};
    double t = 0.0;
};

}  // namespace

TG_EXPORT int tupan_gb300_sakura_destroy(void *handle);

TG_EXPORT int tupan_gb300_sakura_create(uint64_t n, const double *m,
                                        const double *e2, const double *rx,
                                        const double *ry, const double *rz,
                                        const double *vx, const double *vy,
                                        const double *vz, void **handle)
{
    if (!handle || n == 0) return ST_BAD_ARGUMENT;
    SakuraSys *S = new SakuraSys();
    CreateGuard guard{S, tupan_gb300_sakura_destroy};
    S->n = n;
    if (cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) !=
            cudaSuccess ||
        cudaMalloc((void **)&S->pool, 14 * n * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&S->xd, 6 * sizeof(double *)) != cudaSuccess ||
        cudaMalloc((void **)&S->dd, 6 * sizeof(double *)) != cudaSuccess)
        return ST_CUDA;
    for (int k = 0; k < 8; ++k) S->a[k] = S->pool + (size_t)k * n;
    for (int k = 0; k < 6; ++k) S->d[k] = S->pool + (size_t)(8 + k) * n;
    const double *src[8] = {m, rx, ry, rz, e2, vx, vy, vz};
    for (int k = 0; k < 8; ++k)
        if (cudaMemcpy(S->a[k], src[k], n * sizeof(double),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return ST_CUDA;
    double *xs[6] = {S->a[1], S->a[2], S->a[3], S->a[5], S->a[6], S->a[7]};
    cudaMemcpy(S->xd, xs, sizeof(xs), cudaMemcpyHostToDevice);
    cudaMemcpy(S->dd, S->d, sizeof(S->d), cudaMemcpyHostToDevice);
    *handle = S;
    guard.keep();
    return ST_OK;
}

// Fixed-step Sakura steps of size tau until t >= t_end (t_end - t a multiple
// of tau is the intended use).  use_mlp: learned Kepler start.  kepler_iters
// (host, 65 bins) accumulates the Laguerre-update histogram if not NULL.
TG_EXPORT int tupan_gb300_sakura_evolve(void *handle, double tau, double t_end,
                                        int use_mlp, double *t_out,
                                        long long *steps_out,
                                        long long *kepler_out,
                                        long long *kepler_iters)
{
    SakuraSys *S = (SakuraSys *)handle;
    if (!S || !(tau > 0)) return ST_BAD_ARGUMENT;
    const uint64_t n = S->n;
    const unsigned g = (unsigned)((n + 255) / 256 < 1216 ? (n + 255) / 256 : 1216);
    void *ia[8];
    for (int k = 0; k < 8; ++k) ia[k] = S->a[k];
    void *oa[6];
    for (int k = 0; k < 6; ++k) oa[k] = S->d[k];
    long long h[65];
    while (S->t < t_end) {
        k_drift<<<g, 256, 0, S->stream>>>(S->a[1], S->a[2], S->a[3], S->a[5],
                                          S->a[6], S->a[7], n, tau);
        g_launch_count += 1;
        for (int flag = -1; flag <= 1; flag += 2) {
            unsigned long long nk = 0;
            int st = tupan_gb300_sakura_queue(n, ia, n, ia, tau / 2, flag, oa,
                                              use_mlp, 0, S->stream, &nk,
                                              kepler_iters ? h : nullptr,
                                              S->mode);
            if (st) return st;
            S->kepler_total += (long long)nk;
            if (kepler_iters)
                for (int k = 0; k < 65; ++k) kepler_iters[k] += h[k];
            k_kick<<<g, 256, 0, S->stream>>>(S->xd, S->dd, n);
            g_launch_count += 1;
        }
        k_drift<<<g, 256, 0, S->stream>>>(S->a[1], S->a[2], S->a[3], S->a[5],
                                          S->a[6], S->a[7], n, tau);
        g_launch_count += 1;
        S->t += tau;
        S->steps += 1;
    }
    if (cudaStreamSynchronize(S->stream) != cudaSuccess) return ST_CUDA;
    if (t_out) *t_out = S->t;
    if (steps_out) *steps_out = S->steps;
    if (kepler_out) *kepler_out = S->kepler_total;
    return ST_OK;
}

// Sakura sweeps of the integrator: mode 0 EXACT (default), 1 SPLIT.
TG_EXPORT int tupan_gb300_sakura_set_mode(void *handle, int mode)
{
    SakuraSys *S = (SakuraSys *)handle;
    if (!S || (mode != MODE_EXACT && mode != MODE_SPLIT)) return ST_BAD_ARGUMENT;
    S->mode = mode;
    return ST_OK;
}

TG_EXPORT int tupan_gb300_sakura_get_state(void *handle, double *rx,
                                           double *ry, double *rz, double *vx,
                                           double *vy, double *vz)
{
    SakuraSys *S = (SakuraSys *)handle;
    if (!S) return ST_BAD_ARGUMENT;
    double *dst[6] = {rx, ry, rz, vx, vy, vz};
    double *src[6] = {S->a[1], S->a[2], S->a[3], S->a[5], S->a[6], S->a[7]};
    for (int k = 0; k < 6; ++k)
        if (cudaMemcpy(dst[k], src[k], S->n * sizeof(double),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_CUDA;
    return ST_OK;
}

TG_EXPORT int tupan_gb300_sakura_destroy(void *handle)
{
    SakuraSys *S = (SakuraSys *)handle;
    if (!S) return ST_BAD_ARGUMENT;
    cudaStreamSynchronize(S->stream);
    cudaFree(S->pool);
    cudaFree(S->xd);
    cudaFree(S->dd);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
    return ST_OK;
}
