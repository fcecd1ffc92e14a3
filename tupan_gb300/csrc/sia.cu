// Device-resident SIA driver: tupan's symplectic integrators with
// hierarchical slow/fast splitting (tupan/integrator/sia.py), the particles
// kept in HBM for the whole run.
//
// The reference copies the particle system at every split (ps[condition])
// and concatenates slow and fast again at every join (sia.py:22-55).  Here a
// subsystem is a contiguous index range of one set of SoA arrays: a split is
// a stable in-place partition of its range (slow first, fast after), so the
// join is free and the order of particles -- which fixes the j order of
// every later pairwise sum -- is exactly the reference's.  The recursion
// (SIA.recurse, sia.py:1097-1123) runs on the host, as in the reference; it
// reads back one count per split (and the minimum step per level in shared-
// adaptive mode).  A subsystem of at most 128 particles is handed whole to
// one CTA that runs the rest of its recursion on the device.  Forces use the library's sweeps on sub-ranges: in EXACT
// mode every sweep is bit-identical to the reference C, and the drift,
// kick and bookkeeping kernels are compiled with -fmad=false and round like
// numpy, so a run matches the reference integrator bit for bit except where
// a two-body subsystem calls the Kepler solver (CUDA's transcendental
// functions against libm).
//
// Post-Newtonian corrections (sia.py:84-157) are not implemented: creating
// a system always gives the Newtonian integrator.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cfloat>
#include <chrono>
#include <utility>
#include <vector>

#include "tg_common.cuh"
#include "tg_kepler.cuh"
#include "tg_pairs.cuh"
#include "tg_split_ops.cuh"

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
int split_nf_host(int kernel);
}  // namespace tg

using namespace tg;

namespace {

// SoA fields, the first eight in the kernels' attribute order (m r e2 v).
enum Field {
    F_M = 0, F_RX, F_RY, F_RZ, F_E2, F_VX, F_VY, F_VZ,
    F_AX, F_AY, F_AZ, F_TSTEP, F_TSTEPIJ, F_TIME,
    F_NSTEP,    // int64
    F_ID,       // int64
    NFIELD
};

struct Fields {
    double *f[NFIELD];
};

// Splitting coefficients of tupan/integrator/sia.py:300-864 (Yoshida 1990;
// Omelyan, Mryglod & Folk 2003; Blanes & Moan 2002; Kahan & Li 1997):
// {first list, second list} per scheme.
struct Scheme {
    const char *name;
    int n_first, n_second;
    double first[5], second[5];
};

const Scheme kSchemes[] = {
    {"sia21", 1, 1, {1.0}, {0.5}},
    {"sia22", 1, 2, {0.5}, {0.1931833275037836, 0.6136333449924328}},
    {"sia43", 2, 2, {1.3512071919596575, -1.7024143839193150},
     {0.6756035959798288, -0.17560359597982877}},
    {"sia44", 2, 3, {0.7123418310626056, -0.21234183106260562},
     {0.1786178958448091, -0.06626458266981843, 0.7752933736500186}},
    {"sia45", 3, 3, {-0.0844296195070715, 0.354900057157426, 0.459059124699291},
     {0.2750081212332419, -0.1347950099106792, 0.35978688867743724}},
    {"sia46", 3, 4, {0.209515106613362, -0.143851773179818, 0.434336666566456},
     {0.0792036964311957, 0.353172906049774, -0.0420650803577195,
      0.21937695575349958}},
    {"sia67", 4, 4,
     {0.7845136104775573, 0.23557321335935813, -1.177679984178871,
      1.3151863206839112},
     {0.39225680523877865, 0.5100434119184577, -0.47105338540975644,
      0.06875316825252015}},
    {"sia69", 5, 5,
     {0.39103020330868477, 0.334037289611136, -0.7062272811875614,
      0.08187754964805945, 0.7985644772393624},
     {0.19551510165434238, 0.3625337464599104, -0.1860949957882127,
      -0.31217486576975095, 0.44022101344371095}},
};

// One propagator: the palindrome interleaving the second list ("outer"
// operator) with the first ("inner"): o0 i0 o1 i1 ... mirrored about its
// middle element.  dkd and bridge_sf: outer = drift; kdk: outer = kick.
std::vector<std::pair<bool, double>> make_sequence(const Scheme &s)
{
    std::vector<std::pair<bool, double>> fwd;
    for (int k = 0; k < s.n_second; ++k) {
        fwd.push_back({true, s.second[k]});
        if (k < s.n_first) fwd.push_back({false, s.first[k]});
    }
    std::vector<std::pair<bool, double>> seq = fwd;
    for (int k = (int)fwd.size() - 2; k >= 0; --k) seq.push_back(fwd[k]);
    return seq;
}

// ---------------------------------------------------------------------------
// Kernels on index ranges [lo, lo + n).
// ---------------------------------------------------------------------------
__global__ void k_drift(Fields F, uint64_t lo, uint64_t n, double c)
{
    // sia.py:58-67: r += v * tau
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = lo + k;
        F.f[F_RX][i] = F.f[F_RX][i] + F.f[F_VX][i] * c;
        F.f[F_RY][i] = F.f[F_RY][i] + F.f[F_VY][i] * c;
        F.f[F_RZ][i] = F.f[F_RZ][i] + F.f[F_VZ][i] * c;
    }
}

__global__ void k_kick(Fields F, uint64_t lo, uint64_t n, double c)
{
    // sia.py:70-79: v += a * tau
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = lo + k;
        F.f[F_VX][i] = F.f[F_VX][i] + F.f[F_AX][i] * c;
        F.f[F_VY][i] = F.f[F_VY][i] + F.f[F_AY][i] * c;
        F.f[F_VZ][i] = F.f[F_VZ][i] + F.f[F_AZ][i] * c;
    }
}

__global__ void k_book(Fields F, uint64_t lo, uint64_t n, double tau)
{
    // sia.py:1115-1118: tstep = tau, time += tau, nstep += 1
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = lo + k;
        F.f[F_TSTEP][i] = tau;
        F.f[F_TIME][i] = F.f[F_TIME][i] + tau;
        ((long long *)F.f[F_NSTEP])[i] += 1;
    }
}

// min |x| over the range, as the bit pattern of a non-negative double (such
// patterns order like the values); *out must start at ~0.
__global__ void k_min_abs(const double *x, uint64_t n,
                          unsigned long long *out)
{
    unsigned long long m = ~0ULL;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(
            fabs(x[k]));
        m = b < m ? b : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long p = __shfl_xor_sync(0xffffffffu, m, o);
        m = p < m ? p : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(out, m);
}

constexpr int PART_THREADS = 1024;

// Stable partition of [lo, lo + n) by |tstep| > thr (slow first), through
// the scratch arrays S (indices 0 .. n-1), in one CTA: a counting pass, a
// scatter pass in chunks of PART_THREADS (warp ballots plus a scan of the
// warp counts), and a copy back.  *ns_out receives the slow count.
__global__ void __launch_bounds__(PART_THREADS)
k_partition(Fields F, Fields S, uint64_t lo, uint64_t n, double thr,
            unsigned long long *ns_out)
{
    __shared__ unsigned warp_cnt[PART_THREADS / 32];
    __shared__ unsigned long long total;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) total = 0;
    __syncthreads();
    unsigned long long mine = 0;
    for (uint64_t k = t; k < n; k += PART_THREADS)
        mine += fabs(F.f[F_TSTEP][lo + k]) > thr ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if (lane == 0) atomicAdd(&total, mine);
    __syncthreads();
    const unsigned long long ns = total;
    unsigned long long slow_base = 0, fast_base = 0;
    for (uint64_t base = 0; base < n; base += PART_THREADS) {
        const uint64_t k = base + t;
        const bool valid = k < n;
        const bool slow = valid && fabs(F.f[F_TSTEP][lo + k]) > thr;
        const unsigned b = __ballot_sync(0xffffffffu, slow);
        if (lane == 0) warp_cnt[w] = __popc(b);
        __syncthreads();
        unsigned before = 0, chunk_slow = 0;
        for (int q = 0; q < PART_THREADS / 32; ++q) {
            const unsigned c = warp_cnt[q];
            before += q < w ? c : 0;
            chunk_slow += c;
        }
        const unsigned rank_slow = before + __popc(b & ((1u << lane) - 1u));
        if (valid) {
            const unsigned rank_fast = (unsigned)(k - base) - rank_slow;
            const uint64_t dst = slow ? slow_base + rank_slow
                                      : ns + fast_base + rank_fast;
#pragma unroll
            for (int f = 0; f < NFIELD; ++f) S.f[f][dst] = F.f[f][lo + k];
        }
        const uint64_t in_chunk = (n - base) < (uint64_t)PART_THREADS
                                      ? (n - base) : (uint64_t)PART_THREADS;
        slow_base += chunk_slow;
        fast_base += in_chunk - chunk_slow;
        __syncthreads();
    }
    for (uint64_t k = t; k < n; k += PART_THREADS)
#pragma unroll
        for (int f = 0; f < NFIELD; ++f) F.f[f][lo + k] = S.f[f][k];
    if (t == 0) *ns_out = ns;
}

// ---------------------------------------------------------------------------
// Small subsystems: the whole recursion below one call of SIA.recurse in a
// single CTA.  Deep in the hierarchy the subsystems hold a handful of
// particles and the host-driven path would spend a launch and a host round
// trip on every few-pair sweep; here the subsystem is staged in shared
// memory, the recursion runs on an explicit stack, and every operation --
// Tstep and Acc sums (one i per thread, j in order, the EXACT pair
// arithmetic), block quantisation, stable partition, drift, kick, Kepler
// for two-body subsystems -- is the same arithmetic as the sweeps the host
// path launches, so both paths give identical bits.
// ---------------------------------------------------------------------------
constexpr int SUB_MAX = 128;       // particles (one per thread)
constexpr int SUB_DEPTH = 64;      // recursion levels below the entry
constexpr int SEQ_MAX = 19;        // longest propagator (sia69)

struct SubParams {
    int seq_len;
    int outer[SEQ_MAX];
    double coef[SEQ_MAX];
    int mode;            // 's', 'a' or 'h'
    int kdk;
    int split;           // 1: SPLIT-mode sums (FP32 pairs, DS positions)
    double eta;
    long long budget;
};

// In/out block of one subtree launch.
struct SubCtl {
    double t_curr;
    unsigned status;     // 0 ok, 1 recursion deeper than SUB_DEPTH
    int max_depth;
    long long n_recurse, n_kepler, n_partitions;
    unsigned long long interactions;
};

struct Frame {
    int lo, n, ns, step, sub;
    double tau;
};

__device__ double d_block_tstep(double min_ts, double t, double tau)
{
    // tupan/integrator/__init__.py:59-78
    long long power = quantised_power(min_ts);
    double min_bts = ldexp(1.0, (int)power);
    const double t_next = t + min_bts;
    for (int k = 0; k < 2100 && fmod(t_next, min_bts) != 0.0; ++k)
        min_bts /= 2.0;
    min_bts = copysign(min_bts, tau);
    if (fabs(min_bts) > fabs(tau)) min_bts = tau;
    return min_bts;
}

struct SubState {
    double f[NFIELD][SUB_MAX];
    double x[NFIELD][SUB_MAX];     // partition scratch
    float g[11][SUB_MAX];          // SPLIT images: xh yh zh m xl yl zl e2 v
    Frame stk[SUB_DEPTH];
    int sp;
    double t_curr;
    unsigned status;
    int max_depth;
    long long n_recurse, n_kepler, n_partitions;
    unsigned long long interactions;
    double red[SUB_MAX / 32];
    unsigned wc[SUB_MAX / 32];
    int ns;
    double tau;
};

// i in [ilo, ilo + ni) against j in [jlo, jlo + nj): Acc (out: ax ay az) or
// Tstep (out: tstep tstepij), thread t owns i = ilo + t.
template <class Op>
__device__ void sub_sweep(SubState &S, int ilo, int ni, int jlo, int nj,
                          int first_out, const Sweep &sw)
{
    const int t = threadIdx.x;
    if (t == 0) S.interactions += (unsigned long long)ni * nj;
    if (t < ni) {
        double ip[Op::NA], jp[Op::NA], o[Op::NO];
#pragma unroll
        for (int a = 0; a < Op::NA; ++a) ip[a] = S.f[a][ilo + t];
        Op::init(o);
        for (int j = 0; j < nj; ++j) {
#pragma unroll
            for (int a = 0; a < Op::NA; ++a) jp[a] = S.f[a][jlo + j];
            Op::pair(ip, jp, o, sw);
        }
        Op::finish(ip, o, sw);
#pragma unroll
        for (int c = 0; c < Op::NO; ++c) S.f[first_out + c][ilo + t] = o[c];
    }
    __syncthreads();
}

// SPLIT mode: the same FP32 pair operators as the sweep kernels on
// double-single images of the subsystem, each run of 16 pair terms summed
// in FP32 and added to a double accumulator.
__device__ void sub_images(SubState &S, int lo, int n)
{
    const int t = threadIdx.x;
    if (t < n) {
        const int i = lo + t;
        split2(S.f[F_RX][i], S.g[0][i], S.g[4][i]);
        split2(S.f[F_RY][i], S.g[1][i], S.g[5][i]);
        split2(S.f[F_RZ][i], S.g[2][i], S.g[6][i]);
        S.g[3][i] = (float)S.f[F_M][i];
        S.g[7][i] = (float)S.f[F_E2][i];
        S.g[8][i] = (float)S.f[F_VX][i];
        S.g[9][i] = (float)S.f[F_VY][i];
        S.g[10][i] = (float)S.f[F_VZ][i];
    }
}

template <class Op>
__device__ typename Op::P sub_image(const SubState &S, int i)
{
    typename AccJerkS::P p = {S.g[0][i], S.g[1][i], S.g[2][i], S.g[3][i],
                              S.g[4][i], S.g[5][i], S.g[6][i], S.g[7][i],
                              S.g[8][i], S.g[9][i], S.g[10][i]};
    if constexpr (sizeof(typename Op::P) == sizeof(typename AccJerkS::P)) {
        return p;
    } else {
        return {p.xh, p.yh, p.zh, p.m, p.xl, p.yl, p.zl, p.e2};
    }
}

template <class Op>
__device__ void sub_split_sweep(SubState &S, int ilo, int ni, int jlo, int nj,
                                int first_out, double eta)
{
    sub_images(S, ilo, ni);
    sub_images(S, jlo, nj);
    __syncthreads();
    const int t = threadIdx.x;
    if (t == 0) S.interactions += (unsigned long long)ni * nj;
    if (t < ni) {
        const typename Op::P ip = sub_image<Op>(S, ilo + t);
        double v[Op::NO];
        float part[Op::NO];
#pragma unroll
        for (int c = 0; c < Op::NO; ++c) v[c] = 0.0;
        for (int j0 = 0; j0 < nj; j0 += 16) {
#pragma unroll
            for (int c = 0; c < Op::NO; ++c) part[c] = 0.f;
            const int je = j0 + 16 < nj ? j0 + 16 : nj;
            for (int j = j0; j < je; ++j)
                Op::pair(ip, sub_image<Op>(S, jlo + j), part, (float)eta);
#pragma unroll
            for (int c = 0; c < Op::NO; ++c)
                v[c] = c == Op::MAXC ? fmax(v[c], (double)part[c])
                                     : v[c] + (double)part[c];
        }
        Op::finish(v, eta);
#pragma unroll
        for (int c = 0; c < Op::NO; ++c) S.f[first_out + c][ilo + t] = v[c];
    }
    __syncthreads();
}

__device__ void sub_acc(SubState &S, int ilo, int ni, int jlo, int nj,
                        const SubParams &P, const Sweep &acc)
{
    if (P.split) sub_split_sweep<AccSN<false>>(S, ilo, ni, jlo, nj, F_AX, 0.0);
    else sub_sweep<AccPair<double>>(S, ilo, ni, jlo, nj, F_AX, acc);
}

__device__ void sub_drift(SubState &S, int lo, int n, double c)
{
    const int t = threadIdx.x;
    if (t < n) {
        const int i = lo + t;
        S.f[F_RX][i] = S.f[F_RX][i] + S.f[F_VX][i] * c;
        S.f[F_RY][i] = S.f[F_RY][i] + S.f[F_VY][i] * c;
        S.f[F_RZ][i] = S.f[F_RZ][i] + S.f[F_VZ][i] * c;
    }
    __syncthreads();
}

__device__ void sub_kick(SubState &S, int lo, int n, double c)
{
    const int t = threadIdx.x;
    if (t < n) {
        const int i = lo + t;
        S.f[F_VX][i] = S.f[F_VX][i] + S.f[F_AX][i] * c;
        S.f[F_VY][i] = S.f[F_VY][i] + S.f[F_AY][i] * c;
        S.f[F_VZ][i] = S.f[F_VZ][i] + S.f[F_AZ][i] * c;
    }
    __syncthreads();
}

__device__ void sub_fewbody(SubState &S, int lo, int n, double tau,
                            const SubParams &P, unsigned *err)
{
    if (n == 1) {
        sub_drift(S, lo, 1, tau);
        return;
    }
    if (n == 2) {
        if (threadIdx.x == 0) {
            double a[8], b[8], a1[6], b1[6];
            for (int k = 0; k < 8; ++k) {
                a[k] = S.f[k][lo];
                b[k] = S.f[k][lo + 1];
            }
            KepCtx<double> ctx = {0, P.budget, 0, false, false, 0.0};
            kepler_two_body(a, b, tau, a1, b1, ctx);
            const int outs[6] = {F_RX, F_RY, F_RZ, F_VX, F_VY, F_VZ};
            for (int q = 0; q < 6; ++q) {
                S.f[outs[q]][lo] = a1[q];
                S.f[outs[q]][lo + 1] = b1[q];
            }
            S.n_kepler += 1;
            if (ctx.exhausted) atomicOr(err, (unsigned)DERR_KEPLER_BUDGET);
        }
        __syncthreads();
    }
}

// SIAnn.dkd / SIAnn.kdk on [lo, lo + n).
__device__ void sub_evolve(SubState &S, int lo, int n, double tau,
                           const SubParams &P, const Sweep &acc,
                           unsigned *err)
{
    if (n <= 2) {
        sub_fewbody(S, lo, n, tau, P, err);
        return;
    }
    for (int k = 0; k < P.seq_len; ++k) {
        const double c = P.coef[k] * tau;
        if ((P.outer[k] != 0) != (P.kdk != 0)) {
            sub_drift(S, lo, n, c);
        } else {
            sub_acc(S, lo, n, lo, n, P, acc);
            sub_kick(S, lo, n, c);
        }
    }
}

// Entry half of SIA.recurse: Tstep, shared-step quantisation, split; pushes
// the frame (nothing for an empty subsystem).
__device__ void sub_enter(SubState &S, int lo, int n, double tau,
                          const SubParams &P, const Sweep &tst)
{
    if (n == 0) return;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) {
        S.n_recurse += 1;
        if (S.sp >= SUB_DEPTH) S.status = 1;
        if (S.sp + 1 > S.max_depth) S.max_depth = S.sp + 1;
        S.tau = tau;
    }
    __syncthreads();
    if (S.status) return;
    double flag = -1.0;
    if (P.mode != 's') {
        flag = 1.0;
        if (P.split)
            sub_split_sweep<TstepSN<false>>(S, lo, n, lo, n, F_TSTEP, P.eta);
        else
            sub_sweep<TstepPair<double>>(S, lo, n, lo, n, F_TSTEP, tst);
        if (P.mode == 'a') {
            double v = t < n ? fabs(S.f[F_TSTEP][lo + t]) : INFINITY;
            for (int o = 16; o > 0; o >>= 1)
                v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
            if (lane == 0) S.red[w] = v;
            __syncthreads();
            if (t == 0) {
                double m = S.red[0];
                for (int q = 1; q < SUB_MAX / 32; ++q) m = fmin(m, S.red[q]);
                S.tau = d_block_tstep(m, S.t_curr, tau);
            }
            __syncthreads();
        }
    }
    const double tq = S.tau;
    const double thr = flag * fabs(tq);
    int ns = n;
    if (n > 2 && !(flag < 0 && thr < 0)) {
        const bool slow = t < n && fabs(S.f[F_TSTEP][lo + t]) > thr;
        const unsigned b = __ballot_sync(0xffffffffu, slow);
        if (lane == 0) S.wc[w] = __popc(b);
        __syncthreads();
        unsigned before = 0, total = 0;
        for (int q = 0; q < SUB_MAX / 32; ++q) {
            before += q < w ? S.wc[q] : 0;
            total += S.wc[q];
        }
        const unsigned rs = before + __popc(b & ((1u << lane) - 1u));
        if (t < n) {
            const int dst = slow ? (int)rs : (int)total + (t - (int)rs);
#pragma unroll
            for (int f = 0; f < NFIELD; ++f) S.x[f][dst] = S.f[f][lo + t];
        }
        __syncthreads();
        if (t < n)
#pragma unroll
            for (int f = 0; f < NFIELD; ++f) S.f[f][lo + t] = S.x[f][t];
        ns = (int)total;
        if (t == 0) S.n_partitions += 1;
    }
    if (t == 0) {
        Frame &fr = S.stk[S.sp];
        fr.lo = lo;
        fr.n = n;
        fr.ns = ns;
        fr.step = 0;
        fr.sub = 0;
        fr.tau = tq;
        S.sp += 1;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(SUB_MAX)
k_sia_subtree(Fields F, uint64_t base, int n0, double tau0, SubParams P,
              SubCtl *ctl, unsigned *err)
{
    __shared__ SubState S;
    const int t = threadIdx.x;
    if (t < n0)
        for (int f = 0; f < NFIELD; ++f) S.f[f][t] = F.f[f][base + t];
    if (t == 0) {
        S.sp = 0;
        S.t_curr = ctl->t_curr;
        S.status = 0;
        S.max_depth = 0;
        S.n_recurse = S.n_kepler = S.n_partitions = 0;
        S.interactions = 0;
    }
    __syncthreads();
    Sweep acc, tst;
    memset(&acc, 0, sizeof(acc));
    memset(&tst, 0, sizeof(tst));
    acc.kernel = K_ACC;
    tst.kernel = K_TSTEP;
    tst.scal[0] = P.eta;

    sub_enter(S, 0, n0, tau0, P, tst);
    while (S.sp > 0 && S.status == 0) {
        const Frame fr = S.stk[S.sp - 1];
        const int nf = fr.n - fr.ns;
        __syncthreads();
        if (fr.step == P.seq_len) {
            // exit half of SIA.recurse (sia.py:1112-1123)
            if (t < fr.ns) {
                const int i = fr.lo + t;
                S.f[F_TSTEP][i] = fr.tau;
                S.f[F_TIME][i] = S.f[F_TIME][i] + fr.tau;
                ((long long *)S.f[F_NSTEP])[i] += 1;
            }
            if (t == 0) {
                if (nf == 0) S.t_curr += fr.tau;
                S.sp -= 1;
            }
            __syncthreads();
            continue;
        }
        const double c = P.coef[fr.step] * fr.tau;
        if (P.outer[fr.step]) {
            if (fr.sub == 0) {
                // sf_drift: evolve the slow part, then recurse into the fast
                sub_evolve(S, fr.lo, fr.ns, c, P, acc, err);
                if (t == 0) S.stk[S.sp - 1].sub = 1;
                __syncthreads();
                sub_enter(S, fr.lo + fr.ns, nf, c, P, tst);
                continue;
            }
            if (t == 0) {
                S.stk[S.sp - 1].sub = 0;
                S.stk[S.sp - 1].step += 1;
            }
            __syncthreads();
            continue;
        }
        // sf_kick (sia.py:199-297, Newtonian branch)
        if (fr.ns && nf) {
            sub_acc(S, fr.lo, fr.ns, fr.lo + fr.ns, nf, P, acc);
            sub_acc(S, fr.lo + fr.ns, nf, fr.lo, fr.ns, P, acc);
            sub_kick(S, fr.lo, fr.ns, c);
            sub_kick(S, fr.lo + fr.ns, nf, c);
        }
        if (t == 0) S.stk[S.sp - 1].step += 1;
        __syncthreads();
    }
    __syncthreads();
    if (t < n0)
        for (int f = 0; f < NFIELD; ++f) F.f[f][base + t] = S.f[f][t];
    if (t == 0) {
        ctl->t_curr = S.t_curr;
        ctl->status = S.status;
        ctl->max_depth = S.max_depth;
        ctl->n_recurse = S.n_recurse;
        ctl->n_kepler = S.n_kepler;
        ctl->n_partitions = S.n_partitions;
        ctl->interactions = S.interactions;
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct Sia {
    uint64_t n = 0;
    int sweep_mode = MODE_EXACT;
    char mode = 'h';          // 's' shared fixed, 'a' shared adaptive, 'h'
    bool kdk = false;
    double eta = 0.0;
    double t_curr = 0.0;
    long long steps = 0;
    std::vector<std::pair<bool, double>> seq;
    cudaStream_t stream = nullptr;
    double *pool = nullptr;
    Fields F, S;
    unsigned long long *word = nullptr;     // partition count / min bits
    unsigned *err = nullptr;
    void *pack = nullptr;
    double *partial = nullptr;
    int sms = 152;
    long long kepler_budget = 1LL << 20;
    // subsystems of at most sub_max particles run as one CTA (0: never)
    int sub_max = SUB_MAX;
    SubParams P;
    SubCtl *ctl_dev = nullptr, *ctl_host = nullptr;
    // statistics
    long long n_recurse = 0, n_kepler = 0, n_sweeps = 0, n_partitions = 0;
    long long n_subtrees = 0;
    unsigned long long interactions = 0;   // sum of ni * nj over all sums
    double subtree_s = 0.0;      // wall time inside subtree launches
    int max_depth = 0;
};

constexpr int MAX_DEPTH = 512;

unsigned grid_for(const Sia *S, uint64_t n)
{
    uint64_t b = (n + 255) / 256;
    const uint64_t cap = (uint64_t)S->sms * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// i-range [ilo, ilo+ni) against j-range [jlo, jlo+nj): acc or tstep.
cudaError_t sweep(Sia *S, int kernel, uint64_t ilo, uint64_t ni, uint64_t jlo,
                  uint64_t nj)
{
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = kernel;
    s.mode = S->sweep_mode;
    s.ni = ni;
    s.nj = nj;
    for (int a = 0; a < n_attr(kernel); ++a) {
        s.ip[a] = S->F.f[a] + ilo;
        s.jp[a] = S->F.f[a] + jlo;
    }
    const int first_out = kernel == K_TSTEP ? F_TSTEP : F_AX;
    for (int o = 0; o < n_out(kernel); ++o)
        s.out[o] = S->F.f[first_out + o] + ilo;
    s.scal[0] = kernel == K_TSTEP ? S->eta : 0.0;
    S->n_sweeps += 1;
    S->interactions += (unsigned long long)ni * nj;
    if (S->sweep_mode == MODE_EXACT)
        return launch_exact<double>(s, S->stream, S->kepler_budget, S->err);
    const int nf = split_nf_host(kernel);
    float4 *irec = (float4 *)S->pack;
    float4 *jrec = irec + ni * nf;
    cudaError_t e = launch_pack(kernel, ni, s.ip, irec, S->stream);
    if (e == cudaSuccess) e = launch_pack(kernel, nj, s.jp, jrec, S->stream);
    if (e != cudaSuccess) return e;
    int variant, gsplit;
    choose_split_public(kernel, ni, nj, &variant, &gsplit);
    return launch_split(kernel, irec, jrec, ni, nj, s.out, S->partial, variant,
                        gsplit, s.scal[0], S->err, S->stream);
}

cudaError_t drift(Sia *S, uint64_t lo, uint64_t n, double c)
{
    k_drift<<<grid_for(S, n), 256, 0, S->stream>>>(S->F, lo, n, c);
    g_launch_count += 1;
    return cudaGetLastError();
}

cudaError_t kick_n(Sia *S, uint64_t lo, uint64_t n, double c)
{
    k_kick<<<grid_for(S, n), 256, 0, S->stream>>>(S->F, lo, n, c);
    g_launch_count += 1;
    return cudaGetLastError();
}

// FewBody.evolve (tupan/integrator/fewbody.py:43-60).
cudaError_t fewbody(Sia *S, uint64_t lo, uint64_t n, double tau)
{
    if (n == 0) return cudaSuccess;
    if (n == 1) return drift(S, lo, 1, tau);
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = K_KEPLER;
    s.mode = MODE_EXACT;
    s.ni = s.nj = 2;
    for (int a = 0; a < 8; ++a) s.ip[a] = s.jp[a] = S->F.f[a] + lo;
    const int outs[6] = {F_RX, F_RY, F_RZ, F_VX, F_VY, F_VZ};
    for (int o = 0; o < 6; ++o) s.out[o] = S->F.f[outs[o]] + lo;
    s.scal[0] = tau;
    S->n_kepler += 1;
    return launch_exact<double>(s, S->stream, S->kepler_budget, S->err);
}

// SIAnn.dkd / SIAnn.kdk on one subsystem.
cudaError_t evolve_sub(Sia *S, uint64_t lo, uint64_t n, double tau)
{
    if (n <= 2) return fewbody(S, lo, n, tau);
    for (const auto &op : S->seq) {
        const bool is_drift = op.first != S->kdk;
        cudaError_t e;
        if (is_drift) {
            e = drift(S, lo, n, op.second * tau);
        } else {
            // kick (sia.py:173-182): the subsystem's own acceleration first
            e = sweep(S, K_ACC, lo, n, lo, n);
            if (e == cudaSuccess) e = kick_n(S, lo, n, op.second * tau);
        }
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int recurse(Sia *S, uint64_t lo, uint64_t n, double tau, int depth);

// SIAnn.bridge_sf: sf_drift for the outer coefficients, sf_kick (sia.py:
// 199-297, Newtonian branch) for the inner ones.
int bridge(Sia *S, uint64_t lo, uint64_t ns, uint64_t nf, double tau,
           int depth)
{
    for (const auto &op : S->seq) {
        const double c = op.second * tau;
        if (op.first) {
            if (evolve_sub(S, lo, ns, c) != cudaSuccess) return ST_CUDA;
            const int rc = recurse(S, lo + ns, nf, c, depth + 1);
            if (rc) return rc;
        } else if (ns && nf) {
            if (sweep(S, K_ACC, lo, ns, lo + ns, nf) != cudaSuccess ||
                sweep(S, K_ACC, lo + ns, nf, lo, ns) != cudaSuccess ||
                kick_n(S, lo, ns, c) != cudaSuccess ||
                kick_n(S, lo + ns, nf, c) != cudaSuccess)
                return ST_CUDA;
        }
    }
    return ST_OK;
}

double block_tstep(double min_ts, double t, double tau)
{
    // tupan/integrator/__init__.py:59-78
    long long power = (long long)(log2(min_ts) - 1.0);
    double min_bts = ldexp(1.0, (int)power);
    const double t_next = t + min_bts;
    for (int k = 0; k < 2100 && fmod(t_next, min_bts) != 0.0; ++k)
        min_bts /= 2.0;
    min_bts = copysign(min_bts, tau);
    if (fabs(min_bts) > fabs(tau)) min_bts = tau;
    return min_bts;
}

int read_word(Sia *S, unsigned long long *out)
{
    if (cudaMemcpyAsync(out, S->word, sizeof(*out), cudaMemcpyDeviceToHost,
                        S->stream) != cudaSuccess ||
        cudaStreamSynchronize(S->stream) != cudaSuccess)
        return ST_CUDA;
    return ST_OK;
}

// The whole of SIA.recurse on [lo, lo + n) in one CTA (n <= SUB_MAX).
int subtree(Sia *S, uint64_t lo, uint64_t n, double tau, int depth)
{
    const auto t0 = std::chrono::steady_clock::now();
    SubCtl *h = S->ctl_host;
    memset(h, 0, sizeof(*h));
    h->t_curr = S->t_curr;
    if (cudaMemcpyAsync(S->ctl_dev, h, sizeof(*h), cudaMemcpyHostToDevice,
                        S->stream) != cudaSuccess)
        return ST_CUDA;
    k_sia_subtree<<<1, SUB_MAX, 0, S->stream>>>(S->F, lo, (int)n, tau, S->P,
                                                S->ctl_dev, S->err);
    g_launch_count += 1;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(h, S->ctl_dev, sizeof(*h), cudaMemcpyDeviceToHost,
                        S->stream) != cudaSuccess ||
        cudaStreamSynchronize(S->stream) != cudaSuccess)
        return ST_CUDA;
    S->subtree_s += std::chrono::duration<double>(
                        std::chrono::steady_clock::now() - t0).count();
    S->n_subtrees += 1;
    S->t_curr = h->t_curr;
    S->n_recurse += h->n_recurse;
    S->n_kepler += h->n_kepler;
    S->n_partitions += h->n_partitions;
    S->interactions += h->interactions;
    if (depth + h->max_depth - 1 > S->max_depth)
        S->max_depth = depth + h->max_depth - 1;
    return h->status ? ST_TOO_LARGE : ST_OK;
}

// SIA.recurse (sia.py:1097-1123) on the subsystem [lo, lo + n).
int recurse(Sia *S, uint64_t lo, uint64_t n, double tau, int depth)
{
    if (n == 0) return ST_OK;
    if (depth > MAX_DEPTH) return ST_TOO_LARGE;
    if (n <= (uint64_t)S->sub_max) return subtree(S, lo, n, tau, depth);
    S->n_recurse += 1;
    if (depth > S->max_depth) S->max_depth = depth;
    double flag = -1.0;
    if (S->mode != 's') {
        flag = 1.0;
        if (sweep(S, K_TSTEP, lo, n, lo, n) != cudaSuccess) return ST_CUDA;
        if (S->mode == 'a') {
            cudaMemsetAsync(S->word, 0xff, sizeof(unsigned long long),
                            S->stream);
            k_min_abs<<<grid_for(S, n), 256, 0, S->stream>>>(
                S->F.f[F_TSTEP] + lo, n, S->word);
            g_launch_count += 1;
            unsigned long long bits;
            if (read_word(S, &bits)) return ST_CUDA;
            double min_ts;
            memcpy(&min_ts, &bits, sizeof(min_ts));
            tau = block_tstep(min_ts, S->t_curr, tau);
        }
    }
    uint64_t ns = n;
    const double thr = flag * fabs(tau);
    // split (sia.py:22-39): at most two particles, or a threshold below
    // every |tstep| (fixed shared steps), leave the subsystem whole.
    if (n > 2 && !(flag < 0 && thr < 0)) {
        k_partition<<<1, PART_THREADS, 0, S->stream>>>(S->F, S->S, lo, n, thr,
                                                        S->word);
        g_launch_count += 1;
        S->n_partitions += 1;
        unsigned long long cnt;
        if (read_word(S, &cnt)) return ST_CUDA;
        ns = cnt;
    }
    const uint64_t nf = n - ns;
    int rc = bridge(S, lo, ns, nf, tau, depth);
    if (rc) return rc;
    if (nf == 0) S->t_curr += tau;
    if (ns) {
        k_book<<<grid_for(S, ns), 256, 0, S->stream>>>(S->F, lo, ns, tau);
        g_launch_count += 1;
    }
    return cudaGetLastError() == cudaSuccess ? ST_OK : ST_CUDA;
}

double base_tstep(double t, double t_end, double eta)
{
    // tupan/integrator/__init__.py:48-57
    double dt = fmin(fabs(t_end) - fabs(t), fabs(eta));
    dt = fmax(dt, fabs(t_end) * (2 * DBL_EPSILON));
    return copysign(dt, eta);
}

void release(Sia *S)
{
    if (S->stream) cudaStreamSynchronize(S->stream);
    cudaFree(S->pool);
    cudaFree(S->word);
    cudaFree(S->err);
    cudaFree(S->pack);
    cudaFree(S->partial);
    cudaFree(S->ctl_dev);
    cudaFreeHost(S->ctl_host);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
}

}  // namespace

// ===========================================================================
// C-ABI (no counterpart in the reference, which runs SIA on host arrays).
// ===========================================================================

// method: "sia21s.dkd" .. "sia69h.kdk" (the 48 names of sia.py:969-985);
// mode 0 EXACT, 1 SPLIT force sweeps.  Host arrays are copied in.
TG_EXPORT int tupan_gb300_sia_create(uint64_t n, const char *method, double eta,
                                     int mode, const double *m,
                                     const double *e2, const double *rx,
                                     const double *ry, const double *rz,
                                     const double *vx, const double *vy,
                                     const double *vz, void **handle)
{
    if (!handle || !method || n == 0 || (mode != MODE_EXACT && mode != MODE_SPLIT))
        return ST_BAD_ARGUMENT;
    if (strlen(method) != 10 || method[6] != '.') return ST_BAD_ARGUMENT;
    const Scheme *sc = nullptr;
    for (const Scheme &s : kSchemes)
        if (strncmp(method, s.name, 5) == 0) sc = &s;
    const char md = method[5];
    const bool kdk = strcmp(method + 7, "kdk") == 0;
    if (!sc || (md != 's' && md != 'a' && md != 'h') ||
        (!kdk && strcmp(method + 7, "dkd") != 0))
        return ST_BAD_ARGUMENT;
    Sia *S = new Sia();
    S->n = n;
    S->sweep_mode = mode;
    S->mode = md;
    S->kdk = kdk;
    S->eta = eta;
    S->seq = make_sequence(*sc);
    memset(&S->P, 0, sizeof(S->P));
    S->P.seq_len = (int)S->seq.size();
    for (int k = 0; k < S->P.seq_len && k < SEQ_MAX; ++k) {
        S->P.outer[k] = S->seq[k].first ? 1 : 0;
        S->P.coef[k] = S->seq[k].second;
    }
    S->P.mode = md;
    S->P.kdk = kdk ? 1 : 0;
    S->P.split = mode == MODE_SPLIT ? 1 : 0;
    S->P.eta = eta;
    S->P.budget = S->kepler_budget;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t fb = n * sizeof(double);
    bool ok =
        cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) == cudaSuccess &&
        cudaMalloc((void **)&S->pool, 2 * NFIELD * fb) == cudaSuccess &&
        cudaMalloc((void **)&S->word, sizeof(unsigned long long)) == cudaSuccess &&
        cudaMalloc((void **)&S->err, sizeof(unsigned)) == cudaSuccess &&
        cudaMalloc((void **)&S->ctl_dev, sizeof(SubCtl)) == cudaSuccess &&
        cudaMallocHost((void **)&S->ctl_host, sizeof(SubCtl)) == cudaSuccess;
    if (ok && mode == MODE_SPLIT)
        ok = cudaMalloc(&S->pack, 2 * n * 3 * sizeof(float4) + 256) == cudaSuccess &&
             cudaMalloc((void **)&S->partial, 64 * 3 * fb) == cudaSuccess;
    if (!ok) {
        release(S);
        return ST_CUDA;
    }
    for (int f = 0; f < NFIELD; ++f) {
        S->F.f[f] = S->pool + (size_t)f * n;
        S->S.f[f] = S->pool + (size_t)(NFIELD + f) * n;
    }
    cudaMemsetAsync(S->pool, 0, NFIELD * fb, S->stream);
    cudaMemsetAsync(S->err, 0, sizeof(unsigned), S->stream);
    const double *src[8] = {m, rx, ry, rz, e2, vx, vy, vz};
    for (int f = 0; f < 8; ++f)
        ok = ok && cudaMemcpyAsync(S->F.f[f], src[f], fb, cudaMemcpyHostToDevice,
                                   S->stream) == cudaSuccess;
    std::vector<long long> ids(n);
    for (uint64_t i = 0; i < n; ++i) ids[i] = (long long)i;
    ok = ok && cudaMemcpyAsync(S->F.f[F_ID], ids.data(), fb,
                               cudaMemcpyHostToDevice, S->stream) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(S->stream) == cudaSuccess;
    if (!ok) {
        release(S);
        return ST_CUDA;
    }
    *handle = S;
    return ST_OK;
}

// Base steps (Base.evolve_step + SIA.do_step) until |t| >= t_end or
// max_steps (0: no limit) were taken.  t_log (host, may be NULL) receives
// the time after each step, at most log_cap entries.  Status 3: a Kepler
// solve used up its budget; 5: the recursion went deeper than 512 levels.
TG_EXPORT int tupan_gb300_sia_evolve(void *handle, double t_end,
                                     long long max_steps, double *t_out,
                                     long long *steps_out, double *t_log,
                                     long long log_cap)
{
    Sia *S = (Sia *)handle;
    if (!S) return ST_BAD_ARGUMENT;
    long long taken = 0;
    while (fabs(S->t_curr) < t_end && (max_steps <= 0 || taken < max_steps)) {
        const double tau = base_tstep(S->t_curr, t_end, S->eta);
        const int rc = recurse(S, 0, S->n, tau, 0);
        if (rc) return rc;
        if (t_log && taken < log_cap) t_log[taken] = S->t_curr;
        taken += 1;
        S->steps += 1;
    }
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, S->err, sizeof(h), cudaMemcpyDeviceToHost,
                        S->stream) != cudaSuccess ||
        cudaStreamSynchronize(S->stream) != cudaSuccess)
        return ST_CUDA;
    if (t_out) *t_out = S->t_curr;
    if (steps_out) *steps_out = taken;
    return h ? ST_DEVICE : ST_OK;
}

// State in the current particle order (the reference's order after its
// joins): id, positions, velocities, time, nstep, tstep; any may be NULL.
TG_EXPORT int tupan_gb300_sia_get_state(void *handle, long long *id,
                                        double *rx, double *ry, double *rz,
                                        double *vx, double *vy, double *vz,
                                        double *time, long long *nstep,
                                        double *tstep)
{
    Sia *S = (Sia *)handle;
    if (!S) return ST_BAD_ARGUMENT;
    void *dst[10] = {id, rx, ry, rz, vx, vy, vz, time, nstep, tstep};
    const int src[10] = {F_ID, F_RX, F_RY, F_RZ, F_VX, F_VY, F_VZ, F_TIME,
                         F_NSTEP, F_TSTEP};
    for (int q = 0; q < 10; ++q)
        if (dst[q] && cudaMemcpyAsync(dst[q], S->F.f[src[q]],
                                      S->n * sizeof(double),
                                      cudaMemcpyDeviceToHost,
                                      S->stream) != cudaSuccess)
            return ST_CUDA;
    return cudaStreamSynchronize(S->stream) == cudaSuccess ? ST_OK : ST_CUDA;
}

// Counters since creation: stats[0] recursion calls, [1] Kepler solves,
// [2] force/tstep sweeps launched from the host, [3] partitions, [4]
// deepest level, [5] base steps, [6] single-CTA subtree launches, [7]
// microseconds spent in them, [8] pair interactions summed (ni * nj of
// every Acc and Tstep sum).
TG_EXPORT int tupan_gb300_sia_stats(void *handle, long long *stats)
{
    Sia *S = (Sia *)handle;
    if (!S || !stats) return ST_BAD_ARGUMENT;
    stats[0] = S->n_recurse;
    stats[1] = S->n_kepler;
    stats[2] = S->n_sweeps;
    stats[3] = S->n_partitions;
    stats[4] = S->max_depth;
    stats[5] = S->steps;
    stats[6] = S->n_subtrees;
    stats[7] = (long long)(S->subtree_s * 1e6);
    stats[8] = (long long)S->interactions;
    return ST_OK;
}

// Largest subsystem handed whole to the single-CTA recursion kernel
// (0 .. 128; 0: every level driven from the host).  Both paths give the
// same bits.  Returns the previous value, or -1 for a bad argument.
TG_EXPORT int tupan_gb300_sia_set_subtree(void *handle, int max_n)
{
    Sia *S = (Sia *)handle;
    if (!S || max_n < 0 || max_n > SUB_MAX) return -1;
    const int old = S->sub_max;
    S->sub_max = max_n;
    return old;
}

TG_EXPORT int tupan_gb300_sia_destroy(void *handle)
{
    Sia *S = (Sia *)handle;
    if (!S) return ST_BAD_ARGUMENT;
    release(S);
    return ST_OK;
}
