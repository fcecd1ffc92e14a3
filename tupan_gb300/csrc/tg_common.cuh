// Shared declarations of the GB300 tupan kernel layer.
//
// Kernel identities, the attribute layout each kernel reads, the launch
// descriptor passed from the C-ABI layer to the kernel translation units and
// the device-side error word.  Host code above this file is the C-ABI in
// abi.cu; nothing here depends on PyTorch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace tg {

// Kernels launched by this library since load (defined in abi.cu).
extern std::atomic<unsigned long long> g_launch_count;

// Tries a sweep's main-loop pipeline wait makes before it reports
// DERR_PIPE_TIMEOUT (defined in abi.cu; tupan_gb300_set_pipe_spin_limit).
uint32_t pipe_spin_limit();
// Reach of the centred sweep's mid tiles, in tile radii.
float centred_mid_reach();

// int(log2(min_ts) - 1), the exponent of tupan's power-of-two step
// (integrator/__init__.py:59-78), as numpy evaluates it with a correctly
// rounded log2.  min_ts = m 2^e exactly (frexp, m in [0.5, 1)); the
// logarithm is taken of whichever of m and 2m lies in [sqrt(1/2), sqrt(2)),
// so near a power of two, where the truncation is decided, it is a value
// near zero whose absolute error is negligible, and the integer part joins
// it in one rounding.  The device log2 of min_ts itself is one ulp off at
// exact powers of two, which the truncation turns into a step twice as
// long.
__device__ __forceinline__ long long quantised_power(double min_ts)
{
    int e;
    const double m = frexp(min_ts, &e);
    const double l = m < 0.70710678118654752
                         ? (double)(e - 1) + log2(2.0 * m)
                         : (double)e + log2(m);
    return (long long)(l - 1.0);
}


// The ten entry points of tupan/lib/src/libtupan.h:2-246.
enum KernelId : int {
    K_PHI = 0,
    K_ACC = 1,
    K_ACC_JERK = 2,
    K_SNAP_CRACKLE = 3,
    K_TSTEP = 4,
    K_PNACC = 5,
    K_NREG_X = 6,
    K_NREG_V = 7,
    K_SAKURA = 8,
    K_KEPLER = 9,
    K_COUNT = 10
};

// Arithmetic used for the pairwise sums.
enum Mode : int {
    MODE_EXACT = 0,   // REAL arithmetic in the reference's order: bit-identical
    MODE_SPLIT = 1    // FP32 pairs, double-single positions, compensated sums
};

// Error word written by kernels (bit flags) and read back by the host.
enum DeviceError : unsigned {
    DERR_NONE = 0,
    DERR_PIPE_TIMEOUT = 1u << 0,     // a bounded mbarrier wait ran out
    DERR_KEPLER_BUDGET = 1u << 1,    // a Kepler solve exhausted its budget
    DERR_BAD_LAUNCH = 1u << 2        // launch geometry inconsistent with data
};

// Host-visible status codes of the C-ABI (tupan_gb300_last_error()).
enum Status : int {
    ST_OK = 0,
    ST_CUDA = 1,            // a CUDA runtime call failed
    ST_BAD_ARGUMENT = 2,    // a size or pointer the entry point cannot take
    ST_DEVICE = 3,          // a kernel reported an error word
    ST_NO_DEVICE = 4,       // no CUDA device / library not usable
    ST_TOO_LARGE = 5        // request beyond a fixed maximum
};

constexpr int MAX_ATTR = 14;   // m r(3) e2 v(3) a(3) j(3)
constexpr int MAX_OUT = 7;

// Number of per-particle input attributes read by each kernel, in the
// order the ABI passes them (i side and j side alike).
__host__ __device__ constexpr int n_attr(int k)
{
    return k == K_PHI || k == K_ACC ? 5
         : k == K_SNAP_CRACKLE ? 14
         : k == K_NREG_V ? 7
         : 8;
}

__host__ __device__ constexpr int n_out(int k)
{
    return k == K_PHI ? 1
         : k == K_ACC || k == K_PNACC ? 3
         : k == K_TSTEP ? 2
         : k == K_NREG_X ? 7
         : k == K_NREG_V ? 4
         : 6;
}

// One pairwise sweep: outputs for ni i-particles summed over nj j-particles.
// Array pointers are DEVICE pointers of `real` (double or float) values.
struct Sweep {
    int kernel;
    int mode;
    uint64_t ni, nj;
    const void *ip[MAX_ATTR];
    const void *jp[MAX_ATTR];
    void *out[MAX_OUT];
    double scal[8];        // eta | dt | inv1..inv7 (scal[1..7]) for PN
    int64_t iscal;         // flag (Sakura) | order (PNAcc)
    // When set, the i count is read on the device from here when the sweep
    // runs (ni is then its upper bound, used for the launch shape): a sweep
    // over a set whose size the GPU decides, launched without a host sync.
    const unsigned *ni_dev;
};

// Launch configuration of the FP32-split sweep, chosen by the autotuner.
struct SplitConfig {
    int variant;     // index into the compiled variant table of the kernel
    int gsplit;      // j ranges handled by separate CTAs (partials reduced)
};

// Device workspace owned by the C-ABI layer (grown on demand).
struct Workspace {
    void *pack_i;        // packed FP32 i-records
    void *pack_j;        // packed FP32 j-records
    double *partial;     // gsplit x n_out x ni partial sums
    size_t pack_i_bytes, pack_j_bytes, partial_bytes;
    unsigned *err;       // device error word
};

// Frees a half-built object when a create entry point fails part way:
// construct right after `new`, call keep() once the object is complete.
struct CreateGuard {
    void *obj;
    int (*destroy)(void *);
    bool kept = false;
    void keep() { kept = true; }
    ~CreateGuard()
    {
        if (!kept && obj) destroy(obj);
    }
};

}  // namespace tg

#define TG_CUDA_TRY(expr)                                                   \
    do {                                                                    \
        cudaError_t e_ = (expr);                                            \
        if (e_ != cudaSuccess) return e_;                                   \
    } while (0)
