// A SPLIT-mode acc_jerk sweep that allocates nothing.
//
// Some callers cannot let this library call cudaMalloc: an application whose
// own memory manager reserves the whole device heap up front (a large
// simulation framework hosting tupan's kernels as a plugin), and time-step
// loops that must not pay cudaMalloc's implicit device-wide synchronisation
// in the middle of a run.  They give their own device buffers for inputs and
// outputs; the scratch this sweep needs -- the packed FP32 particle records --
// lives in a fixed static device array declared below.
//
// Limits: at most TG_NOALLOC_MAX_N i-particles and TG_NOALLOC_MAX_N
// j-particles per call.  The static arrays take 12 MiB of device memory (6 MiB
// of packed records, 6 MiB of grid j-split partial sums), held by every GPU
// that loads this library until the process exits.  Larger requests are
// rejected with ST_TOO_LARGE before anything is launched.
//
// The arrays are shared by all calls and keep the previous call's contents:
// the error word is cleared at the start of each call, the records are
// rewritten for the particles of the call, and every partial sum that is
// read was written by the same call.  Calls whose work overlaps on the GPU
// (different streams, or threads calling concurrently) race on the arrays.
//
// The first call on a device looks up the arrays' device addresses there
// (host code cannot use an array's name as a device pointer); make that
// first call outside any stream capture.

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>

#include "tg_common.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace tg {
cudaError_t launch_pack(int kernel, uint64_t n, const void *const *attrs,
                        float4 *out, cudaStream_t st);
cudaError_t launch_split(int kernel, const float4 *irec, const float4 *jrec,
                         uint64_t ni, uint64_t nj, void *const *out,
                         double *partial, int variant, int gsplit, double eta,
                         unsigned *err, cudaStream_t st);
int split_variant_count();
void split_variant_info(int v, int *ni_per_thread, int *jsplit, int *threads);
}  // namespace tg

using namespace tg;

#define TG_NOALLOC_MAX_N 65536
#define TG_NOALLOC_REC 3   // float4 per acc_jerk record
// grid j-split partial sums: gsplit x 6 outputs x ni doubles, gsplit x ni at
// most this many (so small i-sets can be spread over the whole GPU)
#define TG_NOALLOC_PARTIAL_IN (2 * TG_NOALLOC_MAX_N)

namespace {

// Packed i-records followed by packed j-records, and the error word.
static __device__ __align__(256) float4
    g_noalloc_records[2 * TG_NOALLOC_MAX_N * TG_NOALLOC_REC];
static __device__ __align__(256) double
    g_noalloc_partial[(size_t)TG_NOALLOC_PARTIAL_IN * 6];
static __device__ __align__(256) unsigned g_noalloc_err;

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
float4 *g_records_ptr[MAX_DEVICES];
double *g_partial_ptr[MAX_DEVICES];
unsigned *g_err_ptr[MAX_DEVICES];
int g_sms[MAX_DEVICES];
bool g_ready[MAX_DEVICES];

// Once per device, with that device current: the device addresses of the
// static arrays and the SM count.  Nothing here allocates.  A failure is
// described in msg (the caller's buffer).
int setup_device(int *dev_out, char *msg, size_t cap)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        snprintf(msg, cap, "no usable CUDA device");
        return ST_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_ready[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_records);
        if (e != cudaSuccess) {
            snprintf(msg, cap, "cudaGetSymbolAddress(records): %s",
                     cudaGetErrorString(e));
            return ST_CUDA;
        }
        g_records_ptr[dev] = (float4 *)p;
        e = cudaGetSymbolAddress(&p, g_noalloc_partial);
        if (e != cudaSuccess) {
            snprintf(msg, cap, "cudaGetSymbolAddress(partials): %s",
                     cudaGetErrorString(e));
            return ST_CUDA;
        }
        g_partial_ptr[dev] = (double *)p;
        e = cudaGetSymbolAddress(&p, g_noalloc_err);
        if (e != cudaSuccess) {
            snprintf(msg, cap, "cudaGetSymbolAddress(error): %s",
                     cudaGetErrorString(e));
            return ST_CUDA;
        }
        g_err_ptr[dev] = (unsigned *)p;
        e = cudaDeviceGetAttribute(&g_sms[dev],
                                   cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) {
            snprintf(msg, cap, "cudaDeviceGetAttribute: %s",
                     cudaGetErrorString(e));
            return ST_CUDA;
        }
        g_ready[dev] = true;
    }
    *dev_out = dev;
    return ST_OK;
}

// Launch shape: the packed sweep without the Newton step (variant 9, two i
// per thread, the library's default for large split sweeps) and the grid
// j-split whose waves x j per CTA is smallest, within the partial-sum array.
constexpr int NOALLOC_VARIANT = 9;

int pick_gsplit(uint64_t ni, uint64_t nj, int sms)
{
    int nip, js, nt;
    split_variant_info(NOALLOC_VARIANT, &nip, &js, &nt);
    const double ipc = (double)(nt / js) * nip;
    const double gx = ceil((double)ni / ipc);
    const double cap = (double)sms * 2;          // two 256-thread CTAs per SM
    const uint64_t tiles = (nj + 255) / 256;
    int best_g = 1;
    double best = 1e300;
    for (int g = 1; g <= 64; g *= 2) {
        if (g > 1 && ((uint64_t)g > tiles ||
                      (uint64_t)g * ni > TG_NOALLOC_PARTIAL_IN))
            break;
        const double t = ceil(gx * g / cap) * ((double)nj / g) +
                         (g > 1 ? 0.02 * (double)nj / g : 0.0);
        if (t < best * 0.999) {
            best = t;
            best_g = g;
        }
    }
    return best_g;
}

}  // namespace

// acc_jerk_kernel's sum in SPLIT arithmetic on DEVICE arrays, with the
// i-set's eight inputs (m, rx, ry, rz, e2, vx, vy, vz), then nj and the
// j-set's eight, then the six outputs (ax, ay, az, jx, jy, jz), on `stream`
// (NULL: the default stream), with no allocation.  Returns 0, ST_TOO_LARGE
// (5) for ni or nj above 65536 (nothing launched), ST_NO_DEVICE (4),
// ST_CUDA (1) or ST_DEVICE (3); failures are also printed on stderr.
// With err_out == NULL the call is asynchronous and reports no device error
// (the next call clears the error word).  With a host pointer err_out, the
// call waits for the stream, stores the sweep's device error word there
// (0: the outputs are complete; non-zero: see DeviceError) and returns
// ST_DEVICE when it is non-zero.
TG_EXPORT int tupan_gb300_acc_jerk_split_noalloc(
    uint64_t ni, const double *im, const double *irx, const double *iry,
    const double *irz, const double *ie2, const double *ivx,
    const double *ivy, const double *ivz, uint64_t nj, const double *jm,
    const double *jrx, const double *jry, const double *jrz,
    const double *je2, const double *jvx, const double *jvy,
    const double *jvz, double *iax, double *iay, double *iaz, double *ijx,
    double *ijy, double *ijz, void *stream, unsigned *err_out)
{
    if (ni > TG_NOALLOC_MAX_N || nj > TG_NOALLOC_MAX_N) {
        fprintf(stderr,
                "tupan_gb300: acc_jerk_split_noalloc: ni=%llu nj=%llu, at most "
                "%d i- and %d j-particles\n",
                (unsigned long long)ni, (unsigned long long)nj,
                TG_NOALLOC_MAX_N, TG_NOALLOC_MAX_N);
        return ST_TOO_LARGE;
    }
    if (err_out) *err_out = 0;
    if (ni == 0) return ST_OK;
    int dev;
    char msg[256];
    int rc = setup_device(&dev, msg, sizeof(msg));
    if (rc) {
        fprintf(stderr, "tupan_gb300: acc_jerk_split_noalloc: %s\n", msg);
        return rc;
    }
    cudaStream_t st = (cudaStream_t)stream;
    float4 *irec = g_records_ptr[dev];
    float4 *jrec = irec + (size_t)TG_NOALLOC_MAX_N * TG_NOALLOC_REC;
    const void *ia[8] = {im, irx, iry, irz, ie2, ivx, ivy, ivz};
    const void *ja[8] = {jm, jrx, jry, jrz, je2, jvx, jvy, jvz};
    void *out[6] = {iax, iay, iaz, ijx, ijy, ijz};
    const int gsplit = pick_gsplit(ni, nj, g_sms[dev]);
    cudaError_t e = cudaMemsetAsync(g_err_ptr[dev], 0, sizeof(unsigned), st);
    if (e == cudaSuccess) e = launch_pack(K_ACC_JERK, ni, ia, irec, st);
    if (e == cudaSuccess) e = launch_pack(K_ACC_JERK, nj, ja, jrec, st);
    if (e == cudaSuccess)
        e = launch_split(K_ACC_JERK, irec, jrec, ni, nj, out,
                         g_partial_ptr[dev], NOALLOC_VARIANT, gsplit, 0.0,
                         g_err_ptr[dev], st);
    if (e == cudaSuccess && err_out) {
        e = cudaMemcpyAsync(err_out, g_err_ptr[dev], sizeof(unsigned),
                            cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        fprintf(stderr, "tupan_gb300: acc_jerk_split_noalloc: %s\n",
                cudaGetErrorString(e));
        return ST_CUDA;
    }
    if (err_out && *err_out) {
        fprintf(stderr, "tupan_gb300: acc_jerk_split_noalloc: device error "
                        "word 0x%x\n", *err_out);
        return ST_DEVICE;
    }
    return ST_OK;
}
