// C-ABI of the GB300 tupan kernel layer.
//
// Compiled twice: with TG_ABI_FLOAT64 it exports the float64 prototypes of
// tupan/lib/src/libtupan.h:2-246 (REAL=double, UINT=uint64, INT=int64) as
// libtupan_gb300.so; with TG_ABI_FLOAT32 the float32 ones (REAL=float,
// UINT=uint32, INT=int32) as libtupan_gb300_sp.so -- the two libraries
// tupan's cffi backend builds per precision (cffi_backend.py:84-87).
//
// The ten entry points take HOST arrays, copy them to the device, run the
// sweep and copy the results back before returning, like tupan's OpenCL
// backend does per call (opencl_backend.py:117-171).  They return void as in
// the reference; failures are reported through tupan_gb300_last_error().
// Extra entry points (tupan_gb300_*) select the arithmetic mode, expose a
// device-pointer sweep for callers that keep particles resident in HBM, and
// report errors.  No entry point falls back to the CPU.

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <initializer_list>
#include <mutex>
#include <unordered_map>

#include "tg_common.cuh"

#if defined(TG_ABI_FLOAT64)
typedef double REAL;
typedef uint64_t UINT;
typedef int64_t INT;
#define TG_PREC_SPLIT_OK 1
#elif defined(TG_ABI_FLOAT32)
typedef float REAL;
typedef uint32_t UINT;
typedef int32_t INT;
#define TG_PREC_SPLIT_OK 0
#else
#error "define TG_ABI_FLOAT64 or TG_ABI_FLOAT32"
#endif

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
cudaError_t launch_split_pn(int kernel, const float4 *irec,
                            const float4 *jrec, uint64_t ni, uint64_t nj,
                            void *const *out, double *partial, int variant,
                            int gsplit, double eta, const double *pn,
                            unsigned *err, cudaStream_t st);
int split_variant_count();
void split_variant_info(int v, int *ni_per_thread, int *jsplit, int *threads);
bool split_supported(int kernel);
bool split_has_x2(int kernel);
bool split_has_raw(int kernel);
int split_nf_host(int kernel);
bool centred_supported(int k);
int centred_shape_count();
int centred_choose_gsplit(uint64_t ni, uint64_t nj, int shape, int sms);
size_t centred_workspace_bytes(int k, uint64_t ni, uint64_t nj, bool same,
                               int gsplit);
cudaError_t launch_centred(int k, uint64_t ni, const void *const *ia,
                           uint64_t nj, const void *const *ja, bool same,
                           void *const *out, void *ws, int shape, int gsplit,
                           unsigned *err, cudaStream_t st);
}  // namespace tg

namespace tg {
std::atomic<unsigned long long> g_launch_count{0};
std::atomic<uint32_t> g_pipe_spin{1u << 20};
uint32_t pipe_spin_limit() { return g_pipe_spin.load(); }
std::atomic<float> g_centred_mid{3.0f};
float centred_mid_reach() { return g_centred_mid.load(); }
}

using namespace tg;

namespace {

std::mutex g_mu;
int g_status = ST_OK;
char g_message[512] = "";
int g_mode = MODE_EXACT;
long long g_kepler_budget = 1LL << 20;
unsigned g_last_device_error = 0;
int g_override_variant[K_COUNT];
int g_override_gsplit[K_COUNT];
bool g_override_init = false;
// Centred sweeps: -1 automatic (large Phi/Acc/AccJerk sweeps), 0 never,
// 1 always where supported; shape and grid split (< 0 / 0: automatic).
int g_centred_policy = -1;
int g_centred_shape = -1;
int g_centred_gsplit = 0;
// Sweeps of at least this many interactions (and 512 j) take the centred
// path automatically: below it the sort and tile build cost more than the
// sweep saves (measured on Plummer spheres, AccJerk / Acc: N = 16384
// centred 480 / 665 Gint/s against 657 / 1108 on the split variants;
// N = 65536 centred 943 / 1665 against 860 / 1416).
constexpr double CENTRED_MIN_INTERACTIONS = 2147483648.0;  // 2^31

struct Tuned {
    int variant, gsplit;
};
std::unordered_map<uint64_t, Tuned> g_tuned;

void set_error(int status, const char *fmt, ...)
    __attribute__((format(printf, 2, 3)));

void set_error(int status, const char *fmt, ...)
{
    g_status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_message, sizeof(g_message), fmt, ap);
    va_end(ap);
    fprintf(stderr, "tupan_gb300: %s\n", g_message);
}

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(ST_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return ST_CUDA;
}

// Per-device state: a stream, an error word and grow-only buffers.
struct DeviceState {
    int device = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    unsigned *err = nullptr;       // device error word
    void *io = nullptr;            // staged inputs/outputs of host-array calls
    size_t io_bytes = 0;
    void *pack = nullptr;          // packed FP32 records (i then j)
    size_t pack_bytes = 0;
    double *partial = nullptr;     // grid j-split partial sums
    size_t partial_bytes = 0;
};

std::unordered_map<int, DeviceState *> g_devices;

int grow(void **p, size_t *have, size_t need, const char *what)
{
    if (need <= *have) return ST_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    size_t want = need + need / 4;
    cudaError_t e = cudaMalloc(p, want);
    if (e != cudaSuccess) return cuda_fail(e, what);
    *have = want;
    return ST_OK;
}

int device_state(DeviceState **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(ST_NO_DEVICE, "no usable CUDA device: %s",
                  cudaGetErrorString(e));
        return ST_NO_DEVICE;
    }
    auto it = g_devices.find(dev);
    if (it != g_devices.end()) {
        *out = it->second;
        return ST_OK;
    }
    DeviceState *d = new DeviceState();
    d->device = dev;
    e = cudaDeviceGetAttribute(&d->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    e = cudaMalloc((void **)&d->err, sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(error word)");
    e = cudaMemset(d->err, 0, sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(error word)");
    g_devices[dev] = d;
    *out = d;
    return ST_OK;
}

void init_overrides()
{
    if (g_override_init) return;
    for (int k = 0; k < K_COUNT; ++k) {
        g_override_variant[k] = -1;
        g_override_gsplit[k] = 0;
    }
    const char *m = getenv("TUPAN_GB300_MODE");
    if (m && (!strcmp(m, "split") || !strcmp(m, "1"))) g_mode = MODE_SPLIT;
    g_override_init = true;
}

int ilog2_bucket(uint64_t n)
{
    int b = 0;
    while ((1ull << (b + 1)) <= n && b < 62) ++b;
    return b;
}

uint64_t tune_key(int kernel, uint64_t ni, uint64_t nj)
{
    return ((uint64_t)kernel << 16) | ((uint64_t)ilog2_bucket(ni) << 8) |
           (uint64_t)ilog2_bucket(nj);
}

// Occupancy model of one split variant: predicted time of a sweep in units
// of "one CTA over all j", i.e. waves x work per CTA, with small penalties
// for lanes that split j (shuffles, shorter runs) and for the partial-sum
// pass of grid splits.
void choose_split(const DeviceState *d, int kernel, uint64_t ni, uint64_t nj,
                  int *variant, int *gsplit)
{
    if (g_override_variant[kernel] >= 0) {
        *variant = g_override_variant[kernel];
        *gsplit = g_override_gsplit[kernel] > 0 ? g_override_gsplit[kernel] : 1;
        return;
    }
    auto it = g_tuned.find(tune_key(kernel, ni, nj));
    if (it != g_tuned.end()) {
        *variant = it->second.variant;
        *gsplit = it->second.gsplit;
        return;
    }
    const int nv = split_variant_count();
    const uint64_t jt = (nj + 255) / 256;
    double best = 1e300;
    *variant = 0;
    *gsplit = 1;
    const bool x2 = split_has_x2(kernel);
    for (int v = 0; v < nv; ++v) {
        int nip, js, nt;
        split_variant_info(v, &nip, &js, &nt);
        // variants 5 and 6 are the packed-pair forms of 0 and (2 i, JS=4)
        // (measured 12-18 % faster on every SPLIT kernel); 7 and 8 are
        // packed forms with one CTA per SM, left to measured tuning; 9-11
        // are the no-Newton forms of 5, 7 and 0, substituted below.
        const bool packed = (v >= 5);
        if (packed && !x2) continue;
        if (v >= 7) continue;
        const double ipc = (double)(nt / js) * nip;
        const uint64_t gx = (uint64_t)((ni + ipc - 1) / ipc);
        const int per_sm = nt >= 256 ? 2 : 4;
        const double cap = (double)d->sms * per_sm;
        const double eff = (nip == 2 ? 1.0 : 0.9) *
                           (js == 1 ? 1.0 : js <= 4 ? 0.95 : 0.88) *
                           (packed ? 1.15 : 1.0);
        for (int g = 1; g <= 64; g *= 2) {
            if ((uint64_t)g > jt && g > 1) break;
            const double waves = ceil((double)gx * g / cap);
            const double t = waves * (double)nip / js * ((double)nj / g) / eff +
                             (g > 1 ? 0.02 * (double)nj / g : 0.0);
            if (t < best * 0.999) {
                best = t;
                *variant = v;
                *gsplit = g;
            }
        }
    }
    // Phi, Acc and AccJerk take 1/sqrt from the MUFU approximation alone
    // where that form exists (variants 9 and 11): measured 7-16 % faster
    // at N = 2^16-2^18, with max |da|/|a| 1.0e-7 against the fp64 oracle
    // (1.3e-7 with the Newton step, whose rounding adds a small bias).
    if (split_has_raw(kernel)) {
        if (*variant == 5) *variant = 9;
        else if (*variant == 0) *variant = 11;
    }
}

// Whether a SPLIT sweep takes the centred kernels (csweep.cu).
bool use_centred(int k, uint64_t ni, uint64_t nj)
{
    if (!centred_supported(k) || g_centred_policy == 0 || nj == 0) return false;
    if (ni > 0xffffffffull || nj > 0xffffffffull) return false;
    if (g_centred_policy == 1) return true;
    return nj >= 512 && (double)ni * (double)nj >= CENTRED_MIN_INTERACTIONS;
}

// Launch shape and grid j-split of a centred sweep.
void centred_plan(const DeviceState *d, uint64_t ni, uint64_t nj, int *shape,
                  int *gsplit)
{
    *shape = g_centred_shape >= 0 ? g_centred_shape : 0;
    *gsplit = g_centred_gsplit > 0
                  ? g_centred_gsplit
                  : centred_choose_gsplit(ni, nj, *shape, d->sms);
}

template <typename T>
const T *cptr(const void *p) { return (const T *)p; }

// ---------------------------------------------------------------------------
// Core: run one sweep on DEVICE arrays.
// ---------------------------------------------------------------------------
int run_device_sweep(DeviceState *d, Sweep &s, cudaStream_t st)
{
    const int k = s.kernel;
    int mode = s.mode;
    if (!TG_PREC_SPLIT_OK || !split_supported(k)) mode = MODE_EXACT;
    cudaError_t e;
    if (mode == MODE_EXACT) {
        e = launch_exact<REAL>(s, st, g_kepler_budget, d->err);
        if (e != cudaSuccess) return cuda_fail(e, "exact sweep launch");
        return ST_OK;
    }
#if TG_PREC_SPLIT_OK
    if (s.ni == 0) return ST_OK;
    const int nf = split_nf_host(k);
    const bool same = (s.ni == s.nj) && [&] {
        for (int a = 0; a < n_attr(k); ++a)
            if (s.ip[a] != s.jp[a]) return false;
        return true;
    }();
    if (use_centred(k, s.ni, s.nj)) {
        int shape, gsplit;
        centred_plan(d, s.ni, s.nj, &shape, &gsplit);
        int rc = grow(&d->pack, &d->pack_bytes,
                      centred_workspace_bytes(k, s.ni, s.nj, same, gsplit),
                      "centred sweep workspace");
        if (rc) return rc;
        e = launch_centred(k, s.ni, s.ip, s.nj, s.jp, same, s.out, d->pack,
                           shape, gsplit, d->err, st);
        if (e != cudaSuccess) return cuda_fail(e, "centred sweep launch");
        return ST_OK;
    }
    int variant, gsplit;
    choose_split(d, k, s.ni, s.nj, &variant, &gsplit);
    const size_t ibytes = (size_t)s.ni * nf * sizeof(float4);
    const size_t jbytes = same ? 0 : (size_t)s.nj * nf * sizeof(float4);
    int rc = grow(&d->pack, &d->pack_bytes, ibytes + jbytes + 256, "pack buffer");
    if (rc) return rc;
    float4 *irec = (float4 *)d->pack;
    float4 *jrec = same ? irec : (float4 *)((char *)d->pack + ibytes);
    e = launch_pack(k, s.ni, s.ip, irec, st);
    if (e != cudaSuccess) return cuda_fail(e, "pack launch");
    if (!same) {
        e = launch_pack(k, s.nj, s.jp, jrec, st);
        if (e != cudaSuccess) return cuda_fail(e, "pack launch");
    }
    if (gsplit > 1) {
        rc = grow((void **)&d->partial, &d->partial_bytes,
                  (size_t)gsplit * n_out(k) * s.ni * sizeof(double),
                  "partial buffer");
        if (rc) return rc;
    }
    double pn[8] = {(double)s.iscal, s.scal[1], s.scal[2], s.scal[3],
                    s.scal[4], s.scal[5], s.scal[6], s.scal[7]};
    e = launch_split_pn(k, irec, jrec, s.ni, s.nj, s.out, d->partial, variant,
                        gsplit, s.scal[0], pn, d->err, st);
    if (e != cudaSuccess) return cuda_fail(e, "split sweep launch");
    return ST_OK;
#else
    return ST_OK;
#endif
}

// Reads and clears the device error word (synchronises the stream).
int check_device_error(DeviceState *d, cudaStream_t st)
{
    unsigned h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, d->err, sizeof(unsigned),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "sweep execution");
    g_last_device_error = h;
    if (h) {
        cudaMemsetAsync(d->err, 0, sizeof(unsigned), st);
        cudaStreamSynchronize(st);
        set_error(ST_DEVICE, "device error word 0x%x%s%s", h,
                  (h & DERR_PIPE_TIMEOUT) ? " (copy pipeline timed out)" : "",
                  (h & DERR_KEPLER_BUDGET) ? " (Kepler solve budget exhausted)" : "");
        return ST_DEVICE;
    }
    return ST_OK;
}

// ---------------------------------------------------------------------------
// Host-array calls: stage inputs, run, copy outputs back.
// ---------------------------------------------------------------------------
struct HostCall {
    int kernel;
    uint64_t ni, nj;
    const REAL *ip[MAX_ATTR];
    const REAL *jp[MAX_ATTR];
    REAL *out[MAX_OUT];
    double scal[8];
    int64_t iscal;
};

int host_call(const HostCall &c)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    g_status = ST_OK;
    g_message[0] = 0;
    const int k = c.kernel;
    const int na = n_attr(k), no = n_out(k);
    const bool kepler = (k == K_KEPLER);
    const uint64_t ni = kepler ? 2 : c.ni;
    const uint64_t nj = kepler ? 0 : c.nj;
    for (int a = 0; a < na; ++a) {
        if ((ni && !c.ip[a]) || (!kepler && nj && !c.jp[a])) {
            set_error(ST_BAD_ARGUMENT, "null input array for a non-empty set");
            return ST_BAD_ARGUMENT;
        }
    }
    for (int o = 0; o < no; ++o)
        if (ni && !c.out[o]) {
            set_error(ST_BAD_ARGUMENT, "null output array");
            return ST_BAD_ARGUMENT;
        }
    if (ni == 0) return ST_OK;

    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    cudaStream_t st = d->stream;

    // Stage each distinct host array once (i and j sets often alias).
    const REAL *host[2 * MAX_ATTR];
    uint64_t len[2 * MAX_ATTR];
    int nh = 0;
    int slot_i[MAX_ATTR], slot_j[MAX_ATTR];
    auto slot_of = [&](const REAL *p, uint64_t n) {
        for (int h = 0; h < nh; ++h)
            if (host[h] == p && len[h] == n) return h;
        host[nh] = p;
        len[nh] = n;
        return nh++;
    };
    for (int a = 0; a < na; ++a) slot_i[a] = slot_of(c.ip[a], ni);
    if (!kepler && nj)
        for (int a = 0; a < na; ++a) slot_j[a] = slot_of(c.jp[a], nj);
    size_t off[2 * MAX_ATTR + MAX_OUT];
    size_t total = 0;
    for (int h = 0; h < nh; ++h) {
        off[h] = total;
        total += (len[h] * sizeof(REAL) + 255) / 256 * 256;
    }
    for (int o = 0; o < no; ++o) {
        off[nh + o] = total;
        total += (ni * sizeof(REAL) + 255) / 256 * 256;
    }
    rc = grow(&d->io, &d->io_bytes, total, "staging buffer");
    if (rc) return rc;
    char *base = (char *)d->io;
    cudaError_t e;
    for (int h = 0; h < nh; ++h) {
        e = cudaMemcpyAsync(base + off[h], host[h], len[h] * sizeof(REAL),
                            cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
    }
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = k;
    s.mode = g_mode;
    s.ni = ni;
    s.nj = nj;
    for (int a = 0; a < na; ++a) {
        s.ip[a] = base + off[slot_i[a]];
        s.jp[a] = (!kepler && nj) ? base + off[slot_j[a]] : nullptr;
    }
    for (int o = 0; o < no; ++o) s.out[o] = base + off[nh + o];
    memcpy(s.scal, c.scal, sizeof(s.scal));
    s.iscal = c.iscal;
    rc = run_device_sweep(d, s, st);
    if (rc) return rc;
    for (int o = 0; o < no; ++o) {
        e = cudaMemcpyAsync(c.out[o], s.out[o], ni * sizeof(REAL),
                            cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
    }
    return check_device_error(d, st);
}

void fill_side(const REAL **dst, std::initializer_list<const REAL *> src)
{
    int a = 0;
    for (const REAL *p : src) dst[a++] = p;
}

}  // namespace

namespace tg {
// Split configuration for callers inside the library (the drivers).
void choose_split_public(int kernel, uint64_t ni, uint64_t nj, int *variant,
                         int *gsplit)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    DeviceState *d;
    if (device_state(&d)) {
        *variant = 0;
        *gsplit = 1;
        return;
    }
    choose_split(d, kernel, ni, nj, variant, gsplit);
}

int split_nf_host(int k)
{
    return (k == K_PHI || k == K_ACC) ? 2 : (k == K_SNAP_CRACKLE ? 5 : 3);
}
}  // namespace tg

// ===========================================================================
// libtupan.h entry points (tupan/lib/src/libtupan.h:2-246).
// ===========================================================================

// libtupan.h:2-15
TG_EXPORT void phi_kernel(const UINT ni, const REAL *_im, const REAL *_irx,
                          const REAL *_iry, const REAL *_irz,
                          const REAL *_ie2, const UINT nj, const REAL *_jm,
                          const REAL *_jrx, const REAL *_jry,
                          const REAL *_jrz, const REAL *_je2, REAL *_iphi)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_PHI;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2});
    c.out[0] = _iphi;
    host_call(c);
}

// libtupan.h:17-32
TG_EXPORT void acc_kernel(const UINT ni, const REAL *_im, const REAL *_irx,
                          const REAL *_iry, const REAL *_irz,
                          const REAL *_ie2, const UINT nj, const REAL *_jm,
                          const REAL *_jrx, const REAL *_jry,
                          const REAL *_jrz, const REAL *_je2, REAL *_iax,
                          REAL *_iay, REAL *_iaz)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_ACC;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2});
    c.out[0] = _iax;
    c.out[1] = _iay;
    c.out[2] = _iaz;
    host_call(c);
}

// libtupan.h:34-58
TG_EXPORT void acc_jerk_kernel(
    const UINT ni, const REAL *_im, const REAL *_irx, const REAL *_iry,
    const REAL *_irz, const REAL *_ie2, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const UINT nj, const REAL *_jm, const REAL *_jrx,
    const REAL *_jry, const REAL *_jrz, const REAL *_je2, const REAL *_jvx,
    const REAL *_jvy, const REAL *_jvz, REAL *_iax, REAL *_iay, REAL *_iaz,
    REAL *_ijx, REAL *_ijy, REAL *_ijz)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_ACC_JERK;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2, _jvx, _jvy, _jvz});
    REAL *o[] = {_iax, _iay, _iaz, _ijx, _ijy, _ijz};
    for (int q = 0; q < 6; ++q) c.out[q] = o[q];
    host_call(c);
}

// libtupan.h:60-96
TG_EXPORT void snap_crackle_kernel(
    const UINT ni, const REAL *_im, const REAL *_irx, const REAL *_iry,
    const REAL *_irz, const REAL *_ie2, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const REAL *_iax, const REAL *_iay, const REAL *_iaz,
    const REAL *_ijx, const REAL *_ijy, const REAL *_ijz, const UINT nj,
    const REAL *_jm, const REAL *_jrx, const REAL *_jry, const REAL *_jrz,
    const REAL *_je2, const REAL *_jvx, const REAL *_jvy, const REAL *_jvz,
    const REAL *_jax, const REAL *_jay, const REAL *_jaz, const REAL *_jjx,
    const REAL *_jjy, const REAL *_jjz, REAL *_isx, REAL *_isy, REAL *_isz,
    REAL *_icx, REAL *_icy, REAL *_icz)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_SNAP_CRACKLE;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz, _iax,
                     _iay, _iaz, _ijx, _ijy, _ijz});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2, _jvx, _jvy, _jvz, _jax,
                     _jay, _jaz, _jjx, _jjy, _jjz});
    REAL *o[] = {_isx, _isy, _isz, _icx, _icy, _icz};
    for (int q = 0; q < 6; ++q) c.out[q] = o[q];
    host_call(c);
}

// libtupan.h:98-119
TG_EXPORT void tstep_kernel(
    const UINT ni, const REAL *_im, const REAL *_irx, const REAL *_iry,
    const REAL *_irz, const REAL *_ie2, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const UINT nj, const REAL *_jm, const REAL *_jrx,
    const REAL *_jry, const REAL *_jrz, const REAL *_je2, const REAL *_jvx,
    const REAL *_jvy, const REAL *_jvz, const REAL eta, REAL *_idt_a,
    REAL *_idt_b)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_TSTEP;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2, _jvx, _jvy, _jvz});
    c.scal[0] = eta;
    c.out[0] = _idt_a;
    c.out[1] = _idt_b;
    host_call(c);
}

// libtupan.h:121-150
TG_EXPORT void pnacc_kernel(
    const UINT ni, const REAL *_im, const REAL *_irx, const REAL *_iry,
    const REAL *_irz, const REAL *_ie2, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const UINT nj, const REAL *_jm, const REAL *_jrx,
    const REAL *_jry, const REAL *_jrz, const REAL *_je2, const REAL *_jvx,
    const REAL *_jvy, const REAL *_jvz, UINT order, const REAL inv1,
    const REAL inv2, const REAL inv3, const REAL inv4, const REAL inv5,
    const REAL inv6, const REAL inv7, REAL *_ipnax, REAL *_ipnay,
    REAL *_ipnaz)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_PNACC;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2, _jvx, _jvy, _jvz});
    c.iscal = (int64_t)order;
    const REAL inv[7] = {inv1, inv2, inv3, inv4, inv5, inv6, inv7};
    for (int q = 0; q < 7; ++q) c.scal[1 + q] = inv[q];
    c.out[0] = _ipnax;
    c.out[1] = _ipnay;
    c.out[2] = _ipnaz;
    host_call(c);
}

// libtupan.h:152-178
TG_EXPORT void nreg_Xkernel(
    const UINT ni, const REAL *_im, const REAL *_irx, const REAL *_iry,
    const REAL *_irz, const REAL *_ie2, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const UINT nj, const REAL *_jm, const REAL *_jrx,
    const REAL *_jry, const REAL *_jrz, const REAL *_je2, const REAL *_jvx,
    const REAL *_jvy, const REAL *_jvz, const REAL dt, REAL *_idrx,
    REAL *_idry, REAL *_idrz, REAL *_iax, REAL *_iay, REAL *_iaz, REAL *_iu)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_NREG_X;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2, _jvx, _jvy, _jvz});
    c.scal[0] = dt;
    REAL *o[] = {_idrx, _idry, _idrz, _iax, _iay, _iaz, _iu};
    for (int q = 0; q < 7; ++q) c.out[q] = o[q];
    host_call(c);
}

// libtupan.h:180-201
TG_EXPORT void nreg_Vkernel(
    const UINT ni, const REAL *_im, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const REAL *_iax, const REAL *_iay, const REAL *_iaz,
    const UINT nj, const REAL *_jm, const REAL *_jvx, const REAL *_jvy,
    const REAL *_jvz, const REAL *_jax, const REAL *_jay, const REAL *_jaz,
    const REAL dt, REAL *_idvx, REAL *_idvy, REAL *_idvz, REAL *_ik)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_NREG_V;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _ivx, _ivy, _ivz, _iax, _iay, _iaz});
    fill_side(c.jp, {_jm, _jvx, _jvy, _jvz, _jax, _jay, _jaz});
    c.scal[0] = dt;
    REAL *o[] = {_idvx, _idvy, _idvz, _ik};
    for (int q = 0; q < 4; ++q) c.out[q] = o[q];
    host_call(c);
}

// libtupan.h:203-229
TG_EXPORT void sakura_kernel(
    const UINT ni, const REAL *_im, const REAL *_irx, const REAL *_iry,
    const REAL *_irz, const REAL *_ie2, const REAL *_ivx, const REAL *_ivy,
    const REAL *_ivz, const UINT nj, const REAL *_jm, const REAL *_jrx,
    const REAL *_jry, const REAL *_jrz, const REAL *_je2, const REAL *_jvx,
    const REAL *_jvy, const REAL *_jvz, const REAL dt, const INT flag,
    REAL *_idrx, REAL *_idry, REAL *_idrz, REAL *_idvx, REAL *_idvy,
    REAL *_idvz)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_SAKURA;
    c.ni = ni;
    c.nj = nj;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz});
    fill_side(c.jp, {_jm, _jrx, _jry, _jrz, _je2, _jvx, _jvy, _jvz});
    c.scal[0] = dt;
    c.iscal = (int64_t)flag;
    REAL *o[] = {_idrx, _idry, _idrz, _idvx, _idvy, _idvz};
    for (int q = 0; q < 6; ++q) c.out[q] = o[q];
    host_call(c);
}

// libtupan.h:231-246 (two particles; outputs may alias the inputs)
TG_EXPORT void kepler_solver_kernel(
    const REAL *_im, const REAL *_irx, const REAL *_iry, const REAL *_irz,
    const REAL *_ie2, const REAL *_ivx, const REAL *_ivy, const REAL *_ivz,
    const REAL dt, REAL *_ir1x, REAL *_ir1y, REAL *_ir1z, REAL *_iv1x,
    REAL *_iv1y, REAL *_iv1z)
{
    HostCall c;
    memset(&c, 0, sizeof(c));
    c.kernel = K_KEPLER;
    c.ni = 2;
    c.nj = 0;
    fill_side(c.ip, {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz});
    c.scal[0] = dt;
    REAL *o[] = {_ir1x, _ir1y, _ir1z, _iv1x, _iv1y, _iv1z};
    for (int q = 0; q < 6; ++q) c.out[q] = o[q];
    host_call(c);
}

// ===========================================================================
// Extensions of the ABI (no counterpart in the reference).
// ===========================================================================

// Status of the most recent call on this library (0 = success) and its
// message; the libtupan.h entry points return void like the reference.
TG_EXPORT int tupan_gb300_last_error(void) { return g_status; }

TG_EXPORT const char *tupan_gb300_last_error_message(void) { return g_message; }

// Error word of the last sweep as written by the kernels (DeviceError bits).
TG_EXPORT unsigned tupan_gb300_last_device_error(void)
{
    return g_last_device_error;
}

// 0: EXACT (bit-identical to the reference C), 1: SPLIT (FP32 pairs on
// double-single positions; float64 library only).  Returns the previous mode.
TG_EXPORT int tupan_gb300_set_mode(int mode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    int old = g_mode;
    if (mode == MODE_EXACT || (mode == MODE_SPLIT && TG_PREC_SPLIT_OK))
        g_mode = mode;
    return old;
}

TG_EXPORT int tupan_gb300_get_mode(void)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    return g_mode;
}

// Upper bound on single-step Kepler solves per pair solve (the reference
// loops without bound); exceeding it raises DERR_KEPLER_BUDGET.
TG_EXPORT long long tupan_gb300_set_kepler_budget(long long budget)
{
    std::lock_guard<std::mutex> lock(g_mu);
    long long old = g_kepler_budget;
    if (budget > 0) g_kepler_budget = budget;
    return old;
}

// Force a split-sweep configuration for one kernel (variant < 0: automatic).
TG_EXPORT int tupan_gb300_set_split_config(int kernel, int variant, int gsplit)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    const int nv = split_variant_count();
    if (kernel < 0 || kernel >= K_COUNT || variant >= nv)
        return ST_BAD_ARGUMENT;
    g_override_variant[kernel] = variant;
    g_override_gsplit[kernel] = gsplit;
    return ST_OK;
}

// Name of the current CUDA device, NUL-terminated and truncated to len
// bytes (the key of the autotuner's saved table).
TG_EXPORT int tupan_gb300_device_name(char *buf, int len)
{
    if (!buf || len < 1) return ST_BAD_ARGUMENT;
    buf[0] = 0;
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
        cudaGetLastError();
        return ST_CUDA;
    }
    snprintf(buf, (size_t)len, "%s", p.name);
    return ST_OK;
}

// Record a tuned configuration for sizes in the same power-of-two buckets.
TG_EXPORT int tupan_gb300_set_tuned(int kernel, uint64_t ni, uint64_t nj,
                                    int variant, int gsplit)
{
    std::lock_guard<std::mutex> lock(g_mu);
    const int nv = split_variant_count();
    if (kernel < 0 || kernel >= K_COUNT || variant < 0 || variant >= nv ||
        gsplit < 1)
        return ST_BAD_ARGUMENT;
    g_tuned[tune_key(kernel, ni, nj)] = {variant, gsplit};
    return ST_OK;
}

// The configuration a split sweep of this size would use.
TG_EXPORT int tupan_gb300_split_choice(int kernel, uint64_t ni, uint64_t nj,
                                       int *variant, int *gsplit)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    choose_split(d, kernel, ni, nj, variant, gsplit);
    return ST_OK;
}

// Reach of the centred sweep's mid tiles in tile radii (default 3; at most
// 1.25, the near reach, turns them off: every tile beyond 1.25 R takes the
// one-operation far difference).  Returns the previous reach, or -1 (and
// changes nothing) for a reach that is negative, above 64 or not a number.
TG_EXPORT double tupan_gb300_set_centred_mid(double reach)
{
    if (!(reach >= 0.0 && reach <= 64.0)) return -1.0;
    return (double)g_centred_mid.exchange((float)reach);
}

// Centred SPLIT sweeps (Phi, Acc, AccJerk on Morton-ordered, tile-centred
// records; csweep.cu): policy -1 automatic (sweeps of at least 2^31
// interactions), 0 never, 1 always; shape < 0 and gsplit <= 0 automatic.
// Returns ST_OK or ST_BAD_ARGUMENT.
TG_EXPORT int tupan_gb300_set_centred(int policy, int shape, int gsplit)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (policy < -1 || policy > 1 || shape >= centred_shape_count())
        return ST_BAD_ARGUMENT;
    g_centred_policy = policy;
    g_centred_shape = shape;
    g_centred_gsplit = gsplit;
    return ST_OK;
}

// The path a SPLIT sweep of this size takes: *path 1 (centred, *config =
// launch shape) or 0 (split variants, *config = variant); *gsplit the grid
// j-split.
TG_EXPORT int tupan_gb300_sweep_plan(int kernel, uint64_t ni, uint64_t nj,
                                     int *path, int *config, int *gsplit)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    if (kernel < 0 || kernel >= K_COUNT) return ST_BAD_ARGUMENT;
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    if (use_centred(kernel, ni, nj)) {
        *path = 1;
        centred_plan(d, ni, nj, config, gsplit);
    } else {
        *path = 0;
        choose_split(d, kernel, ni, nj, config, gsplit);
    }
    return ST_OK;
}

// Tries each main-loop wait of the pipelined sweeps (split, centred,
// ensemble) makes on its copy barrier before it records DERR_PIPE_TIMEOUT
// and the CTA leaves without writing results (default 2^20; 0 makes every
// such wait time out at once).  Returns the previous limit.
TG_EXPORT unsigned tupan_gb300_set_pipe_spin_limit(unsigned limit)
{
    return g_pipe_spin.exchange(limit);
}

// Variants of the SPLIT sweep (0..8, compiled for every SPLIT kernel).
TG_EXPORT int tupan_gb300_split_variants(void) { return split_variant_count(); }

TG_EXPORT void tupan_gb300_split_variant_info(int v, int *ni_per_thread,
                                              int *jsplit, int *threads)
{
    split_variant_info(v, ni_per_thread, jsplit, threads);
}

// One sweep over DEVICE arrays on a caller's stream (NULL: the legacy
// default stream).  i_attrs/j_attrs: host arrays of n_attr(kernel) device pointers
// in libtupan.h order; outs: n_out(kernel) device pointers; scal: eta or dt
// in scal[0], 1/c^k in scal[k] for PNAcc; iscal: flag or PN order.  Returns
// 0 or a status code.  Asynchronous unless `sync` is non-zero, in which case
// the stream is synchronised and the device error word checked.
TG_EXPORT int tupan_gb300_dev_sweep(int kernel, int mode, uint64_t ni,
                                    const void *const *i_attrs, uint64_t nj,
                                    const void *const *j_attrs,
                                    const double *scal, int64_t iscal,
                                    void *const *outs, void *stream, int sync)
{
    std::lock_guard<std::mutex> lock(g_mu);
    init_overrides();
    g_status = ST_OK;
    g_message[0] = 0;
    if (kernel < 0 || kernel >= K_COUNT) {
        set_error(ST_BAD_ARGUMENT, "unknown kernel id %d", kernel);
        return ST_BAD_ARGUMENT;
    }
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;   // NULL: the default stream
    Sweep s;
    memset(&s, 0, sizeof(s));
    s.kernel = kernel;
    s.mode = mode < 0 ? g_mode : mode;
    s.ni = kernel == K_KEPLER ? 2 : ni;
    s.nj = kernel == K_KEPLER ? 0 : nj;
    for (int a = 0; a < n_attr(kernel); ++a) {
        s.ip[a] = i_attrs[a];
        s.jp[a] = (j_attrs && kernel != K_KEPLER) ? j_attrs[a] : nullptr;
    }
    for (int o = 0; o < n_out(kernel); ++o) s.out[o] = outs[o];
    if (scal) memcpy(s.scal, scal, sizeof(s.scal));
    s.iscal = iscal;
    rc = run_device_sweep(d, s, st);
    if (rc) return rc;
    if (sync) return check_device_error(d, st);
    return ST_OK;
}

// Number of per-particle inputs / outputs of a kernel id.
TG_EXPORT int tupan_gb300_kernel_arity(int kernel, int *n_inputs, int *n_outputs)
{
    if (kernel < 0 || kernel >= K_COUNT) return ST_BAD_ARGUMENT;
    *n_inputs = n_attr(kernel);
    *n_outputs = n_out(kernel);
    return ST_OK;
}

// Streaming multiprocessors of the current device (0 without a device).
TG_EXPORT int tupan_gb300_device_sms(void)
{
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceState *d;
    if (device_state(&d)) return 0;
    return d->sms;
}

// Precision this library was built for: 64 or 32.
TG_EXPORT int tupan_gb300_real_bits(void) { return (int)(8 * sizeof(REAL)); }

// Kernels this library has launched since it was loaded.
TG_EXPORT unsigned long long tupan_gb300_launch_count(void)
{
    return g_launch_count.load();
}
