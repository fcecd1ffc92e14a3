/*
 * tupan_gb300.h -- C-ABI of the GB300 (sm_103a) tupan kernel layer.
 *
 * Two shared libraries implement it:
 *   libtupan_gb300.so     REAL = double, UINT = uint64_t, INT = int64_t
 *   libtupan_gb300_sp.so  REAL = float,  UINT = uint32_t, INT = int32_t
 *                         (compile against this header with TUPAN_GB300_SP)
 * matching the two precisions tupan builds from tupan/lib/src/libtupan.h
 * (tupan/lib/cffi_backend.py:31-87: typedefs at :53-55, libraries at :84-87).
 *
 * The first ten functions replace the reference's kernels one for one: same
 * names, same argument order and meaning, void return.  They take HOST
 * arrays; inputs are copied to the GPU, the pairwise sums run there, results
 * are copied back before the call returns.  Every output array is overwritten
 * for all ni entries, as in the reference.  i and j arrays may be the same
 * arrays.  After a call, tupan_gb300_last_error() is 0 on success.
 */
#ifndef TUPAN_GB300_H
#define TUPAN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef TUPAN_GB300_SP
typedef float TG_REAL;
typedef uint32_t TG_UINT;
typedef int32_t TG_INT;
#else
typedef double TG_REAL;
typedef uint64_t TG_UINT;
typedef int64_t TG_INT;
#endif

/* Replaces phi_kernel, tupan/lib/src/libtupan.h:2-15 (phi_kernel.c:5-34). */
void phi_kernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                const TG_REAL *iry, const TG_REAL *irz, const TG_REAL *ie2,
                const TG_UINT nj, const TG_REAL *jm, const TG_REAL *jrx,
                const TG_REAL *jry, const TG_REAL *jrz, const TG_REAL *je2,
                TG_REAL *iphi);

/* Replaces acc_kernel, libtupan.h:17-32 (acc_kernel.c:5-40). */
void acc_kernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                const TG_REAL *iry, const TG_REAL *irz, const TG_REAL *ie2,
                const TG_UINT nj, const TG_REAL *jm, const TG_REAL *jrx,
                const TG_REAL *jry, const TG_REAL *jrz, const TG_REAL *je2,
                TG_REAL *iax, TG_REAL *iay, TG_REAL *iaz);

/* Replaces acc_jerk_kernel, libtupan.h:34-58 (acc_jerk_kernel.c:5-60). */
void acc_jerk_kernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                     const TG_REAL *iry, const TG_REAL *irz,
                     const TG_REAL *ie2, const TG_REAL *ivx,
                     const TG_REAL *ivy, const TG_REAL *ivz, const TG_UINT nj,
                     const TG_REAL *jm, const TG_REAL *jrx, const TG_REAL *jry,
                     const TG_REAL *jrz, const TG_REAL *je2,
                     const TG_REAL *jvx, const TG_REAL *jvy,
                     const TG_REAL *jvz, TG_REAL *iax, TG_REAL *iay,
                     TG_REAL *iaz, TG_REAL *ijx, TG_REAL *ijy, TG_REAL *ijz);

/* Replaces snap_crackle_kernel, libtupan.h:60-96
 * (snap_crackle_kernel.c:5-82). */
void snap_crackle_kernel(
    const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
    const TG_REAL *iry, const TG_REAL *irz, const TG_REAL *ie2,
    const TG_REAL *ivx, const TG_REAL *ivy, const TG_REAL *ivz,
    const TG_REAL *iax, const TG_REAL *iay, const TG_REAL *iaz,
    const TG_REAL *ijx, const TG_REAL *ijy, const TG_REAL *ijz,
    const TG_UINT nj, const TG_REAL *jm, const TG_REAL *jrx,
    const TG_REAL *jry, const TG_REAL *jrz, const TG_REAL *je2,
    const TG_REAL *jvx, const TG_REAL *jvy, const TG_REAL *jvz,
    const TG_REAL *jax, const TG_REAL *jay, const TG_REAL *jaz,
    const TG_REAL *jjx, const TG_REAL *jjy, const TG_REAL *jjz, TG_REAL *isx,
    TG_REAL *isy, TG_REAL *isz, TG_REAL *icx, TG_REAL *icy, TG_REAL *icz);

/* Replaces tstep_kernel, libtupan.h:98-119 (tstep_kernel.c:5-49). */
void tstep_kernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                  const TG_REAL *iry, const TG_REAL *irz, const TG_REAL *ie2,
                  const TG_REAL *ivx, const TG_REAL *ivy, const TG_REAL *ivz,
                  const TG_UINT nj, const TG_REAL *jm, const TG_REAL *jrx,
                  const TG_REAL *jry, const TG_REAL *jrz, const TG_REAL *je2,
                  const TG_REAL *jvx, const TG_REAL *jvy, const TG_REAL *jvz,
                  const TG_REAL eta, TG_REAL *idt_a, TG_REAL *idt_b);

/* Replaces pnacc_kernel, libtupan.h:121-150 (pnacc_kernel.c:5-60). */
void pnacc_kernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                  const TG_REAL *iry, const TG_REAL *irz, const TG_REAL *ie2,
                  const TG_REAL *ivx, const TG_REAL *ivy, const TG_REAL *ivz,
                  const TG_UINT nj, const TG_REAL *jm, const TG_REAL *jrx,
                  const TG_REAL *jry, const TG_REAL *jrz, const TG_REAL *je2,
                  const TG_REAL *jvx, const TG_REAL *jvy, const TG_REAL *jvz,
                  TG_UINT order, const TG_REAL inv1, const TG_REAL inv2,
                  const TG_REAL inv3, const TG_REAL inv4, const TG_REAL inv5,
                  const TG_REAL inv6, const TG_REAL inv7, TG_REAL *ipnax,
                  TG_REAL *ipnay, TG_REAL *ipnaz);

/* Replaces nreg_Xkernel, libtupan.h:152-178 (nreg_kernels.c:5-67). */
void nreg_Xkernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                  const TG_REAL *iry, const TG_REAL *irz, const TG_REAL *ie2,
                  const TG_REAL *ivx, const TG_REAL *ivy, const TG_REAL *ivz,
                  const TG_UINT nj, const TG_REAL *jm, const TG_REAL *jrx,
                  const TG_REAL *jry, const TG_REAL *jrz, const TG_REAL *je2,
                  const TG_REAL *jvx, const TG_REAL *jvy, const TG_REAL *jvz,
                  const TG_REAL dt, TG_REAL *idrx, TG_REAL *idry,
                  TG_REAL *idrz, TG_REAL *iax, TG_REAL *iay, TG_REAL *iaz,
                  TG_REAL *iu);

/* Replaces nreg_Vkernel, libtupan.h:180-201 (nreg_kernels.c:70-115). */
void nreg_Vkernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *ivx,
                  const TG_REAL *ivy, const TG_REAL *ivz, const TG_REAL *iax,
                  const TG_REAL *iay, const TG_REAL *iaz, const TG_UINT nj,
                  const TG_REAL *jm, const TG_REAL *jvx, const TG_REAL *jvy,
                  const TG_REAL *jvz, const TG_REAL *jax, const TG_REAL *jay,
                  const TG_REAL *jaz, const TG_REAL dt, TG_REAL *idvx,
                  TG_REAL *idvy, TG_REAL *idvz, TG_REAL *ik);

/* Replaces sakura_kernel, libtupan.h:203-229 (sakura_kernel.c:5-63). */
void sakura_kernel(const TG_UINT ni, const TG_REAL *im, const TG_REAL *irx,
                   const TG_REAL *iry, const TG_REAL *irz,
                   const TG_REAL *ie2, const TG_REAL *ivx, const TG_REAL *ivy,
                   const TG_REAL *ivz, const TG_UINT nj, const TG_REAL *jm,
                   const TG_REAL *jrx, const TG_REAL *jry, const TG_REAL *jrz,
                   const TG_REAL *je2, const TG_REAL *jvx, const TG_REAL *jvy,
                   const TG_REAL *jvz, const TG_REAL dt, const TG_INT flag,
                   TG_REAL *idrx, TG_REAL *idry, TG_REAL *idrz,
                   TG_REAL *idvx, TG_REAL *idvy, TG_REAL *idvz);

/* Replaces kepler_solver_kernel, libtupan.h:231-246
 * (kepler_solver_kernel.c:5-49).  Two particles; outputs may alias inputs. */
void kepler_solver_kernel(const TG_REAL *im, const TG_REAL *irx,
                          const TG_REAL *iry, const TG_REAL *irz,
                          const TG_REAL *ie2, const TG_REAL *ivx,
                          const TG_REAL *ivy, const TG_REAL *ivz,
                          const TG_REAL dt, TG_REAL *ir1x, TG_REAL *ir1y,
                          TG_REAL *ir1z, TG_REAL *iv1x, TG_REAL *iv1y,
                          TG_REAL *iv1z);

/* ------------------------------------------------------------------------
 * Extensions (no counterpart in the reference, whose kernels return void
 * and cannot fail, tupan/lib/src/libtupan.h:2-246).
 * ---------------------------------------------------------------------- */

/* Kernel ids used by the extension calls, in libtupan.h order. */
enum {
    TUPAN_GB300_PHI = 0, TUPAN_GB300_ACC = 1, TUPAN_GB300_ACC_JERK = 2,
    TUPAN_GB300_SNAP_CRACKLE = 3, TUPAN_GB300_TSTEP = 4,
    TUPAN_GB300_PNACC = 5, TUPAN_GB300_NREG_X = 6, TUPAN_GB300_NREG_V = 7,
    TUPAN_GB300_SAKURA = 8, TUPAN_GB300_KEPLER = 9
};

/* Status of the last call (0 = success; 1 CUDA error, 2 bad argument,
 * 3 device error word set, 4 no device, 5 request too large) and its text. */
int tupan_gb300_last_error(void);
const char *tupan_gb300_last_error_message(void);
/* Device error word of the last sweep: bit 0 copy-pipeline wait ran out,
 * bit 1 a Kepler solve exceeded its solve budget. */
unsigned tupan_gb300_last_device_error(void);

/* Arithmetic mode: 0 EXACT (default; bit-identical to the reference C for all
 * kernels but Sakura/Kepler, which agree to libm accuracy), 1 SPLIT (FP32
 * pairs on double-single positions with compensated sums; float64 library,
 * kernels phi/acc/acc_jerk/snap_crackle/tstep/pnacc -- the others stay
 * EXACT).
 * Returns the previous mode.  The environment variable TUPAN_GB300_MODE=split
 * selects SPLIT at load time. */
int tupan_gb300_set_mode(int mode);
int tupan_gb300_get_mode(void);

/* Bound on single-step solves per Kepler pair solve (default 2^20); the
 * reference's retry loops have none. Returns the previous bound. */
long long tupan_gb300_set_kepler_budget(long long budget);

/* Name of the current CUDA device (NUL-terminated, at most len bytes);
 * status 1 without a device. */
int tupan_gb300_device_name(char *buf, int len);

/* SPLIT-mode launch configuration: variant in [0, tupan_gb300_split_variants())
 * and grid j-split count; set_split_config forces it for a kernel
 * (variant < 0 restores the automatic choice), set_tuned records it for sizes
 * in the same power-of-two buckets, split_choice reports the choice.
 * Variants 0-8 form 1/sqrt as rsqrt plus one Newton step; 9, 10 and 11 are
 * variants 5, 7 and 0 with rsqrt alone (the automatic choice). */
int tupan_gb300_set_split_config(int kernel, int variant, int gsplit);
int tupan_gb300_set_tuned(int kernel, uint64_t ni, uint64_t nj, int variant,
                          int gsplit);
int tupan_gb300_split_choice(int kernel, uint64_t ni, uint64_t nj,
                             int *variant, int *gsplit);
int tupan_gb300_split_variants(void);
void tupan_gb300_split_variant_info(int variant, int *ni_per_thread,
                                    int *jsplit, int *threads);

/* Centred SPLIT sweeps of phi, acc and acc_jerk: particles in Morton order,
 * j-tiles stored relative to their centre, a one-operation position
 * difference for tiles far from every i of a warp.  policy -1: automatic
 * (sweeps of at least 2^31 interactions), 0: never, 1: always; shape (0: one
 * i per thread, 256 threads, two CTAs per SM; 1: two i per thread, one CTA
 * per SM; 2: one i per thread, 128 threads, four CTAs per SM) and grid
 * j-split gsplit: < 0 / <= 0 automatic.
 * Returns 0 or 2 (bad argument). */
int tupan_gb300_set_centred(int policy, int shape, int gsplit);
/* Reach of the centred sweep's mid tiles in tile radii (default 3): tiles
 * with some i of a warp within that reach (and none within 1.25 R) take the
 * i's low part in the position difference, one FP32 operation per axis more,
 * for the accuracy of particles whose net force is a near-cancelling sum; a
 * reach of at most 1.25 turns mid tiles off.  Returns the previous reach, or
 * -1 (no change) for a reach below 0, above 64 or not a number. */
double tupan_gb300_set_centred_mid(double reach);
/* The path a SPLIT sweep of this size takes: *path 1 = centred (*config =
 * shape), 0 = split variants (*config = variant); *gsplit = grid j-split. */
int tupan_gb300_sweep_plan(int kernel, uint64_t ni, uint64_t nj, int *path,
                           int *config, int *gsplit);
/* Tries of each main-loop wait of the pipelined sweeps on its copy barrier
 * before the CTA records device error bit 0 and leaves without writing
 * results (default 2^20; 0 makes every such wait time out at once, for
 * testing the error path).  The waits that drain copies still in flight keep
 * the full bound.  Returns the previous limit. */
unsigned tupan_gb300_set_pipe_spin_limit(unsigned limit);

/* One sweep over DEVICE arrays.  i_attrs / j_attrs: host arrays holding the
 * device pointers of the kernel's per-particle inputs in libtupan.h order
 * (j_attrs unused for Kepler); outs: device pointers of its outputs.
 * scal[0] = eta (tstep) or dt (nreg, sakura, kepler); scal[1..7] = 1/c^k
 * (pnacc).  iscal = flag (sakura) or PN order (pnacc).  mode < 0 uses the
 * library mode.  stream: a cudaStream_t, NULL meaning the default stream.
 * Asynchronous unless sync != 0.
 * Returns a status code. */
int tupan_gb300_dev_sweep(int kernel, int mode, uint64_t ni,
                          const void *const *i_attrs, uint64_t nj,
                          const void *const *j_attrs, const double *scal,
                          int64_t iscal, void *const *outs, void *stream,
                          int sync);

/* Inputs per particle and outputs of a kernel id. */
int tupan_gb300_kernel_arity(int kernel, int *n_inputs, int *n_outputs);
/* Streaming multiprocessors of the current device (0 without one). */
int tupan_gb300_device_sms(void);
/* 64 for libtupan_gb300.so, 32 for libtupan_gb300_sp.so. */
int tupan_gb300_real_bits(void);
/* Kernels launched by this library since it was loaded. */
unsigned long long tupan_gb300_launch_count(void);

/* FP32 FMA throughput probe: tupan_gb300_fma_sweep launches independent FMA
 * chains on every SM on `stream` and returns the flops it performs (for
 * timing by the caller); tupan_gb300_fp32_peak_tflops times `reps` sweeps
 * itself and returns the best TFLOP/s. */
double tupan_gb300_fma_sweep(int iters, void *stream);
double tupan_gb300_fp32_peak_tflops(int iters, int reps);


/* ------------------------------------------------------------------------
 * Device-resident Hermite driver (libtupan_gb300.so only).  No counterpart
 * in the reference, whose integrators (tupan/integrator/hermite.py:286-410)
 * keep particles in host arrays and call the kernels once per force
 * evaluation.  One system stays in HBM; a step follows Hermite.do_step with
 * epec(2) and, when adaptive, the Tstep kernel plus the power-of-two rule of
 * tupan/integrator/__init__.py:59-78, all on the device.
 * ---------------------------------------------------------------------- */
/* order 2/4/6/8; adaptive 1 = "ahermiteN"; mode 0 EXACT, 1 SPLIT; host
 * arrays are copied in; tau_log_cap step sizes are recorded. */
int tupan_gb300_hermite_create(uint64_t n, int order, int adaptive, int mode,
                               double eta, const double *m, const double *e2,
                               const double *rx, const double *ry,
                               const double *rz, const double *vx,
                               const double *vy, const double *vz,
                               long long tau_log_cap, void **handle);
/* Steps until |t| >= t_end or max_steps (0: no limit) steps were taken,
 * replaying a CUDA graph of `batch` steps between host checks. */
int tupan_gb300_hermite_evolve(void *handle, double t_end,
                               long long max_steps, int batch, double *t_out,
                               long long *steps_out);
int tupan_gb300_hermite_get_state(void *handle, double *rx, double *ry,
                                  double *rz, double *vx, double *vy,
                                  double *vz);
long long tupan_gb300_hermite_tau_log(void *handle, double *out,
                                      long long cap);
/* Kinetic and potential energy, fp64 (EXACT Phi sweep). */
int tupan_gb300_hermite_energy(void *handle, double *ke, double *pe);
int tupan_gb300_hermite_destroy(void *handle);

/* No counterpart in the reference.  The acc_jerk sum in SPLIT arithmetic on
 * DEVICE arrays, for callers that cannot let the library allocate device
 * memory: an application whose memory manager owns the whole device heap,
 * or a step loop that must not stall on cudaMalloc's device-wide
 * synchronisation.  Arguments: ni and the i-set's m, rx, ry, rz, e2, vx, vy,
 * vz; nj and the j-set's eight arrays in the same order; the outputs ax, ay,
 * az, jx, jy, jz (ni each); a cudaStream_t (NULL: the default stream); an
 * optional host pointer for the device error word.  Its scratch (packed
 * particle records and grid j-split partial sums) is 12 MiB of static device
 * arrays, so ni and nj are limited to 65536 each; larger requests return 5
 * before anything runs.  All calls share those arrays: calls that overlap on
 * the GPU race.  The first call on a device looks up the arrays' addresses
 * there; make it outside stream capture.  err_out == NULL: asynchronous, and
 * no device error is reported; otherwise the call waits for the stream,
 * stores the sweep's device error word and returns 3 if it is non-zero.
 * Returns 0 or a status code. */
int tupan_gb300_acc_jerk_split_noalloc(
    uint64_t ni, const double *im, const double *irx, const double *iry,
    const double *irz, const double *ie2, const double *ivx,
    const double *ivy, const double *ivz, uint64_t nj, const double *jm,
    const double *jrx, const double *jry, const double *jrz,
    const double *je2, const double *jvx, const double *jvy,
    const double *jvz, double *iax, double *iay, double *iaz, double *ijx,
    double *ijy, double *ijz, void *stream, unsigned *err_out);

/* ------------------------------------------------------------------------
 * Block time steps (libtupan_gb300.so only).  No counterpart in the
 * reference, whose Hermite integrator (tupan/integrator/hermite.py:286-410)
 * moves every particle with one shared step.  Each particle keeps a
 * power-of-two step (the quantisation of tupan/integrator/__init__.py:59-78
 * applied per particle, capped at dt_max); a block step predicts all
 * particles to the next block time, sweeps forces for the active set only
 * (compacted on the device) and corrects those particles with epec(2).
 * ---------------------------------------------------------------------- */
/* Host arrays are copied in; forces and steps are initialised at t = 0.
 * order 4, 6 or 8; mode 0 EXACT, 1 SPLIT. */
int tupan_gb300_block_create(uint64_t n, int order, int mode, double eta,
                             double dt_max, const double *m, const double *e2,
                             const double *rx, const double *ry,
                             const double *rz, const double *vx,
                             const double *vy, const double *vz,
                             void **handle);
/* Block steps until t >= t_end or max_steps (0: no limit); returns the time
 * reached, the steps taken and the sum of active-set sizes over them. */
int tupan_gb300_block_evolve(void *handle, double t_end, long long max_steps,
                             double *t_out, long long *steps_out,
                             long long *active_out);
/* Positions and velocities at each particle's own last time t[i], and its
 * current step dt[i] (host arrays of n). */
int tupan_gb300_block_get_state(void *handle, double *rx, double *ry,
                                double *rz, double *vx, double *vy,
                                double *vz, double *t, double *dt);
int tupan_gb300_block_destroy(void *handle);
/* How block steps are launched: 1 (default) one CUDA graph per batch of
 * steps, the active set sized on the device (a WHILE node over steps, a
 * SWITCH node over active-count levels whose bodies are captured with the
 * sweep shape of each level); 0 host-synchronised (the active count is read
 * back every step).  Returns the previous setting, -1 for a null handle. */
int tupan_gb300_block_set_graphs(void *handle, int on);
/* 1 when evolve runs the graph path, 0 the host-synchronised one (also when
 * the graph could not be built). */
int tupan_gb300_block_launch_mode(void *handle);

/* ------------------------------------------------------------------------
 * Sakura and Kepler (libtupan_gb300.so only).  The pair arithmetic is that
 * of sakura_kernel (libtupan.h:203-229) and kepler_solver_kernel
 * (libtupan.h:231-246); these entry points reorganise its schedule: the
 * pairs that need the universal Kepler solver are queued and solved by a
 * separate pass, so one expensive pair does not stall a warp of cheap
 * ones.  All pointers are DEVICE pointers unless marked host.  Status 3:
 * a solve used up the retry budget (0: 2^20 single-step solves).
 * ---------------------------------------------------------------------- */
/* Learned start of the universal-anomaly iteration: bf16 weights w1 (64x4),
 * w2 (64x64), w3 (64), fp32 biases b1 b2 b3 and norm[8] = mean[4],
 * 1/std[4] of the features.  The network replaces the plain starting guess
 * only where the feature log(|dt| sqrt(m/r^3)) exceeds gate.  w1 == NULL
 * removes it.  The arrays must outlive the installation. */
int tupan_gb300_kepler_set_mlp(const void *w1, const float *b1,
                               const void *w2, const float *b2,
                               const void *w3, const float *b3,
                               const float *norm, float gate);
/* Form of the universal-Kepler root solve for kepler_pairs, sakura_queue and
 * the device Sakura integrator (no counterpart in the reference): 0 the
 * reference's structure (default), 1 the same arithmetic with cos/sin (or
 * cosh/sinh) evaluated once per Laguerre update (bit-identical results),
 * 2 mixed precision: FP32 Laguerre updates, then FP64 updates until the
 * reference's 2^-42 tolerance is met.  The libtupan.h entry points always use
 * form 0.  Returns the previous form, or -1 for an unknown form. */
int tupan_gb300_kepler_set_form(int form);

/* n independent pairs over dt: m[n], e2[n], state[n x 6] (relative r, v)
 * -> out[n x 6].  iters[n] (Laguerre updates), rec_x[n x 4] and rec_y[n]
 * (learned-start features and targets) may be NULL.  Synchronous. */
int tupan_gb300_kepler_pairs(uint64_t n, double dt, const double *m,
                             const double *e2, const double *state,
                             double *out, int *iters, float *rec_x,
                             float *rec_y, int use_mlp, long long budget,
                             void *stream);
/* sakura_kernel on device arrays: i_attrs / j_attrs are 8 pointers each in
 * the kernel's order (m, rx, ry, rz, e2, vx, vy, vz), outs 6 (drx .. dvz);
 * flag -1 or +1.  *n_kepler (host) receives the number of queued pairs;
 * kepler_iters (host, 65 bins, may be NULL) accumulates their update
 * counts.  mode 0 EXACT; 1 SPLIT: leapfrog-branch pairs in FP32 on
 * double-single positions, the Kepler branch in fp64.  Synchronous. */
int tupan_gb300_sakura_queue(uint64_t ni, const void *const *i_attrs,
                             uint64_t nj, const void *const *j_attrs,
                             double dt, int64_t flag, void *const *outs,
                             int use_mlp, long long budget, void *stream,
                             unsigned long long *n_kepler,
                             long long *kepler_iters, int mode);
/* Device-resident Sakura integrator (tupan/integrator/sakura.py:100-117,
 * fixed step): drift tau/2, two queued Sakura half-sweeps, drift tau/2. */
int tupan_gb300_sakura_create(uint64_t n, const double *m, const double *e2,
                              const double *rx, const double *ry,
                              const double *rz, const double *vx,
                              const double *vy, const double *vz,
                              void **handle);
int tupan_gb300_sakura_evolve(void *handle, double tau, double t_end,
                              int use_mlp, double *t_out,
                              long long *steps_out, long long *kepler_out,
                              long long *kepler_iters);
/* The integrator's Sakura sweeps: mode 0 EXACT (default), 1 SPLIT. */
int tupan_gb300_sakura_set_mode(void *handle, int mode);
int tupan_gb300_sakura_get_state(void *handle, double *rx, double *ry,
                                 double *rz, double *vx, double *vy,
                                 double *vz);
int tupan_gb300_sakura_destroy(void *handle);

/* ------------------------------------------------------------------------
 * Training kernels of the learned Kepler start (4 -> 64 -> 64 -> 1, SiLU),
 * libtupan_gb300.so only; no counterpart in the reference.  The parameter
 * vector is fp32 (tupan_gb300_mlp_param_count entries); the forward pass
 * uses bf16 weights with fp32 accumulation.  Device pointers throughout.
 * ---------------------------------------------------------------------- */
int tupan_gb300_mlp_param_count(void);
/* bf16 copies w1 w2 w3 of params' weights and rw = params with its weights
 * rounded through bf16 (what the forward pass computes with). */
int tupan_gb300_mlp_round(const float *params, void *w1, void *w2, void *w3,
                          float *rw, void *stream);
/* grad += d/dparams of scale * sum (net(X) - Y)^2 over n samples
 * (X: n x 4 raw features); *loss += the sum of squared errors. */
int tupan_gb300_mlp_grad(const float *rw, const float *norm, const float *X,
                         const float *Y, uint64_t n, float scale,
                         float *grad, float *loss, void *stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) at step >= 1; zeroes grad. */
int tupan_gb300_mlp_adam(float *params, float *m, float *v, float *grad,
                         float lr, int step, void *stream);

/* ------------------------------------------------------------------------
 * Ensembles (libtupan_gb300.so only; no counterpart in the reference, which
 * integrates one system per process).  n_sys independent systems of 1..512
 * particles each, concatenated in host arrays with offsets sys_off[n_sys +
 * 1]; every system takes its own shared adaptive Hermite-4 steps
 * (SPLIT forces), all systems advancing in one persistent sweep per force
 * evaluation.
 * ---------------------------------------------------------------------- */
int tupan_gb300_ensemble_create(unsigned n_sys, const uint64_t *sys_off,
                                double eta, const double *m, const double *e2,
                                const double *rx, const double *ry,
                                const double *rz, const double *vx,
                                const double *vy, const double *vz,
                                void **handle);
/* Steps every system to t_end, `batch` steps per graph replay; *max_steps_out
 * (host) receives the largest step count over systems. */
int tupan_gb300_ensemble_evolve(void *handle, double t_end, int batch,
                                long long *max_steps_out);
/* Per-system kinetic and potential energies (host arrays of n_sys). */
int tupan_gb300_ensemble_energy(void *handle, double *ke, double *pe);
/* Per-system time and step count (host, n_sys) and the concatenated state
 * (host, n). */
int tupan_gb300_ensemble_get(void *handle, double *t, long long *nsteps,
                             double *rx, double *ry, double *rz, double *vx,
                             double *vy, double *vz);
int tupan_gb300_ensemble_destroy(void *handle);
/* mode 0 (default): every step of every system is five batched launches.
 * mode 1: persistent launches in which one CTA steps one whole system for up
 * to steps_per_launch steps (records resident in shared memory, no
 * inter-CTA waits), until fewer than switch_below systems are left, which
 * finish in mode 0 (switch_below 0: persistent to the end). */
int tupan_gb300_ensemble_set_mode(void *handle, int mode, int steps_per_launch,
                                  int switch_below);
/* Launch shape of the batched sweep: nt threads per CTA (128: four CTAs per
 * SM; 256: two), ib the i-block of a work item while the active systems fill
 * the grid (32, 64, 128, 256 or 512; halved and quartered, not below 32, as
 * systems finish), prefetch 1 to copy the next item's records while the
 * current one computes.  handle NULL sets the default of ensembles created
 * later (the autotuner's table sets it on load).  A shape outside these
 * sets returns status 2 (bad argument). */
int tupan_gb300_ensemble_set_shape(void *handle, int nt, int ib, int prefetch);
int tupan_gb300_ensemble_get_shape(void *handle, int *nt, int *ib,
                                   int *prefetch);
/* split 1: the predictor/corrector after each AccJerk sweep runs as a
 * launch of its own over the step's work items; 0 (default, faster): inside
 * the sweep, by the CTA that computed each work item.  Results are
 * bit-identical. */
int tupan_gb300_ensemble_set_stage(void *handle, int split);

/* ------------------------------------------------------------------------
 * SIA integrators (libtupan_gb300.so only).  No counterpart in the
 * reference's C ABI: tupan/integrator/sia.py:965-1123 runs the recursion on
 * host arrays, copying the particle system at every split.  Here the system
 * stays in HBM, a split is a stable in-place partition of an index range,
 * and every force sweep runs on sub-ranges; with mode 0 (EXACT) a run is
 * bit-identical to the reference's except where a two-body subsystem calls
 * the Kepler solver.  Newtonian only.
 * ---------------------------------------------------------------------- */
/* method: "sia21s.dkd" .. "sia69h.kdk"; mode 0 EXACT, 1 SPLIT sweeps. */
int tupan_gb300_sia_create(uint64_t n, const char *method, double eta,
                           int mode, const double *m, const double *e2,
                           const double *rx, const double *ry,
                           const double *rz, const double *vx,
                           const double *vy, const double *vz,
                           void **handle);
/* Base steps until |t| >= t_end or max_steps (0: no limit); t_log (host,
 * may be NULL) receives the time after each step (at most log_cap).
 * Status 5: recursion deeper than 512 levels. */
int tupan_gb300_sia_evolve(void *handle, double t_end, long long max_steps,
                           double *t_out, long long *steps_out,
                           double *t_log, long long log_cap);
/* Current particle order (the reference's order after its joins). */
int tupan_gb300_sia_get_state(void *handle, long long *id, double *rx,
                              double *ry, double *rz, double *vx, double *vy,
                              double *vz, double *time, long long *nstep,
                              double *tstep);
/* stats[9]: recursion calls, Kepler solves, host-launched sweeps,
 * partitions, deepest level, base steps, single-CTA subtree launches, the
 * microseconds spent in them, and the pair interactions summed (ni * nj of
 * every Acc and Tstep sum). */
int tupan_gb300_sia_stats(void *handle, long long *stats);
/* Subsystems of at most max_n (0 .. 128) particles run the rest of their
 * recursion inside one CTA, staged in shared memory; 0 drives every level
 * from the host.  Both paths give the same bits.  Returns the previous
 * value, or -1 for a bad argument. */
int tupan_gb300_sia_set_subtree(void *handle, int max_n);
int tupan_gb300_sia_destroy(void *handle);

/* ------------------------------------------------------------------------
 * NREG integrators (libtupan_gb300.so only).  No counterpart in the
 * reference's C ABI: tupan/integrator/nreg.py runs the regularised-time
 * recurrences on host arrays around the nreg_X / nreg_V kernels.  Here the
 * particles stay in HBM; sums are taken in numpy's pairwise order, so a run
 * is bit-identical to the reference's.
 * ---------------------------------------------------------------------- */
/* anreg 0: "nreg", 1: "anreg".  Host arrays are copied in. */
int tupan_gb300_nreg_create(uint64_t n, int anreg, double eta,
                            const double *m, const double *e2,
                            const double *rx, const double *ry,
                            const double *rz, const double *vx,
                            const double *vy, const double *vz,
                            void **handle);
/* Steps until |t| >= t_end or max_steps (0: no limit); t_log (host, may be
 * NULL) receives the time after each step (at most log_cap). */
int tupan_gb300_nreg_evolve(void *handle, double t_end, long long max_steps,
                            double *t_out, long long *steps_out,
                            double *t_log, long long log_cap);
/* State (host arrays of n, may be NULL) and scalars[5] = {W, U, S, E0, t}. */
int tupan_gb300_nreg_get_state(void *handle, double *rx, double *ry,
                               double *rz, double *vx, double *vy,
                               double *vz, double *scalars);
int tupan_gb300_nreg_destroy(void *handle);

#ifdef __cplusplus
}
#endif

#endif /* TUPAN_GB300_H */
