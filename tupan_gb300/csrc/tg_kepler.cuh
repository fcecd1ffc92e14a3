// Universal-variable two-body propagator and the Sakura pair kernel
// (tupan/lib/src/universal_kepler_solver.h, sakura_kernel_common.h,
// kepler_solver_kernel_common.h) in REAL precision.
//
// Same steps and order of operations as the reference.  Two differences:
//  * cos/sin/cosh/sinh/log are CUDA's, not the host libm: results may differ
//    from the reference C in the last bits (the leapfrog branch, which uses
//    only + - * / sqrt, stays bit-identical);
//  * the reference's retry loops (step halving on solver failure and the
//    energy-check subdivision, universal_kepler_solver.h:486-499 and
//    :580-606) have no bound; here one pair solve may spend at most
//    `budget` single-step solves, after which the pair keeps its last state
//    and DERR_KEPLER_BUDGET is raised in the error word.
// An optional learned start replaces the plain first guess s0 = dt/r; the
// Laguerre iteration and its stopping rule are unchanged.
#pragma once

#include "tg_pairs.cuh"

namespace tg {

template <typename R> struct KeplerTol;
template <> struct KeplerTol<double> {
    __device__ static double v() { return 2.2737367544323205948e-13; }  // 2^-42
};
template <> struct KeplerTol<float> {
    __device__ static float v() { return 1.52587890625e-5f; }           // 2^-16
};

constexpr int KEPLER_MAXITER = 64;
// Laguerre updates allowed from a learned start before the solve falls back
// to the plain guess (the plain guess needs at most a handful on the
// Kepler-branch pairs of a Sakura step: mean 2.0 at dt = 1/512, 2.8 at 1/8).
constexpr int KEPLER_LEARNED_MAXITER = 8;
constexpr int KEPLER_MAX_HALVINGS = 40;

template <typename R>
__device__ __forceinline__ int sgn(R x) { return (x > R(0)) - (x < R(0)); }

// Stumpff functions, universal_kepler_solver.h:17-79
template <typename R>
__device__ R stumpff0(R z)
{
    if (z < R(0)) return cos(sqrt(-z));
    if (z > R(0)) return cosh(sqrt(z));
    return R(1);
}
template <typename R>
__device__ R stumpff1(R z)
{
    if (z < R(0)) { R w = sqrt(-z); return sin(w) / w; }
    if (z > R(0)) { R w = sqrt(z); return sinh(w) / w; }
    return R(1);
}
template <typename R>
__device__ R stumpff2(R z)
{
    if (z < R(0)) { R w = sqrt(-z); return (cos(w) - R(1)) / z; }
    if (z > R(0)) { R w = sqrt(z); return (cosh(w) - R(1)) / z; }
    return R(1) / R(2);
}
template <typename R>
__device__ R stumpff3(R z)
{
    if (z < R(0)) { R w = sqrt(-z); return (sin(w) / w - R(1)) / z; }
    if (z > R(0)) { R w = sqrt(z); return (sinh(w) / w - R(1)) / z; }
    return R(1) / R(6);
}

// S0..S3, universal_kepler_solver.h:82-120
template <typename R> __device__ __forceinline__ R kS0(R s, R al) { R s2 = s * s; return stumpff0(al * s2); }
template <typename R> __device__ __forceinline__ R kS1(R s, R al) { R s2 = s * s; return s * stumpff1(al * s2); }
template <typename R> __device__ __forceinline__ R kS2(R s, R al) { R s2 = s * s; return s2 * stumpff2(al * s2); }
template <typename R> __device__ __forceinline__ R kS3(R s, R al)
{
    R s2 = s * s;
    R s3 = s * s2;
    return s3 * stumpff3(al * s2);
}

template <typename R>
struct KepArg { R dt, r0, rv0, m, al; };

// universal_kepler{,_ds,_dsds}, universal_kepler_solver.h:166-222
template <typename R>
__device__ __forceinline__ R kep_f(R s, const KepArg<R> &k)
{
    return (k.r0 * s + k.rv0 * kS2(s, k.al) + (k.m + k.al * k.r0) * kS3(s, k.al)) - k.dt;
}
template <typename R>
__device__ __forceinline__ R kep_df(R s, const KepArg<R> &k)
{
    return k.r0 + k.rv0 * kS1(s, k.al) + (k.m + k.al * k.r0) * kS2(s, k.al);
}
template <typename R>
__device__ __forceinline__ R kep_ddf(R s, const KepArg<R> &k)
{
    return k.rv0 * kS0(s, k.al) + (k.m + k.al * k.r0) * kS1(s, k.al);
}

// Laguerre iteration of order 5, universal_kepler_solver.h:225-254.
template <typename R>
__device__ int kep_laguerre(R x0, R *x, const KepArg<R> &k, int *iters,
                            int maxit = KEPLER_MAXITER)
{
    const int ORDER = 5;
    int it = 0;
    R delta;
    *x = x0;
    do {
        R fv = kep_f(*x, k);
        R dfv = kep_df(*x, k);
        R ddfv = kep_ddf(*x, k);
        R a = dfv;
        R a2 = a * a;
        R b = a2 - fv * ddfv;
        R g = R(ORDER) * fv;
        R h = a + R(sgn(a)) * sqrt(fabs(R(ORDER - 1) * (R(ORDER) * b - a2)));
        if (h == R(0)) { *iters = it; return -1; }
        delta = -g / h;
        *x += delta;
        it += 1;
        if (it > maxit) { *iters = it; return -2; }
    } while (fabs(delta) > KeplerTol<R>::v());
    *iters = it;
    if (sgn(*x) != sgn(x0)) return -3;
    return 0;
}

// set_new_pos_vel, universal_kepler_solver.h:312-357, from S1..S3 at the root
template <typename R>
__device__ void kep_update_S(R dt, const R *S, R r0, R m, R e2, R *p)
{
    R r0x = p[0], r0y = p[1], r0z = p[2];
    R v0x = p[3], v0y = p[4], v0z = p[5];
    R lf = R(1) - m * S[2] / r0;
    R lg = dt - m * S[3];
    R r1x = r0x * lf + v0x * lg;
    R r1y = r0y * lf + v0y * lg;
    R r1z = r0z * lf + v0z * lg;
    R r1sq = r1x * r1x + r1y * r1y + r1z * r1z;
    R r1 = sqrt(r1sq + e2);
    R ldf = -m * S[1] / (r0 * r1);
    R ldg = (R(1) + lg * ldf) / lf;
    p[0] = r1x;
    p[1] = r1y;
    p[2] = r1z;
    p[3] = r0x * ldf + v0x * ldg;
    p[4] = r0y * ldf + v0y * ldg;
    p[5] = r0z * ldf + v0z * ldg;
}

// set_new_pos_vel, universal_kepler_solver.h:312-357
template <typename R>
__device__ void kep_update(R dt, R s, R r0, R m, R e2, R al, R *p)
{
    R r0x = p[0], r0y = p[1], r0z = p[2];
    R v0x = p[3], v0y = p[4], v0z = p[5];
    R lf = R(1) - m * kS2(s, al) / r0;
    R lg = dt - m * kS3(s, al);
    R r1x = r0x * lf + v0x * lg;
    R r1y = r0y * lf + v0y * lg;
    R r1z = r0z * lf + v0z * lg;
    R r1sq = r1x * r1x + r1y * r1y + r1z * r1z;
    R r1 = sqrt(r1sq + e2);
    R ldf = -m * kS1(s, al) / (r0 * r1);
    R ldg = (R(1) + lg * ldf) / lf;
    p[0] = r1x;
    p[1] = r1y;
    p[2] = r1z;
    p[3] = r0x * ldf + v0x * ldg;
    p[4] = r0y * ldf + v0y * ldg;
    p[5] = r0z * ldf + v0z * ldg;
}

// ---------------------------------------------------------------------------
// Forms of the single-step root solve.
//   KEP_REFERENCE  the reference's structure: each of S0..S3 evaluates its own
//                  sqrt and cos/sin (or cosh/sinh), six per Laguerre update.
//   KEP_SHARED     the same arithmetic with cos/sin (cosh/sinh) of the one
//                  argument of an update evaluated once: bit-identical roots
//                  and states, a sixth of the transcendentals.
//   KEP_MIXED      Laguerre updates in FP32 (Stumpff c2, c3 from their power
//                  series where the closed forms cancel), then FP64 Laguerre
//                  updates until the predicted next update is below the
//                  reference's tolerance, and S1..S3 at the root by a Taylor
//                  shift from the last FP64 evaluation: about one FP64
//                  cos/sin per solve.
// ---------------------------------------------------------------------------
enum KeplerForm : int { KEP_REFERENCE = 0, KEP_SHARED = 1, KEP_MIXED = 2 };

// Per-solve bookkeeping: budget, counters and the optional learned start.
template <typename R>
struct KepCtx {
    long long solves;      // single-step solves spent on this pair solve
    long long budget;      // upper bound on `solves`
    long long iterations;  // Laguerre updates summed (FP64 updates, KEP_MIXED)
    bool exhausted;
    bool use_start;        // take `start` instead of dt/r on the first try
    R start;
    int form = KEP_REFERENCE;
    long long iterations32 = 0;   // FP32 updates (KEP_MIXED)
    long long fallbacks = 0;      // learned starts redone from the plain guess
};

// Stumpff c0..c3 of z from one transcendental evaluation: the reference's
// closed forms (universal_kepler_solver.h:17-79) with cos(w), sin(w) (or
// cosh, sinh) of w = sqrt(|z|) computed once; each value is the one the
// separate functions return.
template <typename R>
__device__ __forceinline__ void stumpff_all(R z, R *c)
{
    if (z < R(0)) {
        const R w = sqrt(-z);
        const R cw = cos(w), sw = sin(w);
        const R s1 = sw / w;
        c[0] = cw;
        c[1] = s1;
        c[2] = (cw - R(1)) / z;
        c[3] = (s1 - R(1)) / z;
    } else if (z > R(0)) {
        const R w = sqrt(z);
        const R cw = cosh(w), sw = sinh(w);
        const R s1 = sw / w;
        c[0] = cw;
        c[1] = s1;
        c[2] = (cw - R(1)) / z;
        c[3] = (s1 - R(1)) / z;
    } else {
        c[0] = R(1);
        c[1] = R(1);
        c[2] = R(1) / R(2);
        c[3] = R(1) / R(6);
    }
}

// S0..S3 at s (the products of kS0..kS3, universal_kepler_solver.h:82-120).
template <typename R>
__device__ __forceinline__ void kep_S(R s, R al, R *S)
{
    R c[4];
    const R s2 = s * s;
    stumpff_all(al * s2, c);
    S[0] = c[0];
    S[1] = s * c[1];
    S[2] = s2 * c[2];
    S[3] = (s * s2) * c[3];
}

// f, f', f'' of universal_kepler{,_ds,_dsds} from precomputed S values.
template <typename R>
__device__ __forceinline__ void kep_fdd(const R *S, R s, const KepArg<R> &k,
                                        R *f, R *df, R *ddf)
{
    const R b = k.m + k.al * k.r0;
    *f = (k.r0 * s + k.rv0 * S[2] + b * S[3]) - k.dt;
    *df = k.r0 + k.rv0 * S[1] + b * S[2];
    *ddf = k.rv0 * S[0] + b * S[1];
}

// One Laguerre update of order 5 (universal_kepler_solver.h:233-243);
// false when the denominator vanishes.
template <typename R>
__device__ __forceinline__ bool lag_delta(R fv, R dfv, R ddfv, R *delta)
{
    const int ORDER = 5;
    const R a = dfv;
    const R a2 = a * a;
    const R b = a2 - fv * ddfv;
    const R g = R(ORDER) * fv;
    const R h = a + R(sgn(a)) * sqrt(fabs(R(ORDER - 1) * (R(ORDER) * b - a2)));
    if (h == R(0)) return false;
    *delta = -g / h;
    return true;
}

// kep_laguerre with one S evaluation per update (KEP_SHARED).
template <typename R>
__device__ int kep_laguerre_shared(R x0, R *x, const KepArg<R> &k, int *iters,
                                   int maxit = KEPLER_MAXITER)
{
    int it = 0;
    R delta;
    *x = x0;
    do {
        R S[4], fv, dfv, ddfv;
        kep_S(*x, k.al, S);
        kep_fdd(S, *x, k, &fv, &dfv, &ddfv);
        if (!lag_delta(fv, dfv, ddfv, &delta)) { *iters = it; return -1; }
        *x += delta;
        it += 1;
        if (it > maxit) { *iters = it; return -2; }
    } while (fabs(delta) > KeplerTol<R>::v());
    *iters = it;
    if (sgn(*x) != sgn(x0)) return -3;
    return 0;
}

// FP32 Stumpff c0..c3 for the mixed form's first stage.  For |z| < 1 the
// closed forms (cos w - 1) / z and (sin w / w - 1) / z lose most of FP32's
// digits to cancellation; there c2 and c3 come from their power series
// c_k(z) = sum_n z^n / (2n + k)! (positive z is the hyperbolic branch, as
// in the closed forms; eight terms: the next is below 2^-24 relative), and
// c0 = 1 + z c2, c1 = 1 + z c3.  Elsewhere the closed forms, with cos/sin
// (cosh/sinh) evaluated once.
__device__ __forceinline__ void stumpff_all_f32(float z, float *c)
{
    if (fabsf(z) < 1.0f) {
        // Horner from the eighth term: c2 = 1/2! + z/4! + z^2/6! + ...,
        // c3 = 1/3! + z/5! + z^2/7! + ...
        float c2 = 1.0f / 20922789888000.0f;   // 1/16!
        float c3 = 1.0f / 355687428096000.0f;  // 1/17!
        c2 = __fmaf_rn(c2, z, 1.0f / 87178291200.0f);    // 1/14!
        c3 = __fmaf_rn(c3, z, 1.0f / 1307674368000.0f);  // 1/15!
        c2 = __fmaf_rn(c2, z, 1.0f / 479001600.0f);      // 1/12!
        c3 = __fmaf_rn(c3, z, 1.0f / 6227020800.0f);     // 1/13!
        c2 = __fmaf_rn(c2, z, 1.0f / 3628800.0f);        // 1/10!
        c3 = __fmaf_rn(c3, z, 1.0f / 39916800.0f);       // 1/11!
        c2 = __fmaf_rn(c2, z, 1.0f / 40320.0f);          // 1/8!
        c3 = __fmaf_rn(c3, z, 1.0f / 362880.0f);         // 1/9!
        c2 = __fmaf_rn(c2, z, 1.0f / 720.0f);            // 1/6!
        c3 = __fmaf_rn(c3, z, 1.0f / 5040.0f);           // 1/7!
        c2 = __fmaf_rn(c2, z, 1.0f / 24.0f);             // 1/4!
        c3 = __fmaf_rn(c3, z, 1.0f / 120.0f);            // 1/5!
        c2 = __fmaf_rn(c2, z, 0.5f);                     // 1/2!
        c3 = __fmaf_rn(c3, z, 1.0f / 6.0f);              // 1/3!
        c[0] = __fmaf_rn(z, c2, 1.0f);
        c[1] = __fmaf_rn(z, c3, 1.0f);
        c[2] = c2;
        c[3] = c3;
    } else if (z < 0.0f) {
        const float w = sqrtf(-z);
        float sw, cw;
        sincosf(w, &sw, &cw);
        const float s1 = sw / w;
        c[0] = cw;
        c[1] = s1;
        c[2] = (cw - 1.0f) / z;
        c[3] = (s1 - 1.0f) / z;
    } else {
        const float w = sqrtf(z);
        const float cw = coshf(w), sw = sinhf(w);
        const float s1 = sw / w;
        c[0] = cw;
        c[1] = s1;
        c[2] = (cw - 1.0f) / z;
        c[3] = (s1 - 1.0f) / z;
    }
}

// FP32 Laguerre updates from x0 until |delta| <= 2^-20 |x| (FP32 cannot
// resolve the root much better: f is a difference of terms of size dt).
// Returns 0, or -1 / -2 (vanishing denominator or a value that is not
// finite, no convergence in 16 updates).
__device__ inline int kep_laguerre_f32(float x0, float *x,
                                       const KepArg<float> &k, int *iters)
{
    int it = 0;
    float s = x0, delta;
    const float b = k.m + k.al * k.r0;
    do {
        float c[4];
        const float s2 = s * s;
        stumpff_all_f32(k.al * s2, c);
        const float S1 = s * c[1], S2 = s2 * c[2], S3 = (s * s2) * c[3];
        const float fv = __fmaf_rn(k.r0, s, __fmaf_rn(k.rv0, S2, __fmaf_rn(b, S3, -k.dt)));
        const float dfv = k.r0 + __fmaf_rn(k.rv0, S1, b * S2);
        const float ddfv = __fmaf_rn(k.rv0, c[0], b * S1);
        if (!lag_delta(fv, dfv, ddfv, &delta) || !isfinite(delta)) {
            *iters = it;
            return -1;
        }
        s += delta;
        it += 1;
        if (it >= 16) { *iters = it; return -2; }
    } while (fabsf(delta) > 9.5367431640625e-7f * fabsf(s));   // 2^-20
    *x = s;
    *iters = it;
    return 0;
}

// KEP_MIXED root: FP32 stage from x0, then FP64 Laguerre updates.  An FP64
// update d is accepted when |d| <= 2^-42 (the reference's rule) or when the
// next update it predicts, |f'' / (2 f')| d^2 (Newton's quadratic bound;
// Laguerre's order-5 update converges at least as fast), is below a quarter
// of 2^-42: the root then lies within that bound of the reference's.
// S[1..3] receive S1..S3 at the root, shifted from the last evaluation point
// by their Taylor series in d (dS_{k+1}/ds = S_k, dS_0/ds = al S_1) to
// second order when |d| <= 2^-20 |s| (the third-order term is then below
// double rounding), else evaluated at the root.
__device__ inline int kep_laguerre_mixed(double x0, double *x,
                                         const KepArg<double> &k, int *iters,
                                         int *iters32, double *S,
                                         int maxit = KEPLER_MAXITER)
{
    const double tol = KeplerTol<double>::v();
    KepArg<float> kf = {(float)k.dt, (float)k.r0, (float)k.rv0, (float)k.m,
                        (float)k.al};
    float xf = 0.f;
    int n32 = 0;
    double s = x0;
    if (kep_laguerre_f32((float)x0, &xf, kf, &n32) == 0 &&
        sgn((double)xf) == sgn(x0))
        s = (double)xf;
    *iters32 = n32;
    int it = 0;
    for (;;) {
        double Sp[4], fv, dfv, ddfv, delta;
        kep_S(s, k.al, Sp);
        kep_fdd(Sp, s, k, &fv, &dfv, &ddfv);
        if (!lag_delta(fv, dfv, ddfv, &delta)) { *iters = it; return -1; }
        s += delta;
        it += 1;
        const bool done =
            fabs(delta) <= tol ||
            fabs(ddfv / (2.0 * dfv)) * (delta * delta) <= 0.25 * tol;
        if (done) {
            if (fabs(delta) <= 9.5367431640625e-7 * fabs(s)) {   // 2^-20 |s|
                const double d = delta, h = 0.5 * delta * delta;
                S[1] = Sp[1] + d * Sp[0] + h * (k.al * Sp[1]);
                S[2] = Sp[2] + d * Sp[1] + h * Sp[0];
                S[3] = Sp[3] + d * Sp[2] + h * Sp[1];
            } else {
                // a large last update (an FP32 stage that did not converge):
                // the Taylor shift would not be exact enough, evaluate
                kep_S(s, k.al, S);
            }
            break;
        }
        if (it > maxit) { *iters = it; return -2; }
    }
    *x = s;
    *iters = it;
    if (sgn(*x) != sgn(x0)) return -3;
    return 0;
}

// Plain first guess of _universal_kepler_solver (:405-425) and the quantities
// it derives; returns false for a zero separation (no motion, :384-394).
template <typename R>
__device__ bool kep_setup(R dt0, R m, R e2, const R *p, KepArg<R> *ka, R *s0)
{
    R rx = p[0], ry = p[1], rz = p[2];
    R vx = p[3], vy = p[4], vz = p[5];
    R r2 = rx * rx + ry * ry + rz * rz;
    if (!(r2 > R(0))) return false;
    r2 += e2;
    R r = sqrt(r2);
    R v2 = vx * vx + vy * vy + vz * vz;
    R rv = rx * vx + ry * vy + rz * vz;
    R beta = R(2) - (e2 / r2);
    R al = v2 - beta * m / r;
    R dt = dt0;
    if (al < R(0)) {
        R a = m / fabs(al);
        R T = R(2) * R(3.141592653589793) * a * sqrt(a / m);
        R ratio = dt0 / T;
        dt = (ratio - R((long long)(ratio))) * T;
    }
    R g = dt / r;
    if (al > R(0)) {
        R sal = sqrt(al);
        R ss = fabs(R(2) * al * dt / (rv + (m + al * r) / sal));
        if (ss > R(1)) g = R(sgn(dt)) * log(ss) / sal;
    }
    ka->dt = dt;
    ka->r0 = r;
    ka->rv0 = rv;
    ka->m = m;
    ka->al = al;
    *s0 = g;
    return true;
}

// _universal_kepler_solver, universal_kepler_solver.h:360-463.  A learned
// start is taken only inside a trust region around the plain guess, and
// gets KEPLER_LEARNED_MAXITER updates; a solve from it that has not
// converged by then (or fails) is redone from the plain guess, so the plain
// iteration stays the fallback and judges the network's guess.
template <typename R>
__device__ int kep_single(R dt0, R m, R e2, R *p, KepCtx<R> &c)
{
    for (;;) {
        if (c.solves >= c.budget) { c.exhausted = true; return -4; }
        KepArg<R> ka;
        R s0;
        if (!kep_setup(dt0, m, e2, p, &ka, &s0)) return 0;
        bool learned = false;
        if (c.use_start) {
            // A learned start must keep the plain guess's sign (the
            // reference rejects roots whose sign differs from the start,
            // :252) and stay where the Stumpff functions are well scaled:
            // w = sqrt|al| s (the eccentric or hyperbolic anomaly swept) at
            // most 4 times the plain guess's or 8 (a bound orbit sweeps
            // less than 2 pi after the period reduction).  Far beyond, cosh
            // and sinh reach 1e150 and a cancelling f can pass the stopping
            // rule at a wrong root.
            const R sal = sqrt(fabs(ka.al));
            if (sgn(c.start) == sgn(s0) && isfinite(c.start) &&
                sal * fabs(c.start) <= fmax(R(4) * sal * fabs(s0), R(8))) {
                s0 = c.start;
                learned = true;
            }
            c.use_start = false;
        }
        const int maxit = learned ? KEPLER_LEARNED_MAXITER : KEPLER_MAXITER;
        R s;
        int it = 0;
        int err;
        bool done = false;
        if constexpr (sizeof(R) == sizeof(double)) {
            if (c.form == KEP_MIXED) {
                R S[4];
                int it32 = 0;
                err = kep_laguerre_mixed(s0, &s, ka, &it, &it32, S, maxit);
                c.solves += 1;
                c.iterations += it;
                c.iterations32 += it32;
                if (err == 0) kep_update_S(ka.dt, S, ka.r0, m, e2, p);
                done = true;
            }
        }
        if (!done && c.form == KEP_SHARED) {
            err = kep_laguerre_shared(s0, &s, ka, &it, maxit);
            c.solves += 1;
            c.iterations += it;
            if (err == 0) {
                R S[4];
                kep_S(s, ka.al, S);
                kep_update_S(ka.dt, S, ka.r0, m, e2, p);
            }
            done = true;
        }
        if (!done) {
            err = kep_laguerre(s0, &s, ka, &it, maxit);
            c.solves += 1;
            c.iterations += it;
            if (err == 0) kep_update(ka.dt, s, ka.r0, m, e2, ka.al, p);
        }
        if (err != 0 && learned) {
            c.fallbacks += 1;
            continue;          // p unchanged; the plain guess takes over
        }
        return err;
    }
}

// __universal_kepler_solver, universal_kepler_solver.h:466-507
template <typename R>
__device__ void kep_substeps(R dt, R m, R e2, const R *p0, R *p, KepCtx<R> &c)
{
    long long n = 1;
    for (int h = 0; h <= KEPLER_MAX_HALVINGS; ++h, n *= 2) {
        for (int q = 0; q < 6; ++q) p[q] = p0[q];
        long long i;
        for (i = 0; i < n; ++i)
            if (kep_single(dt / R(n), m, e2, p, c) != 0) break;
        if (i == n) return;
        if (c.solves >= c.budget) break;
    }
    c.exhausted = true;
}

// universal_kepler_solver, universal_kepler_solver.h:510-614
template <typename R>
__device__ void kep_solve(R dt, R m, R e2, const R *p0, R *p1, KepCtx<R> &c)
{
    R p[6];
    kep_substeps(dt, m, e2, p0, p, c);
    if (e2 == R(0)) {
        for (int q = 0; q < 6; ++q) p1[q] = p[q];
        return;
    }
    R r2 = p0[0] * p0[0] + p0[1] * p0[1] + p0[2] * p0[2];
    if (!(r2 > R(0))) {
        for (int q = 0; q < 6; ++q) p1[q] = p0[q];
        return;
    }
    r2 += e2;
    R r = sqrt(r2);
    R v2 = p0[3] * p0[3] + p0[4] * p0[4] + p0[5] * p0[5];
    R u0 = R(2) * m / r;
    R e0 = v2 - u0;
    r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    r2 += e2;
    r = sqrt(r2);
    v2 = p[3] * p[3] + p[4] * p[4] + p[5] * p[5];
    R u1 = R(2) * m / r;
    R e1 = v2 - u1;
    R tol = R(64) * KeplerTol<R>::v();
    R err = fabs(e1 - e0);
    if (R(2) * err < tol * (u1 + u0)) {
        for (int q = 0; q < 6; ++q) p1[q] = p[q];
        return;
    }
    long long n = 1;
    for (int h = 0; h < KEPLER_MAX_HALVINGS; ++h) {
        n *= 2;
        for (int q = 0; q < 6; ++q) p[q] = p0[q];
        long long i;
        for (i = 0; i < n; ++i) {
            R qv[6];
            for (int q = 0; q < 6; ++q) qv[q] = p[q];
            kep_substeps(dt / R(n), m, e2, qv, p, c);
            r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
            r2 += e2;
            r = sqrt(r2);
            v2 = p[3] * p[3] + p[4] * p[4] + p[5] * p[5];
            u1 = R(2) * m / r;
            e1 = v2 - u1;
            err = fabs(e1 - e0);
            if (R(2) * err > tol * (u1 + u0)) break;
        }
        if (i == n) {
            for (int q = 0; q < 6; ++q) p1[q] = p[q];
            return;
        }
        if (c.solves >= c.budget) break;
    }
    c.exhausted = true;
    for (int q = 0; q < 6; ++q) p1[q] = p[q];
}

// leapfrog + get_acc, sakura_kernel_common.h:24-91
template <typename R>
__device__ void two_body_leapfrog(R dt, R m, R e2, const R *p0, R *p1)
{
    R half = dt / R(2);
    R rx = p0[0], ry = p0[1], rz = p0[2];
    R vx = p0[3], vy = p0[4], vz = p0[5];
    rx += vx * half;
    ry += vy * half;
    rz += vz * half;
    R r2 = rx * rx + ry * ry + rz * rz;
    R q = masked_inv_r2(r2, e2);
    R k = q * sqrt(q);
    R mk = m * k;
    R ax = -mk * rx, ay = -mk * ry, az = -mk * rz;
    vx += ax * dt;
    vy += ay * dt;
    vz += az * dt;
    rx += vx * half;
    ry += vy * half;
    rz += vz * half;
    p1[0] = rx; p1[1] = ry; p1[2] = rz;
    p1[3] = vx; p1[4] = vy; p1[5] = vz;
}

// Branch test of twobody_solver, sakura_kernel_common.h:111-114
template <typename R>
__device__ __forceinline__ bool takes_leapfrog(R m, const R *p0)
{
    R r2 = p0[0] * p0[0] + p0[1] * p0[1] + p0[2] * p0[2];
    R v2 = p0[3] * p0[3] + p0[4] * p0[4] + p0[5] * p0[5];
    R Rr = R(64) * (m / v2);
    return r2 > Rr * Rr;
}

template <typename R>
__device__ void two_body(R dt, R m, R e2, const R *p0, R *p1, KepCtx<R> &c)
{
    if (takes_leapfrog(m, p0)) {
        two_body_leapfrog(dt, m, e2, p0, p1);
    } else {
        c.solves = 0;
        kep_solve(dt, m, e2, p0, p1, c);
    }
}

// evolve_twobody, sakura_kernel_common.h:126-191
template <typename R>
__device__ void evolve_pair(R dt, long long flag, R m, R e2, const R *p0,
                            R *p1, KepCtx<R> &c)
{
    R p[6], q[6];
    for (int k = 0; k < 6; ++k) p[k] = p0[k];
    if (flag == -1) {
        p[0] -= p[3] * dt;
        p[1] -= p[4] * dt;
        p[2] -= p[5] * dt;
        two_body(dt, m, e2, p, q, c);
        for (int k = 0; k < 6; ++k) p[k] = q[k];
    }
    if (flag == 1) {
        two_body(dt, m, e2, p, q, c);
        for (int k = 0; k < 6; ++k) p[k] = q[k];
        p[0] -= p[3] * dt;
        p[1] -= p[4] * dt;
        p[2] -= p[5] * dt;
    }
    if (flag == -2) {
        p[0] -= p[3] * dt / R(2);
        p[1] -= p[4] * dt / R(2);
        p[2] -= p[5] * dt / R(2);
        two_body(dt, m, e2, p, q, c);
        for (int k = 0; k < 6; ++k) p[k] = q[k];
        p[0] -= p[3] * dt / R(2);
        p[1] -= p[4] * dt / R(2);
        p[2] -= p[5] * dt / R(2);
    }
    if (flag == 2) {
        two_body(dt / R(2), m, e2, p, q, c);
        for (int k = 0; k < 6; ++k) p[k] = q[k];
        p[0] -= p[3] * dt;
        p[1] -= p[4] * dt;
        p[2] -= p[5] * dt;
        two_body(dt / R(2), m, e2, p, q, c);
        for (int k = 0; k < 6; ++k) p[k] = q[k];
    }
    for (int k = 0; k < 6; ++k) p1[k] = p[k];
}

// Relative state of an (i, j) pair and its total mass / softening.
template <typename R>
__device__ __forceinline__ void pair_state(const R *ip, const R *jp, R *p0,
                                           R *m, R *e2)
{
    p0[0] = ip[1] - jp[1];
    p0[1] = ip[2] - jp[2];
    p0[2] = ip[3] - jp[3];
    *e2 = ip[4] + jp[4];
    p0[3] = ip[5] - jp[5];
    p0[4] = ip[6] - jp[6];
    p0[5] = ip[7] - jp[7];
    *m = ip[0] + jp[0];
}

// kepler_solver_kernel_common.h:39-79: particles a and b (m r e2 v) evolved
// over dt in their centre-of-mass frame; a1/b1 receive r and v (6 each) and
// may alias nothing the caller still needs from a or b.
template <typename R>
__device__ void kepler_two_body(const R *a, const R *b, R dt, R *a1, R *b1,
                                KepCtx<R> &ctx)
{
    R p0[6], p1[6], m, e2;
    pair_state(a, b, p0, &m, &e2);
    R amu = a[0] / m;
    R bmu = b[0] / m;
    R cm[6];
    for (int c = 0; c < 3; ++c) cm[c] = amu * a[1 + c] + bmu * b[1 + c];
    for (int c = 0; c < 3; ++c) cm[3 + c] = amu * a[5 + c] + bmu * b[5 + c];
    for (int c = 0; c < 3; ++c) cm[c] += cm[3 + c] * dt;
    kep_solve(dt, m, e2, p0, p1, ctx);
    for (int q = 0; q < 6; ++q) {
        a1[q] = cm[q] + bmu * p1[q];
        b1[q] = cm[q] - amu * p1[q];
    }
}

}  // namespace tg
