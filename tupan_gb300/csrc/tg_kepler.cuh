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
__device__ int kep_laguerre(R x0, R *x, const KepArg<R> &k, int *iters)
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
        if (it > KEPLER_MAXITER) { *iters = it; return -2; }
    } while (fabs(delta) > KeplerTol<R>::v());
    *iters = it;
    if (sgn(*x) != sgn(x0)) return -3;
    return 0;
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

// Per-solve bookkeeping: budget, counters and the optional learned start.
template <typename R>
struct KepCtx {
    long long solves;      // single-step solves spent on this pair solve
    long long budget;      // upper bound on `solves`
    long long iterations;  // Laguerre updates summed
    bool exhausted;
    bool use_start;        // take `start` instead of dt/r on the first try
    R start;
};

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

// _universal_kepler_solver, universal_kepler_solver.h:360-463
template <typename R>
__device__ int kep_single(R dt0, R m, R e2, R *p, KepCtx<R> &c)
{
    if (c.solves >= c.budget) { c.exhausted = true; return -4; }
    KepArg<R> ka;
    R s0;
    if (!kep_setup(dt0, m, e2, p, &ka, &s0)) return 0;
    if (c.use_start) {
        // A learned start must keep the plain guess's sign: the reference
        // rejects roots whose sign differs from the start (:252).
        if (sgn(c.start) == sgn(s0) && isfinite(c.start)) s0 = c.start;
        c.use_start = false;
    }
    R s;
    int it = 0;
    int err = kep_laguerre(s0, &s, ka, &it);
    c.solves += 1;
    c.iterations += it;
    if (err == 0) kep_update(ka.dt, s, ka.r0, m, e2, ka.al, p);
    return err;
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
