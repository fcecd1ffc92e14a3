// Pair arithmetic of the tupan kernels in REAL precision (double or float),
// evaluated in the same order as the reference C so that, compiled without
// multiply-add contraction (-fmad=false) and with IEEE division and square
// root (nvcc's defaults), every pair term rounds exactly as in
// tupan/lib/src/*_common.h.  Used by the EXACT sweeps and by Sakura/Kepler.
//
// Attribute order of a particle record p[]: m, rx, ry, rz, e2, vx, vy, vz,
// ax, ay, az, jx, jy, jz (NREG_V: m, vx, vy, vz, ax, ay, az).
#pragma once

#include "tg_common.cuh"

namespace tg {

template <typename R>
__device__ __forceinline__ R masked_inv_r2(R r2, R h2)
{
    // smoothing.h:10-184: 1/(r2+h2), zeroed where r2 == 0 (self pairs)
    R q = R(1) / (r2 + h2);
    return (r2 > R(0)) ? q : R(0);
}

// phi_kernel_common.h:7-32
template <typename R>
struct PhiPair {
    static constexpr int NA = 5, NO = 1;
    __device__ static void init(R *o) { o[0] = R(0); }
    __device__ static void pair(const R *ip, const R *jp, R *o, const Sweep &)
    {
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R r2 = dx * dx + dy * dy + dz * dz;
        R q = masked_inv_r2(r2, h2);
        R inv_r1 = sqrt(q);
        o[0] -= jp[0] * inv_r1;
    }
    __device__ static void finish(const R *, R *, const Sweep &) {}
};

// acc_kernel_common.h:7-38
template <typename R>
struct AccPair {
    static constexpr int NA = 5, NO = 3;
    __device__ static void init(R *o) { o[0] = o[1] = o[2] = R(0); }
    __device__ static void pair(const R *ip, const R *jp, R *o, const Sweep &)
    {
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R r2 = dx * dx + dy * dy + dz * dz;
        R q = masked_inv_r2(r2, h2);
        R k = q * sqrt(q);
        k *= jp[0];
        o[0] -= k * dx;
        o[1] -= k * dy;
        o[2] -= k * dz;
    }
    __device__ static void finish(const R *, R *, const Sweep &) {}
};

// acc_jerk_kernel_common.h:7-56
template <typename R>
struct AccJerkPair {
    static constexpr int NA = 8, NO = 6;
    __device__ static void init(R *o)
    {
        for (int c = 0; c < NO; ++c) o[c] = R(0);
    }
    __device__ static void pair(const R *ip, const R *jp, R *o, const Sweep &)
    {
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
        R r2 = dx * dx + dy * dy + dz * dz;
        R rv = dx * ux + dy * uy + dz * uz;
        R q = masked_inv_r2(r2, h2);
        R k = q * sqrt(q);
        R alpha = R(3) * rv * q;
        ux -= alpha * dx;
        uy -= alpha * dy;
        uz -= alpha * dz;
        k *= jp[0];
        o[0] -= k * dx;
        o[1] -= k * dy;
        o[2] -= k * dz;
        o[3] -= k * ux;
        o[4] -= k * uy;
        o[5] -= k * uz;
    }
    __device__ static void finish(const R *, R *, const Sweep &) {}
};

// snap_crackle_kernel_common.h:7-95
template <typename R>
struct SnapCracklePair {
    static constexpr int NA = 14, NO = 6;
    __device__ static void init(R *o)
    {
        for (int c = 0; c < NO; ++c) o[c] = R(0);
    }
    __device__ static void pair(const R *ip, const R *jp, R *o, const Sweep &)
    {
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
        R Ax = ip[8] - jp[8], Ay = ip[9] - jp[9], Az = ip[10] - jp[10];
        R Jx = ip[11] - jp[11], Jy = ip[12] - jp[12], Jz = ip[13] - jp[13];
        R r2 = dx * dx + dy * dy + dz * dz;
        R rv = dx * ux + dy * uy + dz * uz;
        R v2 = ux * ux + uy * uy + uz * uz;
        R rJ = dx * Jx + dy * Jy + dz * Jz;
        R rA = dx * Ax + dy * Ay + dz * Az;
        R vA = ux * Ax + uy * Ay + uz * Az;
        R q = masked_inv_r2(r2, h2);
        R k = q * sqrt(q);
        R al = rv * q;
        R al2 = al * al;
        R be = R(3) * ((v2 + rA) * q + al2);
        R ga = (R(3) * vA + rJ) * q + al * (be - R(4) * al2);
        al *= R(3);
        ga *= R(3);
        ux -= al * dx;
        uy -= al * dy;
        uz -= al * dz;
        R two_al = R(2) * al;
        Ax -= two_al * ux + be * dx;
        Ay -= two_al * uy + be * dy;
        Az -= two_al * uz + be * dz;
        al *= R(3);
        be *= R(3);
        Jx -= al * Ax + be * ux + ga * dx;
        Jy -= al * Ay + be * uy + ga * dy;
        Jz -= al * Az + be * uz + ga * dz;
        k *= jp[0];
        o[0] -= k * Ax;
        o[1] -= k * Ay;
        o[2] -= k * Az;
        o[3] -= k * Jx;
        o[4] -= k * Jy;
        o[5] -= k * Jz;
    }
    __device__ static void finish(const R *, R *, const Sweep &) {}
};

// tstep_kernel_common.h:7-60 and tstep_kernel.c:43-47
template <typename R>
struct TstepPair {
    static constexpr int NA = 8, NO = 2;
    __device__ static void init(R *o) { o[0] = o[1] = R(0); }
    __device__ static void pair(const R *ip, const R *jp, R *o,
                                const Sweep &s)
    {
        R eta = R(s.scal[0]);
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
        R msum = ip[0] + jp[0];
        R r2 = dx * dx + dy * dy + dz * dz;
        R rv = dx * ux + dy * uy + dz * uz;
        R v2 = ux * ux + uy * uy + uz * uz;
        bool mask = r2 > R(0);
        R q = masked_inv_r2(r2, h2);
        R inv_r1 = sqrt(q);
        R two = R(2);
        R b = (R(1) + two / R(2)) * q;
        R w2 = q;
        R g = q;
        R phi = msum * inv_r1;
        w2 *= (v2 + two * phi);
        g *= (w2 + b * phi);
        g *= (eta / sqrt(w2));
        w2 -= g * rv;
        w2 = mask ? w2 : R(0);
        o[0] += w2;
        o[1] = fmax(w2, o[1]);
    }
    __device__ static void finish(const R *, R *o, const Sweep &s)
    {
        R eta = R(s.scal[0]);
        o[0] = eta / sqrt(R(1) + o[0]);
        o[1] = eta / sqrt(R(1) + o[1]);
    }
};

// nreg_kernels_common.h:7-61 and nreg_kernels.c:59-66
template <typename R>
struct NregXPair {
    static constexpr int NA = 8, NO = 7;
    __device__ static void init(R *o)
    {
        for (int c = 0; c < NO; ++c) o[c] = R(0);
    }
    __device__ static void pair(const R *ip, const R *jp, R *o,
                                const Sweep &s)
    {
        R dt = R(s.scal[0]);
        R dx = ip[1] - jp[1], dy = ip[2] - jp[2], dz = ip[3] - jp[3];
        R h2 = ip[4] + jp[4];
        R ux = ip[5] - jp[5], uy = ip[6] - jp[6], uz = ip[7] - jp[7];
        dx += ux * dt;
        dy += uy * dt;
        dz += uz * dt;
        R r2 = dx * dx + dy * dy + dz * dz;
        R q = masked_inv_r2(r2, h2);
        R inv_r1 = sqrt(q);
        R k = q * inv_r1;
        R jm = jp[0];
        k *= jm;
        o[0] += jm * dx;
        o[1] += jm * dy;
        o[2] += jm * dz;
        o[3] -= k * dx;
        o[4] -= k * dy;
        o[5] -= k * dz;
        o[6] += jm * inv_r1;
    }
    __device__ static void finish(const R *ip, R *o, const Sweep &)
    {
        o[6] = ip[0] * o[6];
    }
};

// nreg_kernels_common.h:63-102 and nreg_kernels.c:107-114
template <typename R>
struct NregVPair {
    static constexpr int NA = 7, NO = 4;
    __device__ static void init(R *o)
    {
        for (int c = 0; c < NO; ++c) o[c] = R(0);
    }
    __device__ static void pair(const R *ip, const R *jp, R *o,
                                const Sweep &s)
    {
        R dt = R(s.scal[0]);
        R ux = ip[1] - jp[1], uy = ip[2] - jp[2], uz = ip[3] - jp[3];
        R wx = ip[4] - jp[4], wy = ip[5] - jp[5], wz = ip[6] - jp[6];
        ux += wx * dt;
        uy += wy * dt;
        uz += wz * dt;
        R v2 = ux * ux + uy * uy + uz * uz;
        R jm = jp[0];
        o[0] += jm * ux;
        o[1] += jm * uy;
        o[2] += jm * uz;
        o[3] += jm * v2;
    }
    __device__ static void finish(const R *ip, R *o, const Sweep &)
    {
        o[3] = ip[0] * o[3];
    }
};

}  // namespace tg
