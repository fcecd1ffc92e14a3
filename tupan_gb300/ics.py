"""Seeded synthetic initial conditions (host, numpy).

Plummer spheres in N-body units (G = M = 1, E = -1/4) with the same
construction as ``tupan/ics/plummer.py:65-127`` -- cumulative-mass sampling of
radii, isotropic directions, von Neumann rejection for the speed -- but using
the analytic Plummer potential for the escape speed instead of an O(N^2)
potential sweep, so that large spheres are cheap.  Softening is stored as
eps^2/2 per particle, as ``Plummer.set_eps2`` does (plummer.py:62-63), so
that e2_i + e2_j = eps^2.

``salpeter_masses`` samples dN/dm ~ m^alpha on [mlow, mhigh] by inverting
the cumulative distribution (the reference's ``salpeter1955`` refuses
mlow < 0.4, ``tupan/ics/imf.py:87``).
"""

import numpy as np

_SCALE = 3.0 * np.pi / 16.0   # virial radius of a Plummer sphere, a = 1


def salpeter_masses(n, rng, alpha=-2.35, mlow=0.1, mhigh=100.0):
    u = rng.random(n)
    a1 = alpha + 1.0
    lo, hi = mlow ** a1, mhigh ** a1
    return (lo + u * (hi - lo)) ** (1.0 / a1)


def plummer(n, eps=1e-4, seed=1, masses="equal", mfrac=0.999):
    """Dict of float64 arrays m, rx, ry, rz, e2, vx, vy, vz (+ zero ax..jz)."""
    rng = np.random.default_rng(seed)
    if masses == "equal":
        m = np.full(n, 1.0 / n)
    elif masses == "salpeter":
        m = salpeter_masses(n, rng)
        m /= m.sum()
    else:
        m = np.asarray(masses, dtype=np.float64)
        m = m / m.sum()
    # radii from the cumulative mass profile, stratified like
    # tupan/ics/plummer.py:65-68 (irand permutation + uniform jitter)
    irand = rng.permutation(n)
    x = (irand + rng.random(n)) * mfrac / n
    r = 1.0 / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
    ct = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    st = np.sqrt(1.0 - ct * ct)
    pos = np.stack([r * st * np.cos(ph), r * st * np.sin(ph), r * ct])
    # speed fraction q with density q^2 (1 - q^2)^(7/2), rejection sampling
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        a = rng.random(todo.size)
        b = rng.random(todo.size) * 0.1
        ok = b < a * a * (1.0 - a * a) ** 3.5
        q[todo[ok]] = a[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0) * (1.0 + r * r) ** (-0.25)
    v = q * vesc
    ct = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    st = np.sqrt(1.0 - ct * ct)
    vel = np.stack([v * st * np.cos(ph), v * st * np.sin(ph), v * ct])
    # centre of mass to the origin, then to N-body units
    pos -= (pos * m).sum(axis=1, keepdims=True)
    vel -= (vel * m).sum(axis=1, keepdims=True)
    pos *= _SCALE
    vel /= np.sqrt(_SCALE)
    out = {"m": m, "e2": np.full(n, eps * eps / 2.0)}
    out["rx"], out["ry"], out["rz"] = (np.ascontiguousarray(c) for c in pos)
    out["vx"], out["vy"], out["vz"] = (np.ascontiguousarray(c) for c in vel)
    for c in ("ax", "ay", "az", "jx", "jy", "jz"):
        out[c] = np.zeros(n)
    return out


def ensemble_sizes(count, lo=3, hi=512, seed=1):
    """System sizes drawn uniformly from [lo, hi] (inclusive)."""
    rng = np.random.default_rng(seed)
    return rng.integers(lo, hi + 1, size=count)
