"""tupan's Plummer initial conditions (tupan/ics/plummer.py, make_plummer)
with the three O(N^2) potential sweeps on the GPU.

The model is built exactly as the reference builds it: the same calls on
numpy's legacy global random stream in the same order (masses from the IMF
with the stream state restored afterwards, a permutation, radii, angles,
rejection-sampled speeds), the same numpy expressions for positions,
velocities, centre of mass and the rescalings to N-body units and virial
equilibrium.  What changes is where the potential comes from: set_phi in
set_bodies, the virial radius in to_nbody_units and the potential energy in
scale_to_virial each need a full Phi sweep, which on the CPU is O(N^2) and
dominates the setup at N >= 2^18; here each is one EXACT-mode sweep on the
GPU (bit-identical to the reference's phi_kernel).  The O(N) sampling stays
on numpy because its output is defined by numpy's random stream.

    from tupan_gb300.plummer import make_plummer
    ps = make_plummer(262144, 1e-4, ("equalmass",), seed=1)

    python -m tupan_gb300.plummer --n 262144     # timing of the two parts
"""

import time

import numpy as np


# ---------------------------------------------------------------------------
# IMFs (tupan/ics/imf.py:20-121): the mass function, its normalisation over
# [min_mlow, max_mhigh] and the rejection sampler over [mlow, mhigh].
# ---------------------------------------------------------------------------
class IMFSample(object):
    def __init__(self, imf_func, min_mlow, max_mhigh, mlow, mhigh):
        from scipy.integrate import quad
        from scipy.optimize import fminbound
        if mlow < min_mlow or mhigh > max_mhigh:
            raise ValueError("Mass range outer of limits [{0}:{1}]."
                             .format(min_mlow, max_mhigh))
        norm, _ = quad(lambda m: imf_func(m) / m, min_mlow, max_mhigh)
        func = lambda m: imf_func(m) / norm
        mpeak = float(fminbound(lambda m: -func(m), min_mlow, max_mhigh,
                                xtol=1.0e-8))
        self.func = func
        self.peak = func(mpeak)
        self.mlow = mlow
        self.mhigh = mhigh

    def sample(self, n):
        """imf.py:55-66: accept m ~ exp(U(log mlow, log mhigh)) where
        U(0, peak) < f(m), growing the batch until n are accepted."""
        size = n
        ran_mass = []
        while len(ran_mass) < n:
            ran_imf = np.random.uniform(0.0, self.peak, size=size)
            ran_mass = np.exp(np.random.uniform(np.log(self.mlow),
                                                np.log(self.mhigh), size=size))
            ran_mass = ran_mass[np.where((ran_imf < self.func(ran_mass)))]
            size *= int(1 + n / len(ran_mass))
        return ran_mass[:n]


def make_imf(spec):
    """("equalmass",), ("salpeter1955", mlow, mhigh), ("padoan2007", mlow,
    mhigh) or ("parravano2011", mlow, mhigh) (imf.py:69-121)."""
    name, args = spec[0], tuple(spec[1:])
    if name == "equalmass":
        return IMFSample(lambda m: (1.0 + m) - m, 0.1, 10.0, 1.0, 1.0)
    if name == "salpeter1955":
        return IMFSample(lambda m: m**(-1.35), 0.4, 120.0, *args)
    if name == "padoan2007":
        from scipy.special import erf
        gamma, m_ch, sigma = 1.4, 1.0, 1.8
        f = lambda m: ((m**(-gamma)) * (1.0 + erf(
            (4.0 * np.log(m / m_ch) + sigma**2) / (np.sqrt(8.0) * sigma))))
        return IMFSample(f, 0.004, 120.0, *args)
    if name == "parravano2011":
        f = lambda m: (m**(-1.35)) * (1.0 - np.exp(-(m / 0.35)**(0.51 + 1.35)))
        return IMFSample(f, 0.004, 120.0, *args)
    raise ValueError("unknown IMF: %r" % (name,))


# ---------------------------------------------------------------------------
# The potential sweep.
# ---------------------------------------------------------------------------
def gpu_phi(ps, mode="exact"):
    """phi_kernel(ps, ps) on the GPU through the C-ABI: EXACT mode
    (bit-identical to the reference's kernel) or SPLIT (FP32 pairs on
    double-single positions, |dphi|/|phi| <= 1e-6, about 100x faster)."""
    from . import abi, lib
    old = lib.set_mode(lib.MODE_SPLIT if mode == "split" else lib.MODE_EXACT)
    try:
        fn = lib.bind("phi_kernel")
        vals = abi.make_args("phi_kernel", "float64", ps, ps)
        abi.call(fn, "phi_kernel", "float64", vals)
        lib.check()
        return np.array(abi.outputs("phi_kernel", vals)[0], copy=True)
    finally:
        lib.set_mode(old)


def _ps_view(ps):
    return {"m": ps["m"], "rx": ps["rx"], "ry": ps["ry"], "rz": ps["rz"],
            "e2": ps["e2"]}


def _total_mass(ps):
    return float(ps["m"].sum())


def _kinetic(ps):
    ke = 0.5 * ps["m"] * (ps["vx"]**2 + ps["vy"]**2 + ps["vz"]**2)
    return float(ke.sum())


def _potential(ps, phi_fn, timing):
    t0 = time.perf_counter()
    ps["phi"] = phi_fn(_ps_view(ps))
    timing["phi_s"] += time.perf_counter() - t0
    timing["phi_sweeps"] += 1
    return 0.5 * float((ps["m"] * ps["phi"]).sum())


def _set_eps2(ps, n, eps2, softening_type):
    """plummer.py:35-62 (returns half the per-particle value)."""
    mass = ps["m"]
    if softening_type == 0:
        e = np.ones(n)
    elif softening_type == 1:
        e = mass**2
    elif softening_type == 2:
        e = mass / n
    elif softening_type == 3:
        e = (mass / n**2)**(2.0 / 3)
    elif softening_type == 4:
        e = (1.0 / (mass * n**2))**2
    else:
        raise ValueError("Unexpected value for softening_type: {}."
                         .format(softening_type))
    e *= eps2 / np.mean(e)
    return e / 2


def make_plummer(n, eps, imf, seed=None, mfrac=0.999, softening_type=0,
                 phi_fn=None, timing=None, phi_mode="exact"):
    """make_plummer (plummer.py:213-221): a dict of float64 arrays m, e2
    (the per-particle eps^2/2 tupan stores), rx, ry, rz, vx, vy, vz and phi
    (the potential of the last sweep).  phi_fn: the Phi sweep (default: the
    GPU in phi_mode "exact" -- the reference's model bit for bit -- or
    "split"); timing: optional dict receiving host/phi seconds."""
    if phi_fn is None:
        phi_fn = lambda p: gpu_phi(p, phi_mode)
    if timing is None:
        timing = {}
    timing.update(phi_s=0.0, phi_sweeps=0)
    t_start = time.perf_counter()
    if n < 2:
        n = 2
    imf_obj = make_imf(imf)
    np.random.seed(seed)
    ps = {}
    # set_bodies (plummer.py:93-124)
    ilist = np.arange(n)
    srand = np.random.get_state()
    ps["m"] = np.array(imf_obj.sample(n), dtype=np.float64)
    ps["m"] /= _total_mass(ps)
    ps["e2"] = _set_eps2(ps, n, eps * eps, softening_type)
    np.random.set_state(srand)
    # set_pos (plummer.py:64-74)
    irand = np.random.permutation(ilist)
    mrand = (irand + np.random.random(n)) * mfrac / n
    radius = 1.0 / np.sqrt(np.power(mrand, -2.0 / 3.0) - 1.0)
    theta = np.arccos(np.random.uniform(-1.0, 1.0, size=n))
    phi = np.random.uniform(0.0, 2.0 * np.pi, size=n)
    ps["rx"] = radius * np.sin(theta) * np.cos(phi)
    ps["ry"] = radius * np.sin(theta) * np.sin(phi)
    ps["rz"] = radius * np.cos(theta)
    # set_phi, then set_vel (plummer.py:76-91)
    _potential(ps, phi_fn, timing)
    count = 0
    rnd = np.empty(n)
    while count < n:
        r1 = np.random.random()
        r2 = np.random.random()
        if r2 < r1:
            rnd[count] = r2
            count += 1
    velocity = np.sqrt(-2 * rnd * ps["phi"])
    theta = np.arccos(np.random.uniform(-1.0, 1.0, size=n))
    phi = np.random.uniform(0.0, 2.0 * np.pi, size=n)
    ps["vx"] = velocity * np.sin(theta) * np.cos(phi)
    ps["vy"] = velocity * np.sin(theta) * np.sin(phi)
    ps["vz"] = velocity * np.cos(theta)
    # make_model (plummer.py:126-130): com_to_origin (body.py:86-176)
    mtot = _total_mass(ps)
    com_r = np.array([ps["m"] * ps["rx"], ps["m"] * ps["ry"],
                      ps["m"] * ps["rz"]]).T.sum(0) / mtot
    com_v = np.array([ps["m"] * ps["vx"], ps["m"] * ps["vy"],
                      ps["m"] * ps["vz"]]).T.sum(0) / mtot
    com_r, com_v = -com_r, -com_v
    for k, c in enumerate("xyz"):
        ps["r" + c] += com_r[k]
    for k, c in enumerate("xyz"):
        ps["v" + c] += com_v[k]
    # to_nbody_units (body.py:405-461)
    m_ratio = 1.0 / _total_mass(ps)
    ps["m"] *= m_ratio
    for c in "xyz":
        ps["r" + c] *= m_ratio
    mtot = _total_mass(ps)
    pe = _potential(ps, phi_fn, timing)
    r_scale = 1.0 / ((mtot**2) / (-2 * pe))
    v_scale = 1 / r_scale**0.5
    for c in "xyz":
        ps["r" + c] *= r_scale
    for c in "xyz":
        ps["v" + c] *= v_scale
    # scale_to_virial (body.py:444-453)
    ke = _kinetic(ps)
    pe = _potential(ps, phi_fn, timing)
    v_scale = ((-0.5 * pe) / ke)**0.5
    for c in "xyz":
        ps["v" + c] *= v_scale
    timing["total_s"] = time.perf_counter() - t_start
    timing["host_s"] = timing["total_s"] - timing["phi_s"]
    return ps


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=262144)
    ap.add_argument("--eps", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--phi-mode", default="exact", choices=["exact", "split"])
    a = ap.parse_args(argv)
    timing = {}
    make_plummer(a.n, a.eps, ("equalmass",), seed=a.seed, timing=timing,
                 phi_mode=a.phi_mode)
    timing["n"] = a.n
    timing["phi_mode"] = a.phi_mode
    timing["phi_gint_per_s"] = (timing["phi_sweeps"] * float(a.n)**2 /
                                timing["phi_s"] / 1e9)
    print(json.dumps(timing))


if __name__ == "__main__":
    main()
