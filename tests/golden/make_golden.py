"""Generate the golden fixtures in this directory from the REFERENCE itself.

Run (needs the reference source tree; it is imported, never copied):

    HOME=<a writable directory> python tests/golden/make_golden.py <reference tree>

The script imports ``tupan.lib.extensions`` from the reference, which builds
the reference's own C kernels through its cffi backend
(``tupan/lib/cffi_backend.py:31-87``), and calls every extension through the
reference's public ``calc`` API (``tupan/lib/extensions.py:94-97``) on seeded
inputs.  Inputs and outputs are stored in ``golden_<case>.npz``; the sha256 of
every reference source file used is stored with them.

Cases follow the reference's own test (``tupan/tests/test_extensions.py``):
uniform masses and x10 positions/velocities with eps2=0 at N=256, j-prefix
and swapped i/j roles, eta=1/64, PN order 7 with c=128, dt=1/64; plus a
softened Plummer sphere and a set of close two-body systems that drive the
Sakura/Kepler solver through its Kepler branch, its period reduction, the
hyperbolic start and the softened energy check.
"""

import glob
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

ATTRS = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz",
         "ax", "ay", "az", "jx", "jy", "jz")
SHORT = {"mass": "m", "eps2": "e2"}


class Bodies(object):
    """Duck-typed particle set: the attributes the extensions read, plus
    ``register_auxiliary_attribute`` (tupan/particles/allparticles.py:64)."""

    def __init__(self, arrays, dtype):
        self.n = len(arrays["m"])
        self._dtype = dtype
        for a in ATTRS:
            setattr(self, a, np.ascontiguousarray(arrays[SHORT.get(a, a)],
                                                  dtype=dtype).copy())

    def register_auxiliary_attribute(self, name, kind):
        setattr(self, name, np.zeros(self.n, dtype=self._dtype))


def uniform(n, rng):
    """tupan/tests/test_extensions.py:28-36 with a seeded generator."""
    d = {"m": rng.random(n), "e2": np.zeros(n)}
    d["rx"], d["ry"], d["rz"] = rng.random((n, 3)).T * 10
    d["vx"], d["vy"], d["vz"] = rng.random((n, 3)).T * 10
    for k in ("ax", "ay", "az", "jx", "jy", "jz"):
        d[k] = rng.standard_normal(n)
    return d


def plummer(n, eps, rng):
    """Small Plummer sphere (analytic potential, N-body units, G=M=1) with
    per-particle eps2 = eps^2/2 as tupan/ics/plummer.py:62-63 stores it."""
    m = np.full(n, 1.0 / n)
    x = rng.random(n) * 0.999
    r = 1.0 / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
    ct = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    st = np.sqrt(1 - ct ** 2)
    pos = np.stack([r * st * np.cos(ph), r * st * np.sin(ph), r * ct])
    q = np.empty(n)
    k = 0
    while k < n:
        a, b = rng.random(2)
        if b < a:
            q[k] = b
            k += 1
    v = np.sqrt(-2 * q * (-1.0 / np.sqrt(1 + r * r)))
    ct = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    st = np.sqrt(1 - ct ** 2)
    vel = np.stack([v * st * np.cos(ph), v * st * np.sin(ph), v * ct])
    s = 3 * np.pi / 16
    pos *= s
    vel /= np.sqrt(s)
    d = {"m": m, "e2": np.full(n, eps * eps / 2)}
    d["rx"], d["ry"], d["rz"] = pos
    d["vx"], d["vy"], d["vz"] = vel
    for c in ("ax", "ay", "az", "jx", "jy", "jz"):
        d[c] = rng.standard_normal(n)
    return d


def close_pairs(rng, n_pairs):
    """Interleaved two-body systems: bound, near-parabolic and hyperbolic
    pairs at small separation (Kepler branch of twobody_solver,
    sakura_kernel_common.h:111-122), widely separated from one another."""
    d = {k: [] for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    for p in range(n_pairs):
        m1, m2 = rng.uniform(0.1, 1.0, 2) * 1e-2
        sep = rng.uniform(1e-3, 5e-2)
        mu = m1 + m2
        vc = np.sqrt(mu / sep)
        kind = p % 4
        fac = [0.3, 0.9, 1.4142, 2.5][kind] * rng.uniform(0.8, 1.2)
        u = rng.standard_normal(3)
        u /= np.linalg.norm(u)
        w = rng.standard_normal(3)
        w -= w.dot(u) * u
        w /= np.linalg.norm(w)
        rel_r = sep * u
        rel_v = fac * vc * (w * 0.9 + u * 0.1 * rng.standard_normal())
        centre = rng.uniform(-50, 50, 3)
        for (mm, sgn, mo) in ((m1, 1, m2), (m2, -1, m1)):
            d["m"].append(mm)
            d["e2"].append(0.0 if p % 3 else 1e-8)
            pos = centre + sgn * rel_r * mo / mu
            vel = sgn * rel_v * mo / mu
            d["rx"].append(pos[0]); d["ry"].append(pos[1]); d["rz"].append(pos[2])
            d["vx"].append(vel[0]); d["vy"].append(vel[1]); d["vz"].append(vel[2])
    out = {k: np.array(v) for k, v in d.items()}
    n = len(out["m"])
    for c in ("ax", "ay", "az", "jx", "jy", "jz"):
        out[c] = rng.standard_normal(n)
    return out


def subset(d, sl):
    return {k: v[sl] for k, v in d.items()}


def main(refroot):
    sys.path.insert(0, refroot)
    from tupan.lib import extensions as ext

    src = sorted(glob.glob(os.path.join(refroot, "tupan/lib/src/*")))
    digests = {os.path.relpath(p, refroot):
               hashlib.sha256(open(p, "rb").read()).hexdigest() for p in src}
    for f in ("tupan/lib/extensions.py", "tupan/lib/cffi_backend.py"):
        digests[f] = hashlib.sha256(
            open(os.path.join(refroot, f), "rb").read()).hexdigest()

    ext.clight.pn_order = 7
    ext.clight.clight = 128

    kernels = [
        ("phi_kernel", ext.Phi, ()),
        ("acc_kernel", ext.Acc, ()),
        ("acc_jerk_kernel", ext.AccJerk, ()),
        ("snap_crackle_kernel", ext.SnapCrackle, ()),
        ("tstep_kernel", ext.Tstep, (1.0 / 64,)),
        ("pnacc_kernel", ext.PNAcc, ()),
        ("nreg_Xkernel", ext.NREG_X, (1.0 / 64,)),
        ("nreg_Vkernel", ext.NREG_V, (1.0 / 64,)),
        ("sakura_kernel", ext.Sakura, (1.0 / 64, 0)),
        ("sakura_kernel", ext.Sakura, (1.0 / 64, -1)),
        ("sakura_kernel", ext.Sakura, (1.0 / 64, 1)),
        ("sakura_kernel", ext.Sakura, (1.0 / 64, -2)),
        ("sakura_kernel", ext.Sakura, (1.0 / 64, 2)),
    ]

    rng = np.random.default_rng(20240611)
    sets = {
        "uniform256": uniform(256, rng),
        "plummer96": plummer(96, 1e-2, rng),
        "pairs": close_pairs(rng, 48),
    }
    roles = {
        "uniform256": [("all", "all"), ("all", "j37"), ("i37", "all"),
                       ("i1", "all")],
        "plummer96": [("all", "all"), ("i5", "all")],
        "pairs": [("all", "all")],
    }
    cut = {"all": slice(None), "j37": slice(0, 37), "i37": slice(0, 37),
           "i5": slice(0, 5), "i1": slice(0, 1)}

    for prec in ("float64", "float32"):
        dtype = np.float64 if prec == "float64" else np.float32
        for sname, data in sets.items():
            store = {"__prec__": np.array(prec)}
            for k, v in data.items():
                store["in/" + k] = np.asarray(v, dtype=dtype)
            for (ir, jr) in roles[sname]:
                for (kname, cls, args) in kernels:
                    # Fresh particle sets per call: extensions write their
                    # results into i-attributes (e.g. Acc into ax/ay/az) that
                    # later kernels read as inputs.
                    I = Bodies(subset(data, cut[ir]), dtype)
                    J = Bodies(subset(data, cut[jr]), dtype)
                    kern = cls("C", prec)
                    res = kern.calc(I, J, *args)
                    tag = "%s|%s|%s|%s" % (kname, ir, jr,
                                           ",".join(repr(a) for a in args))
                    for idx, r in enumerate(res):
                        store["out/%s/%d" % (tag, idx)] = np.array(r, copy=True)
            if sname == "pairs":
                # Kepler extension: each pair on its own, in place
                # (tupan/lib/extensions.py:618-651).
                # Softened pairs only at the short step: with a long step the
                # reference's energy-check subdivision never terminates on
                # them (universal_kepler_solver.h:580-606 has no bound).
                n = len(data["m"]) // 2
                soft = np.asarray(data["e2"])[0::2] > 0
                for dt in (1.0 / 64, 1.0, 37.5):
                    pairs = [p for p in range(n) if dt < 0.1 or not soft[p]]
                    store["kepler_pairs/%r" % dt] = np.array(pairs)
                    res = np.empty((len(pairs), 12), dtype=dtype)
                    for row, p in enumerate(pairs):
                        P = Bodies(subset(data, slice(2 * p, 2 * p + 2)),
                                   dtype)
                        kern = ext.Kepler("C", prec)
                        kern.calc(P, P, dt)
                        res[row] = np.concatenate(
                            [P.rx, P.ry, P.rz, P.vx, P.vy, P.vz])
                    store["kepler/%r" % dt] = res
            store["__sources__"] = np.array(
                "\n".join("%s %s" % (v, k) for k, v in sorted(digests.items())))
            fn = os.path.join(HERE, "golden_%s_%s.npz" % (sname, prec))
            np.savez_compressed(fn, **store)
            print("wrote", fn, os.path.getsize(fn))


INTEGRATOR_RUNS = [
    # (method, n, eps, masses, eta, t_end, max_steps, seed)
    ("ahermite4", 64, 1e-4, "equal", 1.0 / 64, 1.0, 60, 11),
    ("hermite4", 64, 1e-4, "equal", 1.0 / 64, 1.0, 40, 12),
    ("ahermite6", 48, 1e-4, "salpeter", 1.0 / 32, 0.5, 30, 13),
    ("ahermite8", 48, 1e-4, "salpeter", 1.0 / 32, 0.5, 30, 14),
    ("ahermite2", 48, 1e-4, "equal", 1.0 / 64, 1.0, 30, 15),
    ("sakura", 40, 0.0, "salpeter", 1.0 / 256, 0.25, 20, 16),
    ("asakura", 40, 0.0, "salpeter", 1.0 / 64, 0.25, 20, 17),
]


def integrators(refroot):
    """Short runs of the reference's own integrators on its C backend
    (tupan/integrator/__init__.py:108-157, evolve loop as
    tupan/simulation.py:191-198)."""
    sys.path.insert(0, refroot)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tupan.integrator import Integrator
    from tupan.particles.allparticles import ParticleSystem
    from tupan_gb300 import ics

    store = {}
    for (method, n, eps, masses, eta, t_end, max_steps, seed) in \
            INTEGRATOR_RUNS:
        d = ics.plummer(n, eps=eps, seed=seed, masses=masses)
        ps = ParticleSystem(n)
        ps.mass[...] = d["m"]
        ps.eps2[...] = d["e2"]
        for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
            getattr(ps, k)[...] = d[k]
        tag = "%s/" % method
        for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "in/" + k] = d[k].copy()
        integ = Integrator(eta, 0.0, ps, method=method)
        steps = []
        while abs(integ.time) < t_end and len(steps) < max_steps:
            t0 = integ.time
            integ.evolve_step(t_end)
            steps.append(integ.time - t0)
        ps = integ.particle_system
        store[tag + "steps"] = np.array(steps)
        store[tag + "params"] = np.array([eta, t_end, max_steps])
        for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "out/" + k] = np.array(getattr(ps, k), copy=True)
        print(method, len(steps), "steps, t =", integ.time)
    fn = os.path.join(HERE, "golden_integrators.npz")
    np.savez_compressed(fn, **store)
    print("wrote", fn, os.path.getsize(fn))


TINY_RUNS = [
    # (method, first, last particle of a 64-body Plummer sphere, eta, t_end)
    # a lone particle's step is eta exactly, a power of two, where the step
    # quantisation's truncation is decided by the last bit of log2
    ("ahermite4", 0, 1, 1.0 / 64, 1.0 / 16),
    ("ahermite4", 1, 3, 1.0 / 64, 1.0 / 16),
    ("ahermite6", 0, 1, 1.0 / 32, 1.0 / 8),
    ("ahermite6", 1, 3, 1.0 / 32, 1.0 / 8),
]


def tiny(refroot):
    """Runs of the reference's own integrators on 1- and 2-particle systems
    (tupan/integrator/__init__.py:59-78 quantises a lone particle's step
    eta to eta / 2)."""
    sys.path.insert(0, refroot)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tupan.integrator import Integrator
    from tupan.particles.allparticles import ParticleSystem
    from tupan_gb300 import ics

    d = ics.plummer(64, eps=1e-4, seed=3)
    store = {}
    for k, (method, lo, hi, eta, t_end) in enumerate(TINY_RUNS):
        n = hi - lo
        ps = ParticleSystem(n)
        ps.mass[...] = d["m"][lo:hi]
        ps.eps2[...] = d["e2"][lo:hi]
        for a in ("rx", "ry", "rz", "vx", "vy", "vz"):
            getattr(ps, a)[...] = d[a][lo:hi]
        tag = "%d/" % k
        for a in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "in/" + a] = d[a][lo:hi].copy()
        integ = Integrator(eta, 0.0, ps, method=method)
        steps = []
        while abs(integ.time) < t_end:
            t0 = integ.time
            integ.evolve_step(t_end)
            steps.append(integ.time - t0)
        ps = integ.particle_system
        store[tag + "method"] = np.array(method)
        store[tag + "params"] = np.array([eta, t_end])
        store[tag + "steps"] = np.array(steps)
        for a in ("rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "out/" + a] = np.array(getattr(ps, a), copy=True)
        print(method, n, "particles:", len(steps), "steps of", steps[0])
    store["runs"] = np.array(len(TINY_RUNS))
    fn = os.path.join(HERE, "golden_tiny.npz")
    np.savez_compressed(fn, **store)
    print("wrote", fn, os.path.getsize(fn))


def config1(refroot):
    """The CPU-runnable configuration in full: Plummer N=256, equal masses,
    eps=1e-4, tupan's ahermite4 (shared adaptive steps, eta=1/64) to
    t_end=1, on the reference's own C backend; stores every step size, the
    final state and the reference's energies at the start and the end
    (body.py:260-321)."""
    sys.path.insert(0, refroot)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tupan.integrator import Integrator
    from tupan.particles.allparticles import ParticleSystem
    from tupan_gb300 import ics

    n, eta, t_end = 256, 1.0 / 64, 1.0
    d = ics.plummer(n, eps=1e-4, seed=256, masses="equal")
    ps = ParticleSystem(n)
    ps.mass[...] = d["m"]
    ps.eps2[...] = d["e2"]
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        getattr(ps, k)[...] = d[k]
    store = {"in/" + k: d[k].copy() for k in
             ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    store["params"] = np.array([eta, t_end])
    store["energy0"] = np.array([ps.kinetic_energy, ps.potential_energy])
    integ = Integrator(eta, 0.0, ps, method="ahermite4")
    steps = []
    while abs(integ.time) < t_end:
        t0 = integ.time
        integ.evolve_step(t_end)
        steps.append(integ.time - t0)
    ps = integ.particle_system
    store["steps"] = np.array(steps)
    store["energy1"] = np.array([ps.kinetic_energy, ps.potential_energy])
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        store["out/" + k] = np.array(getattr(ps, k), copy=True)
    e0, e1 = store["energy0"].sum(), store["energy1"].sum()
    print("config1:", len(steps), "steps, dE/E =", (e1 - e0) / abs(e0))
    fn = os.path.join(HERE, "golden_config1.npz")
    np.savez_compressed(fn, **store)
    print("wrote", fn, os.path.getsize(fn))


NREG_RUNS = [
    # (method, n, eps, masses, eta, t_end, max_steps, seed)
    ("nreg", 64, 1e-2, "equal", 1.0 / 64, 0.25, 12, 51),
    ("anreg", 64, 1e-2, "equal", 1.0 / 64, 0.25, 12, 52),
    ("nreg", 40, 1e-3, "salpeter", 1.0 / 128, 0.25, 10, 53),
    ("anreg", 200, 1e-3, "salpeter", 1.0 / 128, 0.25, 6, 54),
]


def nreg(refroot):
    """Short runs of the reference's NREG integrators (tupan/integrator/
    nreg.py) on its C backend: the time after each step, the final state
    and the final W, U, S (class attributes of the particle system)."""
    sys.path.insert(0, refroot)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tupan.integrator import Integrator
    from tupan.particles.allparticles import ParticleSystem
    from tupan_gb300 import ics

    store = {}
    for r, (method, n, eps, masses, eta, t_end, max_steps, seed) in \
            enumerate(NREG_RUNS):
        d = ics.plummer(n, eps=eps, seed=seed, masses=masses)
        ps = ParticleSystem(n)
        ps.mass[...] = d["m"]
        ps.eps2[...] = d["e2"]
        for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
            getattr(ps, k)[...] = d[k]
        tag = "%d/" % r
        store[tag + "method"] = np.array(method)
        for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "in/" + k] = d[k].copy()
        integ = Integrator(eta, 0.0, ps, method=method)
        times = []
        while abs(integ.time) < t_end and len(times) < max_steps:
            integ.evolve_step(t_end)
            times.append(integ.time)
        ps = integ.particle_system
        store[tag + "times"] = np.array(times)
        store[tag + "params"] = np.array([eta, t_end, max_steps])
        store[tag + "scalars"] = np.array([type(ps).W, type(ps).U,
                                           type(ps).S, type(ps).E0])
        for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "out/" + k] = np.array(getattr(ps, k), copy=True)
        print(method, n, len(times), "steps, t =", integ.time)
    fn = os.path.join(HERE, "golden_nreg.npz")
    np.savez_compressed(fn, **store)
    print("wrote", fn, os.path.getsize(fn))


PLUMMER_RUNS = [
    # (n, eps, imf, seed, softening_type)
    (256, 1e-4, ("equalmass",), 1, 0),
    (1000, 1e-3, ("salpeter1955", 0.5, 10.0), 2, 0),
    (500, 1e-2, ("equalmass",), 3, 2),
    (300, 1e-3, ("parravano2011", 0.1, 20.0), 4, 1),
]


def plummer(refroot):
    """The reference's own initial conditions (tupan/ics/plummer.py:213-221
    make_plummer) for a few sizes, IMFs and softening types."""
    sys.path.insert(0, refroot)
    from tupan.ics.plummer import make_plummer

    store = {}
    for r, (n, eps, imf, seed, stype) in enumerate(PLUMMER_RUNS):
        ps = make_plummer(n, eps, imf, seed=seed, softening_type=stype)
        tag = "%d/" % r
        store[tag + "params"] = np.array([n, eps, seed, stype])
        store[tag + "imf"] = np.array([str(x) for x in imf])
        for k, a in (("m", "mass"), ("e2", "eps2"), ("rx", "rx"),
                     ("ry", "ry"), ("rz", "rz"), ("vx", "vx"), ("vy", "vy"),
                     ("vz", "vz"), ("phi", "phi")):
            store[tag + k] = np.array(getattr(ps, a), copy=True)
        print("plummer", n, imf, "m sum", ps.mass.sum())
    fn = os.path.join(HERE, "golden_plummer_ics.npz")
    np.savez_compressed(fn, **store)
    print("wrote", fn, os.path.getsize(fn))


SIA_RUNS = [
    # (method, n, eps, masses, eta, t_end, max_steps, seed)
    ("sia21h.dkd", 48, 1e-4, "salpeter", 1.0 / 32, 0.25, 6, 31),
    ("sia21h.kdk", 48, 1e-4, "salpeter", 1.0 / 32, 0.25, 6, 32),
    ("sia21a.dkd", 40, 1e-4, "equal", 1.0 / 32, 0.25, 8, 33),
    ("sia21s.kdk", 40, 1e-4, "equal", 1.0 / 64, 0.25, 8, 34),
    ("sia22h.dkd", 40, 1e-4, "salpeter", 1.0 / 32, 0.25, 4, 35),
    ("sia43h.kdk", 32, 1e-4, "salpeter", 1.0 / 32, 0.25, 2, 36),
    ("sia44a.dkd", 40, 1e-4, "salpeter", 1.0 / 32, 0.25, 4, 37),
    ("sia45s.dkd", 32, 1e-4, "equal", 1.0 / 64, 0.25, 4, 38),
    ("sia46h.kdk", 32, 1e-4, "salpeter", 1.0 / 32, 0.25, 2, 39),
    ("sia67a.kdk", 32, 1e-4, "equal", 1.0 / 32, 0.25, 3, 40),
    ("sia69h.dkd", 16, 1e-4, "equal", 1.0 / 32, 0.25, 1, 41),
    ("sia21h.dkd", 3, 0.0, "salpeter", 1.0 / 16, 0.25, 6, 42),
]


def sia(refroot):
    """Short runs of the reference's SIA integrators (tupan/integrator/
    sia.py:965-1123) on its C backend.  SIA reorders the particle system at
    every split/join, so the final state is stored in the reference's final
    order together with each particle's id, time, nstep and tstep."""
    sys.path.insert(0, refroot)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tupan.integrator import Integrator
    from tupan.particles.allparticles import ParticleSystem
    from tupan_gb300 import ics

    store = {}
    for r, (method, n, eps, masses, eta, t_end, max_steps, seed) in \
            enumerate(SIA_RUNS):
        d = ics.plummer(n, eps=eps, seed=seed, masses=masses)
        ps = ParticleSystem(n)
        ps.id[...] = np.arange(n)
        ps.mass[...] = d["m"]
        ps.eps2[...] = d["e2"]
        for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
            getattr(ps, k)[...] = d[k]
        tag = "%d/" % r
        store[tag + "method"] = np.array(method)
        for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz"):
            store[tag + "in/" + k] = d[k].copy()
        integ = Integrator(eta, 0.0, ps, method=method)
        times = []
        while abs(integ.time) < t_end and len(times) < max_steps:
            integ.evolve_step(t_end)
            times.append(integ.time)
        ps = integ.particle_system
        store[tag + "times"] = np.array(times)
        store[tag + "params"] = np.array([eta, t_end, max_steps])
        for k in ("id", "rx", "ry", "rz", "vx", "vy", "vz", "time", "nstep",
                  "tstep"):
            store[tag + "out/" + k] = np.array(getattr(ps, k), copy=True)
        print(method, n, len(times), "steps, t =", integ.time,
              "nstep range", int(ps.nstep.min()), int(ps.nstep.max()))
    fn = os.path.join(HERE, "golden_sia.npz")
    np.savez_compressed(fn, **store)
    print("wrote", fn, os.path.getsize(fn))


if __name__ == "__main__":
    if len(sys.argv) < 2 or sys.argv[1].startswith("--"):
        sys.exit("usage: make_golden.py <reference tree> [--integrators|"
                 "--sia|--config1|--nreg|--plummer|--tiny]")
    ref = sys.argv[1]
    if "--integrators" in sys.argv:
        integrators(ref)
    elif "--sia" in sys.argv:
        sia(ref)
    elif "--config1" in sys.argv:
        config1(ref)
    elif "--nreg" in sys.argv:
        nreg(ref)
    elif "--plummer" in sys.argv:
        plummer(ref)
    elif "--tiny" in sys.argv:
        tiny(ref)
    else:
        main(ref)
        integrators(ref)
        sia(ref)
        config1(ref)
        nreg(ref)
        plummer(ref)
        tiny(ref)
