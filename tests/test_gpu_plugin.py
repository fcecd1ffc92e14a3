"""The drop-in path on the GPU: tupan's extension objects and tupan's own
integrator running on the CUDA backend.

* ``tupan_gb300.extensions`` (the mirror of tupan/lib/extensions.py:63-651)
  drives every kernel with ``calc(ips, jps, *args)`` on particle sets of
  ordinary pageable numpy arrays, through ``CUDAKernel.run`` (the surface of
  tupan/lib/cffi_backend.py:90-126).  EXACT mode must equal the oracle (the
  reference's arithmetic) bit for bit, Sakura/Kepler within libm accuracy;
  SPLIT mode within the SPLIT bounds.
* Where ``TUPAN_REFERENCE`` names an importable tupan tree, tupan's own
  ``Integrator(1/64, 0, ps, method="ahermite4")`` (integrator/hermite.py:
  390-410) runs the CPU-runnable configuration (Plummer N = 256 to t = 1)
  with ``shim.install()`` routing every kernel to this library, and must
  reproduce the reference's own run (golden_config1.npz) bit for bit: all
  11747 step sizes and the final state.
"""

import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from tupan_gb300 import extensions as ext
from tupan_gb300 import ics, lib
from tupan_gb300.particles import Bodies

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_config1.npz")

# extension class, oracle kernel, positional scalars, oracle scalars,
# output attributes
CASES = [
    (ext.Phi, "phi_kernel", (), None, ("phi",)),
    (ext.Acc, "acc_kernel", (), None, ("ax", "ay", "az")),
    (ext.AccJerk, "acc_jerk_kernel", (), None,
     ("ax", "ay", "az", "jx", "jy", "jz")),
    (ext.SnapCrackle, "snap_crackle_kernel", (), None,
     ("sx", "sy", "sz", "cx", "cy", "cz")),
    (ext.Tstep, "tstep_kernel", (1.0 / 64,), {"eta": 1.0 / 64},
     ("tstep", "tstepij")),
    (ext.PNAcc, "pnacc_kernel", (), None, ("pnax", "pnay", "pnaz")),
    (ext.Sakura, "sakura_kernel", (1.0 / 64, 1), {"dt": 1.0 / 64, "flag": 1},
     ("drx", "dry", "drz", "dvx", "dvy", "dvz")),
    (ext.NREG_X, "nreg_Xkernel", (1.0 / 64,), {"dt": 1.0 / 64},
     ("mrx", "mry", "mrz", "ax", "ay", "az", "u")),
    (ext.NREG_V, "nreg_Vkernel", (1.0 / 64,), {"dt": 1.0 / 64},
     ("mvx", "mvy", "mvz", "mk")),
]


def particle_dicts(n, seed):
    ps = ics.plummer(n, eps=1e-3, seed=seed)
    aj = oracle.run("acc_jerk_kernel", ps, ps)
    for c, v in zip(("ax", "ay", "az", "jx", "jy", "jz"), aj):
        ps[c] = v
    return ps


def pn_scalars():
    d = {"order": 7}
    for k in range(1, 8):
        d["inv%d" % k] = (1.0 / 128) ** k
    return d


@pytest.fixture
def pn_order7():
    old = (ext.clight.pn_order, ext.clight.clight)
    ext.clight.pn_order = 7
    ext.clight.clight = 128.0
    yield
    ext.clight.pn_order = old[0]
    if old[1] is not None:
        ext.clight.clight = old[1]


def calc(cls, mode, ips, jps, args):
    old = lib.set_mode(mode)
    try:
        obj = cls("CUDA", "float64")
        return obj.calc(ips, jps, *args)
    finally:
        lib.set_mode(old)


@pytest.mark.parametrize("case", CASES, ids=[c[1] for c in CASES])
def test_extensions_exact_match_oracle(case, pn_order7):
    cls, name, args, osc, outs = case
    d = particle_dicts(700, 3)
    jd = {k: np.ascontiguousarray(v[100:]) for k, v in d.items()}
    for ips_d, jps_d in ((d, d), (d, jd)):
        ips = Bodies(ips_d)
        jps = ips if jps_d is ips_d else Bodies(jps_d)
        got = calc(cls, lib.MODE_EXACT, ips, jps, args)
        sc = pn_scalars() if name == "pnacc_kernel" else osc
        want = oracle.run(name, ips_d, jps_d, sc)
        assert len(got) == len(want) == len(outs)
        for a, g, w in zip(outs, got, want):
            assert g is getattr(ips, a)        # written into ips in place
            if name == "sakura_kernel":
                scale = np.abs(w).max()
                assert np.max(np.abs(g - w)) <= 1e-12 * max(scale, 1.0), a
            else:
                np.testing.assert_array_equal(g, w, err_msg=name + ":" + a)


def test_kepler_extension_matches_oracle():
    d = particle_dicts(2, 9)
    ips = Bodies(d)
    ext.Kepler("CUDA", "float64").calc(ips, ips, 1.0 / 64)
    want = oracle.run("kepler_solver_kernel", d, None, {"dt": 1.0 / 64})
    for a, w in zip(("rx", "ry", "rz", "vx", "vy", "vz"), want):
        g = getattr(ips, a)
        assert np.max(np.abs(g - w)) <= 1e-12 * np.abs(w).max(), a


@pytest.mark.parametrize("case", CASES[:5], ids=[c[1] for c in CASES[:5]])
def test_extensions_split_within_bounds(case):
    cls, name, args, osc, outs = case
    d = particle_dicts(5000, 4)
    ips = Bodies(d)
    got = calc(cls, lib.MODE_SPLIT, ips, ips, args)
    want = oracle.run(name, d, d, osc)
    if name in ("acc_kernel", "acc_jerk_kernel"):
        g = np.stack(got[:3])
        w = np.stack(want[:3])
        e = np.linalg.norm(g - w, axis=0) / np.linalg.norm(w, axis=0)
        assert np.median(e) <= 1e-7 and e.max() <= 2e-6, e.max()
    elif name == "phi_kernel":
        assert np.max(np.abs(got[0] - want[0]) / np.abs(want[0])) <= 1e-6
    elif name == "tstep_kernel":
        for g, w in zip(got, want):
            assert np.max(np.abs(g - w) / w) <= 1e-5
    else:
        for c in (0, 3):
            g = np.stack(got[c:c + 3])
            w = np.stack(want[c:c + 3])
            e = np.linalg.norm(g - w, axis=0) / np.linalg.norm(w, axis=0)
            assert np.median(e) <= 1e-5, (name, c, np.median(e))


CHILD = r"""
import json, sys, time
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[2])
import numpy as np
from tupan_gb300 import shim
ext = shim.install(mode="exact", before_import=True)
from tupan_gb300.backend import CUDAKernel
from tupan.integrator import Integrator
from tupan.particles.allparticles import ParticleSystem
z = np.load(sys.argv[3])
n = len(z["in/m"])
ps = ParticleSystem(n)
ps.mass[...] = z["in/m"]
ps.eps2[...] = z["in/e2"]
for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
    getattr(ps, k)[...] = z["in/" + k]
eta, t_end = z["params"]
e0 = [ps.kinetic_energy, ps.potential_energy]
integ = Integrator(eta, 0.0, ps, method="ahermite4")
steps = []
t0 = time.time()
while abs(integ.time) < t_end:
    tb = integ.time
    integ.evolve_step(t_end)
    steps.append(integ.time - tb)
wall = time.time() - t0
ps = integ.particle_system
res = {"cuda": all(isinstance(getattr(ext, a).kernel, CUDAKernel)
                   for a, _ in shim.SINGLETONS),
       "nsteps": len(steps),
       "steps_equal": bool(np.array_equal(np.array(steps), z["steps"])),
       "state_equal": {k: bool(np.array_equal(getattr(ps, k), z["out/" + k]))
                       for k in ("rx", "ry", "rz", "vx", "vy", "vz")},
       "energy0": e0, "energy1": [ps.kinetic_energy, ps.potential_energy],
       "wall_s": wall}
print(json.dumps(res))
"""


def test_reference_integrator_through_shim_bit_identical(tmp_path):
    ref = os.environ.get("TUPAN_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "tupan")):
        pytest.skip("TUPAN_REFERENCE does not name a tupan tree")
    env = dict(os.environ, HOME=str(tmp_path), TMPDIR=str(tmp_path))
    r = subprocess.run([sys.executable, "-c", CHILD, ref, ROOT, GOLDEN],
                       env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    print(json.dumps(res))
    z = np.load(GOLDEN)
    assert res["cuda"]
    assert res["nsteps"] == len(z["steps"])
    assert res["steps_equal"]
    assert all(res["state_equal"].values()), res["state_equal"]
    np.testing.assert_allclose(res["energy1"], z["energy1"], rtol=1e-13)
