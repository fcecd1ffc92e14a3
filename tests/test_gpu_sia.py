"""Device-resident SIA driver (csrc/sia.cu) against the reference's own SIA
runs (golden_sia.npz) and the numpy SIA oracle (oracle/sia.py)."""

import os

import numpy as np
import pytest

from oracle import integrators as oi
from oracle import sia as osia
from tupan_gb300 import ics
from tupan_gb300.integrator import DeviceSIA, SIA_METHODS

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_sia.npz")
STATE = ("rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep")


def runs():
    z = np.load(GOLDEN)
    return sorted({int(k.split("/")[0]) for k in z.files})


def load(r):
    z = np.load(GOLDEN)
    tag = "%d/" % r
    ps = {k: z[tag + "in/" + k].copy() for k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    eta, t_end, max_steps = z[tag + "params"]
    out = {k: z[tag + "out/" + k] for k in ("id", "nstep") + STATE}
    return (str(z[tag + "method"]), ps, float(eta), float(t_end),
            int(max_steps), z[tag + "times"], out)


@pytest.mark.parametrize("subtree", [0, 16, 128])
@pytest.mark.parametrize("r", runs())
def test_exact_sia_matches_reference(r, subtree):
    method, ps, eta, t_end, max_steps, times, out = load(r)
    d = DeviceSIA(ps, method, eta, mode="exact")
    d.set_subtree(subtree)
    got = d.evolve(t_end, max_steps=max_steps)
    st = d.state()
    kep = d.stats()["kepler"]
    d.close()
    np.testing.assert_array_equal(got, times)
    np.testing.assert_array_equal(st["id"], out["id"])
    np.testing.assert_array_equal(st["nstep"], out["nstep"])
    for k in STATE:
        if kep == 0:
            # no two-body subsystem: every operation is the reference's
            np.testing.assert_array_equal(st[k], out[k], err_msg=k)
        else:
            # Kepler solves: CUDA's transcendental functions against libm
            scale = np.abs(out[k]).max()
            assert np.abs(st[k] - out[k]).max() <= 1e-9 * scale, k


@pytest.mark.parametrize("method", ["sia21h.dkd", "sia44h.kdk", "sia22a.kdk",
                                    "sia67s.dkd"])
def test_exact_sia_matches_oracle_at_larger_n(method):
    ps = ics.plummer(384, eps=1e-3, seed=5, masses="salpeter")
    eta = 1.0 / 64
    ref, times = osia.evolve(ps, method, eta, 1.0, max_steps=2)
    d = DeviceSIA(ps, method, eta, mode="exact")
    got = d.evolve(1.0, max_steps=2)
    st = d.state()
    kep = d.stats()["kepler"]
    d.close()
    np.testing.assert_array_equal(got, np.array(times))
    np.testing.assert_array_equal(st["id"], ref["id"])
    for k in STATE:
        if kep == 0:
            np.testing.assert_array_equal(st[k], ref[k], err_msg=k)
        else:
            assert np.abs(st[k] - ref[k]).max() <= 1e-9 * np.abs(ref[k]).max()


@pytest.mark.parametrize("method", ["sia21h.dkd", "sia43h.kdk", "sia45a.dkd"])
def test_subtree_and_host_paths_give_identical_bits(method):
    ps = ics.plummer(600, eps=1e-3, seed=12, masses="salpeter")
    res = []
    for sub in (0, 128):
        d = DeviceSIA(ps, method, 1.0 / 64, mode="exact")
        d.set_subtree(sub)
        d.evolve(1.0, max_steps=2)
        res.append((d.state(), d.stats()))
        d.close()
    (a, sa), (b, sb) = res
    for k in ("id", "nstep") + STATE:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert sa["recursions"] == sb["recursions"]
    assert sa["kepler"] == sb["kepler"]
    assert sa["max_depth"] == sb["max_depth"]


def test_split_subtree_close_to_host_path():
    # SPLIT sums in the single-CTA kernel (FP32 runs added in double) and in
    # the sweep kernels (Kahan-folded lanes) differ only by rounding.
    ps = ics.plummer(100, eps=1e-3, seed=21)
    res = []
    for sub in (0, 128):
        d = DeviceSIA(ps, "sia44s.kdk", 1.0 / 128, mode="split")
        d.set_subtree(sub)
        d.evolve(1.0, max_steps=3)
        res.append(d.state())
        d.close()
    a, b = res
    np.testing.assert_array_equal(a["id"], b["id"])
    for k, tol in (("rx", 1e-10), ("vx", 1e-8), ("vz", 1e-8)):
        assert np.abs(a[k] - b[k]).max() <= tol * np.abs(a[k]).max(), k


def test_split_sia_shared_steps_close_to_exact():
    ps = ics.plummer(4096, eps=1e-4, seed=6)
    res = {}
    for mode in ("exact", "split"):
        d = DeviceSIA(ps, "sia21s.dkd", 1.0 / 128, mode=mode)
        d.evolve(1.0, max_steps=4)
        res[mode] = d.state()
        d.close()
    np.testing.assert_array_equal(res["exact"]["id"], res["split"]["id"])
    for k, tol in (("rx", 1e-9), ("ry", 1e-9), ("rz", 1e-9),
                   ("vx", 1e-7), ("vy", 1e-7), ("vz", 1e-7)):
        e, s = res["exact"][k], res["split"][k]
        assert np.abs(e - s).max() <= tol * np.abs(e).max(), k


def test_split_sia_hierarchical_conserves_energy():
    ps = ics.plummer(2048, eps=1e-3, seed=8, masses="salpeter")
    k0, p0 = oi.energies({k: ps[k].copy() for k in ps})
    d = DeviceSIA(ps, "sia21h.dkd", 1.0 / 32, mode="split")
    d.evolve(1.0 / 8)
    st = d.state()
    stats = d.stats()
    d.close()
    assert stats["max_depth"] >= 2 and stats["partitions"] > 0
    fin = {k: ps[k][st["id"]] for k in ("m", "e2")}
    fin.update({k: st[k] for k in ("rx", "ry", "rz", "vx", "vy", "vz")})
    k1, p1 = oi.energies(fin)
    assert abs((k1 + p1) - (k0 + p0)) / abs(k0 + p0) < 1e-4
    assert np.all(st["time"] == 1.0 / 8)


def test_method_names():
    assert len(SIA_METHODS) == 48
    with pytest.raises(ValueError):
        DeviceSIA(ics.plummer(8, eps=1e-2, seed=1), "sia33h.dkd", 0.01)
