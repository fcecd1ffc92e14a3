"""Device-resident NREG driver (csrc/nreg.cu) against the reference's own
nreg/anreg runs (golden_nreg.npz): every step time, the scalars W, U, S,
E0 and the final state, bit for bit."""

import os

import numpy as np
import pytest

from oracle import integrators as oi
from tupan_gb300 import ics
from tupan_gb300.integrator import DeviceNreg

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_nreg.npz")


def runs():
    z = np.load(GOLDEN)
    return sorted({int(k.split("/")[0]) for k in z.files})


@pytest.mark.parametrize("r", runs())
def test_nreg_bit_identical_to_reference(r):
    z = np.load(GOLDEN)
    tag = "%d/" % r
    ps = {k: z[tag + "in/" + k].copy() for k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    eta, t_end, max_steps = z[tag + "params"]
    d = DeviceNreg(ps, str(z[tag + "method"]), float(eta))
    times = d.evolve(float(t_end), max_steps=int(max_steps))
    st = d.state()
    d.close()
    np.testing.assert_array_equal(times, z[tag + "times"])
    np.testing.assert_array_equal([st["W"], st["U"], st["S"], st["E0"]],
                                  z[tag + "scalars"])
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        np.testing.assert_array_equal(st[k], z[tag + "out/" + k], err_msg=k)


@pytest.mark.parametrize("n", [7, 129, 1000, 5003])
def test_nreg_matches_oracle_at_other_sizes(n):
    # sizes that exercise every branch of the pairwise summation tree
    ps = ics.plummer(n, eps=1e-2, seed=n)
    ref = {k: v.copy() for k, v in ps.items()}
    st, times = oi.nreg_evolve(ref, 1.0, 1.0 / 64, "anreg", max_steps=3)
    d = DeviceNreg(ps, "anreg", 1.0 / 64)
    got = d.evolve(1.0, max_steps=3)
    out = d.state()
    d.close()
    np.testing.assert_array_equal(got, np.array(times))
    assert [out["W"], out["U"], out["S"]] == [st.W, st.U, st.S]
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
