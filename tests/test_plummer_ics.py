"""tupan_gb300.plummer.make_plummer against the reference's own
make_plummer (golden_plummer_ics.npz): with the oracle's Phi sweep in place
of the GPU's, every array is bit-identical -- the restated sampling,
rescaling and energies follow the reference's numpy calls exactly."""

import os

import numpy as np
import pytest

import oracle
from tupan_gb300.plummer import make_plummer

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_plummer_ics.npz")
KEYS = ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz", "phi")


def runs():
    z = np.load(GOLDEN)
    return sorted({int(k.split("/")[0]) for k in z.files})


def oracle_phi(ps):
    return oracle.run("phi_kernel", ps, ps)[0]


def params(r):
    z = np.load(GOLDEN)
    tag = "%d/" % r
    n, eps, seed, stype = z[tag + "params"]
    imf = [str(x) for x in z[tag + "imf"]]
    imf = (imf[0],) + tuple(float(x) for x in imf[1:])
    want = {k: z[tag + k] for k in KEYS}
    return int(n), float(eps), imf, int(seed), int(stype), want


@pytest.mark.parametrize("r", runs())
def test_make_plummer_matches_reference(r):
    n, eps, imf, seed, stype, want = params(r)
    timing = {}
    ps = make_plummer(n, eps, imf, seed=seed, softening_type=stype,
                      phi_fn=oracle_phi, timing=timing)
    assert timing["phi_sweeps"] == 3
    for k in KEYS:
        np.testing.assert_array_equal(ps[k], want[k], err_msg=k)
