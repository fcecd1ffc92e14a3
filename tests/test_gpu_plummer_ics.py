"""Plummer initial conditions with the three Phi sweeps on the GPU: EXACT
mode gives exactly the model the oracle's sweeps give on the same host, and
the reference's own model (golden_plummer_ics.npz, made on another host) to
the last bits of numpy's transcendental functions; SPLIT-mode sweeps keep
the model within their error."""

import os

import numpy as np
import pytest

import oracle
from tupan_gb300.plummer import make_plummer

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_plummer_ics.npz")
KEYS = ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz", "phi")


def oracle_phi(ps):
    return oracle.run("phi_kernel", ps, ps)[0]


@pytest.mark.parametrize("imf,n", [(("equalmass",), 2048),
                                   (("salpeter1955", 0.5, 10.0), 777)])
def test_gpu_phi_model_equals_oracle_model(imf, n):
    timing = {}
    got = make_plummer(n, 1e-4, imf, seed=9, timing=timing)
    want = make_plummer(n, 1e-4, imf, seed=9, phi_fn=oracle_phi)
    assert timing["phi_sweeps"] == 3
    for k in KEYS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)


def test_gpu_model_matches_reference_fixture():
    z = np.load(GOLDEN)
    for r in sorted({int(k.split("/")[0]) for k in z.files}):
        tag = "%d/" % r
        n, eps, seed, stype = z[tag + "params"]
        imf = [str(x) for x in z[tag + "imf"]]
        imf = (imf[0],) + tuple(float(x) for x in imf[1:])
        got = make_plummer(int(n), float(eps), imf, seed=int(seed),
                           softening_type=int(stype))
        for k in KEYS:
            w = z[tag + k]
            scale = np.abs(w).max()
            assert np.abs(got[k] - w).max() <= 1e-12 * scale, (r, k)


def test_split_phi_model_close():
    exact = make_plummer(4096, 1e-4, ("equalmass",), seed=5)
    split = make_plummer(4096, 1e-4, ("equalmass",), seed=5,
                         phi_mode="split")
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        scale = np.abs(exact[k]).max()
        assert np.abs(split[k] - exact[k]).max() <= 1e-5 * scale, k
