"""PNAcc in SPLIT mode (FP32 pair arithmetic on double-single positions)
against the fp64 oracle, order by order (pnacc_kernel_common.h:8-70,
pn_terms.h:473-567).

The PN acceleration is a small correction (terms of order v^2/c^2 and
beyond) evaluated from long polynomials whose terms partly cancel, so its
FP32 error relative to itself is larger than the Newtonian force's.  Bounds
per particle, |da_PN| / |a_PN|: median <= 1e-5 and max <= 1e-3; orders 0
and 1 have no terms and must give exactly zero.
"""

import numpy as np
import pytest

import oracle
from tupan_gb300 import abi, ics, lib

pytestmark = pytest.mark.gpu


def pn_scalars(order, c=128.0):
    d = {"order": order}
    for k in range(1, 8):
        d["inv%d" % k] = (1.0 / c) ** k
    return d


def run(ps, sc, mode):
    old = lib.set_mode(mode)
    try:
        fn = lib.bind("pnacc_kernel")
        vals = abi.make_args("pnacc_kernel", "float64", ps, ps, sc)
        abi.call(fn, "pnacc_kernel", "float64", vals)
        lib.check()
        return np.stack(abi.outputs("pnacc_kernel", vals))
    finally:
        lib.set_mode(old)


def systems():
    yield "plummer", ics.plummer(2000, eps=1e-4, seed=41)
    rng = np.random.default_rng(42)
    n = 600
    d = {"m": rng.random(n) / n, "e2": np.zeros(n)}
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        d[k] = rng.random(n) * 10 - 5
    yield "uniform", d


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6, 7])
def test_pnacc_split_per_order(order):
    for tag, ps in systems():
        sc = pn_scalars(order)
        want = np.stack(oracle.run("pnacc_kernel", ps, ps, sc))
        got = run(ps, sc, lib.MODE_SPLIT)
        assert np.all(np.isfinite(got)), tag
        if order <= 1:
            assert np.all(got == 0.0) and np.all(want == 0.0)
            continue
        e = np.linalg.norm(got - want, axis=0) / np.linalg.norm(want, axis=0)
        print(tag, order, "max %.3g median %.3g" % (e.max(), np.median(e)))
        assert np.median(e) <= 1e-5 and e.max() <= 1e-3, (tag, e.max(),
                                                           np.median(e))


def test_pnacc_split_takes_the_split_path():
    pytest.importorskip("torch")
    v, g = lib.split_choice("pnacc_kernel", 2000, 2000)
    assert 0 <= v < lib.load().tupan_gb300_split_variants()
