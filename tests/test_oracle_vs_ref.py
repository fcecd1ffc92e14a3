"""Pin the CPU oracle to the reference kernels compiled from their own
source files (``oracle/_ref``, ``make -C oracle ref``), where those sources
exist: on the inputs of every golden case, in double and float, the two
libraries must agree bit for bit (the same machine and C library, so the
Sakura/Kepler transcendentals agree too)."""

import numpy as np
import pytest

import oracle
from tests import golden_cases

pytestmark = pytest.mark.skipif(
    not (oracle.ref_available("float64") and oracle.ref_available("float32")),
    reason="reference kernels not compiled here (oracle/_ref)")


def _params():
    for path in golden_cases.files():
        prec, data, cases, kepler = golden_cases.load(path)
        for (tag, name, ips, jps, scalars, expect) in cases:
            yield pytest.param(prec, name, ips, jps, scalars,
                               id="%s:%s" % (path.rsplit("/", 1)[1], tag))


@pytest.mark.parametrize("prec,name,ips,jps,scalars", list(_params()))
def test_oracle_bit_identical_to_reference_build(prec, name, ips, jps,
                                                 scalars):
    got = oracle.run(name, ips, jps, scalars, prec)
    want = oracle.run_ref(name, ips, jps, scalars, prec)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


def _kepler_params():
    for path in golden_cases.files():
        prec, data, cases, kepler = golden_cases.load(path)
        for (dt, pairs, res) in kepler:
            yield pytest.param(prec, data, dt, pairs,
                               id="%s:dt=%r" % (path.rsplit("/", 1)[1], dt))


@pytest.mark.parametrize("prec,data,dt,pairs", list(_kepler_params()))
def test_oracle_kepler_bit_identical_to_reference_build(prec, data, dt,
                                                        pairs):
    for p in pairs:
        two = {a: np.ascontiguousarray(v[2 * p:2 * p + 2])
               for a, v in data.items()}
        got = oracle.run("kepler_solver_kernel", two, None, {"dt": dt}, prec)
        two = {a: np.ascontiguousarray(v[2 * p:2 * p + 2])
               for a, v in data.items()}
        want = oracle.run_ref("kepler_solver_kernel", two, None, {"dt": dt},
                              prec)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)
