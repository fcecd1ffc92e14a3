"""Pin the CPU oracle to the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py through tupan's public calc API)."""

import numpy as np
import pytest

import oracle
from tests import golden_cases

TRANSCENDENTAL = ("sakura_kernel", "kepler_solver_kernel")


def _params():
    for path in golden_cases.files():
        prec, data, cases, kepler = golden_cases.load(path)
        for (tag, name, ips, jps, scalars, expect) in cases:
            yield pytest.param(prec, name, ips, jps, scalars, expect,
                               id="%s:%s" % (path.rsplit("/", 1)[1], tag))


@pytest.mark.parametrize("prec,name,ips,jps,scalars,expect", list(_params()))
def test_oracle_matches_reference(prec, name, ips, jps, scalars, expect):
    got = oracle.run(name, ips, jps, scalars, prec)
    assert len(got) == len(expect)
    for g, e in zip(got, expect):
        if name in TRANSCENDENTAL:
            # libm's cos/sin/cosh/sinh/log may differ in the last bit between
            # C libraries; on the same machine the results are identical.
            tol = 1e-12 if prec == "float64" else 2e-5
            scale = np.maximum(np.abs(e), np.abs(e).max() * 1e-3 + 1e-300)
            assert np.all(np.abs(g - e) <= tol * scale), name
        else:
            np.testing.assert_array_equal(g, e)


def _kepler_params():
    for path in golden_cases.files():
        prec, data, cases, kepler = golden_cases.load(path)
        for (dt, pairs, res) in kepler:
            yield pytest.param(prec, data, dt, pairs, res,
                               id="%s:dt=%r" % (path.rsplit("/", 1)[1], dt))


@pytest.mark.parametrize("prec,data,dt,pairs,res", list(_kepler_params()))
def test_oracle_kepler_matches_reference(prec, data, dt, pairs, res):
    for row, p in enumerate(pairs):
        two = {a: np.ascontiguousarray(v[2 * p:2 * p + 2])
               for a, v in data.items()}
        got = np.concatenate(oracle.run("kepler_solver_kernel", two, None,
                                        {"dt": dt}, prec))
        tol = 1e-11 if prec == "float64" else 1e-4
        scale = np.abs(res[row]).max()
        assert np.max(np.abs(got - res[row])) <= tol * scale, (p, dt)
