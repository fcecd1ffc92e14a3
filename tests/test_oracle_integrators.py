"""Pin the numpy integrator restatement (oracle/integrators.py) to short runs
of the reference's own integrators (golden_integrators.npz)."""

import os

import numpy as np
import pytest

from oracle import integrators as oi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_integrators.npz")
METHODS = ["ahermite4", "hermite4", "ahermite6", "ahermite8", "ahermite2",
           "sakura", "asakura"]


def load(method):
    z = np.load(GOLDEN)
    tag = method + "/"
    ps = {k: z[tag + "in/" + k].copy() for k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    eta, t_end, max_steps = z[tag + "params"]
    out = {k: z[tag + "out/" + k] for k in
           ("rx", "ry", "rz", "vx", "vy", "vz")}
    return ps, float(eta), float(t_end), int(max_steps), z[tag + "steps"], out


@pytest.mark.parametrize("method", METHODS)
def test_oracle_integrator_matches_reference(method):
    ps, eta, t_end, max_steps, steps, out = load(method)
    got_steps = oi.evolve(ps, t_end, eta, method, max_steps=max_steps)
    np.testing.assert_array_equal(np.array(got_steps), steps)
    for k, v in out.items():
        if "sakura" in method:
            # Kepler branch: libm transcendental functions
            np.testing.assert_allclose(ps[k], v, rtol=1e-12, atol=1e-14)
        else:
            np.testing.assert_array_equal(ps[k], v)


def test_block_tstep_matches_formula_on_edges():
    # tupan/integrator/__init__.py:59-78 on powers of two and neighbours
    rng = np.random.default_rng(3)
    vals = []
    for k in range(-30, 4):
        p = 2.0 ** k
        vals += [p, np.nextafter(p, 0), np.nextafter(p, 1), p * 1.5]
    vals += list(10 ** rng.uniform(-9, 0.5, 200))
    for t in (0.0, 0.25, 0.125 + 2 ** -20, 3.0):
        for tau in (1.0 / 64, 1.0, -0.5):
            for v in vals:
                got = oi.block_tstep(v, t, tau)
                assert abs(got) <= abs(tau)
                if abs(got) < abs(tau):
                    m = abs(got)
                    assert m == 2.0 ** round(np.log2(m))
                    assert (t + m) % m == 0 or (t + 2 ** int(np.log2(v) - 1)) % m == 0
