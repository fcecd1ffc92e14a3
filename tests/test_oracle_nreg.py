"""Pin the NREG restatement (oracle/integrators.py nreg_*) to short runs of
the reference's own NREG integrators (golden_nreg.npz), and the restated
summation order to numpy's."""

import os

import numpy as np
import pytest

from oracle import integrators as oi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_nreg.npz")


def runs():
    z = np.load(GOLDEN)
    return sorted({int(k.split("/")[0]) for k in z.files})


def load(r):
    z = np.load(GOLDEN)
    tag = "%d/" % r
    ps = {k: z[tag + "in/" + k].copy() for k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    eta, t_end, max_steps = z[tag + "params"]
    out = {k: z[tag + "out/" + k] for k in
           ("rx", "ry", "rz", "vx", "vy", "vz")}
    return (str(z[tag + "method"]), ps, float(eta), float(t_end),
            int(max_steps), z[tag + "times"], z[tag + "scalars"], out)


@pytest.mark.parametrize("r", runs())
def test_oracle_nreg_matches_reference(r):
    method, ps, eta, t_end, max_steps, times, scalars, out = load(r)
    st, got = oi.nreg_evolve(ps, t_end, eta, method, max_steps=max_steps)
    np.testing.assert_array_equal(np.array(got), times)
    np.testing.assert_array_equal([st.W, st.U, st.S, st.E0], scalars)
    for k, v in out.items():
        np.testing.assert_array_equal(ps[k], v, err_msg=k)


@pytest.mark.parametrize("n", list(range(0, 140)) + [255, 256, 257, 1000,
                                                      4097, 65536])
def test_pairwise_sum_is_numpy_sum(n):
    x = np.random.default_rng(n).standard_normal(n) * 10.0 ** \
        np.random.default_rng(n + 1).uniform(-3, 3, n)
    assert oi.pairwise_sum(x) == np.sum(x)
