"""The integrator oracle on 1- and 2-particle systems against the
reference's own runs (golden_tiny.npz): a lone particle's step is eta
exactly, a power of two, which tupan quantises to eta / 2."""

import os

import numpy as np
import pytest

from oracle import integrators as oi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_tiny.npz")
KEYS = ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")


def tiny_runs():
    z = np.load(GOLDEN)
    for k in range(int(z["runs"])):
        tag = "%d/" % k
        ps = {a: z[tag + "in/" + a].copy() for a in KEYS}
        eta, t_end = (float(x) for x in z[tag + "params"])
        out = {a: z[tag + "out/" + a] for a in KEYS[2:]}
        yield str(z[tag + "method"]), ps, eta, t_end, z[tag + "steps"], out


@pytest.mark.parametrize("run", list(tiny_runs()),
                         ids=lambda r: "%s-n%d" % (r[0], len(r[1]["m"])))
def test_oracle_tiny_systems_bit_identical_to_reference(run):
    method, ps, eta, t_end, steps, out = run
    got_steps = oi.evolve(ps, t_end, eta, method)
    np.testing.assert_array_equal(np.array(got_steps), steps)
    for a, v in out.items():
        np.testing.assert_array_equal(ps[a], v)
    if len(ps["m"]) == 1:
        assert steps[0] == eta / 2
