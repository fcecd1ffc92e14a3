"""Pin the numpy SIA restatement (oracle/sia.py) to short runs of the
reference's own SIA integrators (golden_sia.npz, made by
tests/golden/make_golden.py --sia)."""

import os

import numpy as np
import pytest

from oracle import sia

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_sia.npz")


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
           ("id", "rx", "ry", "rz", "vx", "vy", "vz", "time", "nstep",
            "tstep")}
    return (str(z[tag + "method"]), ps, float(eta), float(t_end),
            int(max_steps), z[tag + "times"], out)


@pytest.mark.parametrize("r", runs())
def test_oracle_sia_matches_reference(r):
    method, ps, eta, t_end, max_steps, times, out = load(r)
    st, got_times = sia.evolve(ps, method, eta, t_end, max_steps=max_steps)
    np.testing.assert_array_equal(np.array(got_times), times)
    # same final particle order (the reference reorders at every join)
    np.testing.assert_array_equal(st["id"], out["id"])
    np.testing.assert_array_equal(st["nstep"], out["nstep"])
    for k in ("rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep"):
        np.testing.assert_array_equal(st[k], out[k], err_msg=method + " " + k)


def test_sequences_are_palindromes_with_unit_sums():
    for scheme in sia.COEFS:
        seq = sia.sequence(scheme)
        assert seq == seq[::-1]
        outer = sum(c for o, c in seq if o)
        inner = sum(c for o, c in seq if not o)
        assert abs(outer - 1) < 1e-12 and abs(inner - 1) < 1e-12, scheme
