"""The CPU-runnable configuration in full (Plummer N=256, equal masses,
eps=1e-4, ahermite4 with eta=1/64 to t_end=1): the numpy integrator oracle
against the reference's own run (golden_config1.npz) -- every step size,
the final state and the energies."""

import os

import numpy as np

from oracle import integrators as oi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_config1.npz")


def test_config1_ahermite4_matches_reference_run():
    z = np.load(GOLDEN)
    ps = {k: z["in/" + k].copy() for k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    eta, t_end = z["params"]
    k0, p0 = oi.energies(ps)
    np.testing.assert_allclose([k0, p0], z["energy0"], rtol=1e-13)
    steps = oi.evolve(ps, float(t_end), float(eta), "ahermite4")
    np.testing.assert_array_equal(np.array(steps), z["steps"])
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        np.testing.assert_array_equal(ps[k], z["out/" + k])
    k1, p1 = oi.energies(ps)
    np.testing.assert_allclose([k1, p1], z["energy1"], rtol=1e-13)
    de = ((k1 + p1) - (k0 + p0)) / abs(k0 + p0)
    assert abs(de) < 1e-10
