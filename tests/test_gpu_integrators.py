"""Device-resident Hermite driver against tupan's own integrator runs
(golden_integrators.npz) and the numpy integrator oracle."""

import os

import numpy as np
import pytest

from oracle import integrators as oi
from tupan_gb300 import ics
from tupan_gb300.integrator import DeviceHermite

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "golden_integrators.npz")
ORDER = {"ahermite2": 2, "ahermite4": 4, "hermite4": 4, "ahermite6": 6,
         "ahermite8": 8}


def load(method):
    z = np.load(GOLDEN)
    tag = method + "/"
    ps = {k: z[tag + "in/" + k].copy() for k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    eta, t_end, max_steps = z[tag + "params"]
    out = {k: z[tag + "out/" + k] for k in
           ("rx", "ry", "rz", "vx", "vy", "vz")}
    return ps, float(eta), float(t_end), int(max_steps), z[tag + "steps"], out


@pytest.mark.parametrize("method", list(ORDER))
@pytest.mark.parametrize("batch", [1, 7])
def test_exact_hermite_bit_identical_to_reference(method, batch):
    ps, eta, t_end, max_steps, steps, out = load(method)
    h = DeviceHermite(ps, eta, order=ORDER[method],
                      adaptive=method.startswith("a"), mode="exact",
                      record_steps=1000)
    h.evolve(t_end, max_steps=max_steps, batch=batch)
    np.testing.assert_array_equal(h.steps(), steps)
    got = h.state()
    for k, v in out.items():
        np.testing.assert_array_equal(got[k], v)
    h.close()


@pytest.mark.parametrize("batch", [1, 4])
def test_exact_hermite_tiny_systems_bit_identical_to_reference(batch):
    # 1- and 2-particle systems (golden_tiny.npz): a lone particle's step is
    # eta exactly, a power of two that the quantisation halves
    from tests.test_oracle_tiny import tiny_runs
    for method, ps, eta, t_end, steps, out in tiny_runs():
        h = DeviceHermite(ps, eta, order=ORDER[method], adaptive=True,
                          mode="exact", record_steps=1000)
        h.evolve(t_end, batch=batch)
        np.testing.assert_array_equal(h.steps(), steps)
        got = h.state()
        for k, v in out.items():
            np.testing.assert_array_equal(got[k], v)
        h.close()


def test_split_hermite4_energy_and_steps():
    # Config 1 shape (Plummer, eta = 1/64, eps = 1e-4) over a short time.
    # The energy diagnostic is fp64; SPLIT forces add FP32 force noise, so
    # the bound is the fp64 run's error or 1e-9, whichever is larger.
    ps = ics.plummer(256, eps=1e-4, seed=1)
    ref = {k: v.copy() for k, v in ps.items()}
    ke0, pe0 = oi.energies(ref)
    steps = oi.evolve(ref, 0.0625, 1.0 / 64, "ahermite4")
    ke1, pe1 = oi.energies(ref)
    de_ref = ((ke1 + pe1) - (ke0 + pe0)) / -pe0
    h = DeviceHermite(ps, 1.0 / 64, order=4, adaptive=True, mode="split",
                      record_steps=100000)
    k0, p0 = h.energy()
    assert abs(k0 - ke0) <= 1e-12 * abs(ke0)
    assert abs(p0 - pe0) <= 1e-12 * abs(pe0)
    h.evolve(0.0625, batch=16)
    k1, p1 = h.energy()
    de = ((k1 + p1) - (k0 + p0)) / -p0
    assert abs(h.time - 0.0625) == 0.0
    assert abs(de) <= max(10 * abs(de_ref), 1e-9), (de, de_ref)
    assert len(h.steps()) == len(steps)
    h.close()


def test_split_hermite_at_large_n_takes_the_centred_sweeps():
    # N = 65536: the SPLIT force sweeps of the device driver go through the
    # centred kernels; two fixed steps agree with the fp64 EXACT run to the
    # SPLIT force accuracy carried through the steps: median deviation
    # <= 1e-9 of each field's scale; max <= 1e-6 (close pairs, whose
    # accelerations are large, carry the largest: measured 3.5e-8 in vx)
    from tupan_gb300 import lib
    n = 65536
    assert lib.sweep_plan("acc_jerk_kernel", n, n)[0] == 1
    ps = ics.plummer(n, eps=1e-4, seed=5)
    res = {}
    for mode in ("split", "exact"):
        h = DeviceHermite(ps, 1.0 / 256, order=4, adaptive=False, mode=mode)
        h.evolve(2.0 / 256, batch=2)
        assert h.nsteps == 2
        res[mode] = h.state()
        h.close()
    for c in ("rx", "ry", "rz", "vx", "vy", "vz"):
        scale = np.abs(ps[c]).max()
        dev = np.abs(res["split"][c] - res["exact"][c]) / scale
        assert np.median(dev) <= 1e-9 and dev.max() <= 1e-6, (
            c, np.median(dev), dev.max())


# ---------------------------------------------------------------------------
# Individual block time steps
# ---------------------------------------------------------------------------
from tupan_gb300.integrator import DeviceBlockHermite  # noqa: E402


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("order", [4, 6, 8])
def test_exact_block_steps_bit_identical_to_oracle(order, graphs):
    # graphs: the steps run as CUDA graphs with the active set sized on the
    # device (WHILE over steps, SWITCH over active-count levels); else the
    # active count is read back each step
    ps = ics.plummer(96, eps=1e-4, seed=40 + order, masses="salpeter")
    eta, dt_max = 1.0 / 32, 1.0 / 16
    st = oi.block_init(ps, order, eta, dt_max)
    active = []
    for _ in range(40):
        t, na = oi.block_step(st, order, eta, dt_max)
        active.append(na)
    assert min(active) < len(ps["m"])          # the sets really vary
    b = DeviceBlockHermite(ps, eta, dt_max, order=order, mode="exact",
                           graphs=graphs)
    b.evolve(1e30, max_steps=40)
    assert b.launch_mode == ("graphs" if graphs else "host")
    assert b.nsteps == 40
    assert b.time == t
    assert b.active == sum(active)
    got = b.state()
    for k in ("rx", "ry", "rz", "vx", "vy", "vz", "t", "dt"):
        np.testing.assert_array_equal(got[k], st[k], err_msg=k)
    b.close()


def test_block_steps_switch_between_launch_paths():
    # 15 steps on the graph path, 10 host-synchronised, 15 more on graphs:
    # the device-side block time and counters follow the host's
    ps = ics.plummer(200, eps=1e-4, seed=47, masses="salpeter")
    eta, dt_max, order = 1.0 / 32, 1.0 / 16, 4
    st = oi.block_init(ps, order, eta, dt_max)
    total = 0
    for _ in range(40):
        t, na = oi.block_step(st, order, eta, dt_max)
        total += na
    b = DeviceBlockHermite(ps, eta, dt_max, order=order, mode="exact")
    b.evolve(1e30, max_steps=15)
    b.L.tupan_gb300_block_set_graphs(b.h, 0)
    b.evolve(1e30, max_steps=10)
    b.L.tupan_gb300_block_set_graphs(b.h, 1)
    b.evolve(1e30, max_steps=15)
    assert b.nsteps == 40 and b.time == t and b.active == total
    got = b.state()
    for k in ("rx", "ry", "rz", "vx", "vy", "vz", "t", "dt"):
        np.testing.assert_array_equal(got[k], st[k], err_msg=k)
    b.close()


def test_split_block_steps_energy():
    ps = ics.plummer(2048, eps=1e-4, seed=3, masses="salpeter")
    eta, dt_max, t_end = 1.0 / 32, 1.0 / 32, 1.0 / 16
    k0, p0 = oi.energies(ps)
    b = DeviceBlockHermite(ps, eta, dt_max, order=6, mode="split")
    b.evolve(t_end)
    assert b.time == t_end
    got = b.state()
    assert np.all(got["t"] == t_end)
    fin = dict(ps)
    fin.update({k: got[k] for k in ("rx", "ry", "rz", "vx", "vy", "vz")})
    k1, p1 = oi.energies(fin)
    de = ((k1 + p1) - (k0 + p0)) / -p0
    assert abs(de) < 1e-6, de
    assert b.active < b.nsteps * len(ps["m"])
    b.close()
