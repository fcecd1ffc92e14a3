"""Ensemble driver (batched persistent SPLIT sweeps, or one CTA per system,
per-system steps) against the fp64 integrator oracle run system by system."""

import numpy as np
import pytest

from oracle import integrators as oi
from tupan_gb300.ensemble import DeviceEnsemble, make_systems

pytestmark = pytest.mark.gpu

# (mode, steps per persistent launch, switch to batched below this many
# systems): batched only; persistent to the end in launches of 3 steps;
# persistent launches of 5 steps handing the last systems to batched mode
MODES = [("batched", 1024, 0), ("persistent", 3, 0), ("persistent", 5, 8)]


@pytest.mark.parametrize("mode", MODES)
def test_ensemble_matches_per_system_oracle(mode):
    systems = make_systems(24, lo=3, hi=120, seed=5)
    t_end, eta = 1.0 / 32, 1.0 / 64
    ens = DeviceEnsemble(systems, eta)
    ens.set_mode(*mode)
    ke0, pe0 = ens.energies()
    ens.evolve(t_end, batch=4)
    t, k, st = ens.state()
    ke1, pe1 = ens.energies()
    assert np.all(t == t_end)
    off = ens.off
    for s, ps in enumerate(systems):
        ref = {c: v.copy() for c, v in ps.items()}
        k0, p0 = oi.energies(ref)
        steps = oi.evolve(ref, t_end, eta, "ahermite4")
        assert abs(ke0[s] - k0) <= 1e-13 * abs(k0)
        assert abs(pe0[s] - p0) <= 1e-12 * abs(p0)
        assert k[s] == len(steps), s
        a, b = int(off[s]), int(off[s + 1])
        for c in ("rx", "ry", "rz", "vx", "vy", "vz"):
            scale = np.abs(ref[c]).max() + 1e-30
            assert np.max(np.abs(st[c][a:b] - ref[c])) <= 1e-6 * scale, (s, c)
    de = ((ke1 + pe1) - (ke0 + pe0)) / -pe0
    assert np.all(np.abs(de) < 1e-6), np.abs(de).max()
    ens.close()


@pytest.mark.parametrize("mode", MODES)
def test_ensemble_systems_of_every_size_finish(mode):
    systems = make_systems(300, lo=3, hi=512, seed=9)
    ens = DeviceEnsemble(systems, 1.0 / 64)
    ens.set_mode(*mode)
    ens.evolve(1.0 / 64, batch=8)
    t, k, _ = ens.state()
    assert np.all(t == 1.0 / 64) and np.all(k >= 1)
    ens.close()


@pytest.mark.parametrize("mode", MODES)
def test_ensemble_evolve_in_stages_reaches_each_end_time(mode):
    # the captured step graph must pick up the t_end of each evolve call
    systems = make_systems(40, lo=3, hi=200, seed=10)
    ens = DeviceEnsemble(systems, 1.0 / 64)
    ens.set_mode(*mode)
    for t_end in (1.0 / 256, 1.0 / 128, 1.0 / 64):
        ens.evolve(t_end, batch=4)
        t, k, _ = ens.state()
        assert np.all(t == t_end), (t_end, t.min(), t.max())
    ens.close()


def test_ensemble_persistent_matches_batched():
    # the same stages and arithmetic; only the order of the j sums differs
    # (FP32 sums agree to about 1e-7 of |a|, which a few steps carry into
    # the state at a few 1e-9 of its scale)
    systems = make_systems(60, lo=3, hi=512, seed=12)
    out = []
    for mode in (("batched", 1024, 0), ("persistent", 7, 0)):
        ens = DeviceEnsemble(systems, 1.0 / 64)
        ens.set_mode(*mode)
        ens.evolve(1.0 / 128, batch=4)
        out.append(ens.state())
        ens.close()
    (t0, k0, s0), (t1, k1, s1) = out
    assert np.all(t0 == t1) and np.all(k0 == k1)
    for c in ("rx", "ry", "rz", "vx", "vy", "vz"):
        scale = np.abs(s0[c]).max()
        assert np.max(np.abs(s0[c] - s1[c])) <= 1e-7 * scale, c


def test_ensemble_set_mode_rejects_bad_arguments():
    systems = make_systems(2, lo=3, hi=8, seed=1)
    ens = DeviceEnsemble(systems, 1.0 / 64)
    import tupan_gb300.lib as lib
    for bad in (("persistent", 0, 0), ("persistent", 4, -1)):
        with pytest.raises(lib.TupanGB300Error):
            ens.set_mode(*bad)
    ens.close()


@pytest.mark.parametrize("mode", MODES)
def test_ensemble_one_and_two_particle_systems(mode):
    # a lone particle drifts; a pair is a two-body orbit; both next to a
    # larger system
    big = make_systems(1, lo=64, hi=64, seed=3)[0]
    one = {k: np.ascontiguousarray(v[:1]) for k, v in big.items()}
    two = {k: np.ascontiguousarray(v[1:3]) for k, v in big.items()}
    systems = [big, one, two]
    t_end, eta = 1.0 / 64, 1.0 / 64
    ens = DeviceEnsemble(systems, eta)
    ens.set_mode(*mode)
    ens.evolve(t_end, batch=4)
    t, k, st = ens.state()
    assert np.all(t == t_end) and np.all(k >= 1)
    off = ens.off
    for s, ps in enumerate(systems):
        ref = {c: v.copy() for c, v in ps.items()}
        steps = oi.evolve(ref, t_end, eta, "ahermite4")
        assert k[s] == len(steps), s
        a, b = int(off[s]), int(off[s + 1])
        for c in ("rx", "ry", "rz", "vx", "vy", "vz"):
            scale = np.abs(ref[c]).max() + 1e-30
            assert np.max(np.abs(st[c][a:b] - ref[c])) <= 1e-6 * scale, (s, c)
    ens.close()


# batched sweep launch shapes: (threads per CTA, full i-block, prefetch)
SHAPES = [(128, 128, 0), (128, 128, 1), (256, 256, 1), (128, 32, 1),
          (256, 64, 0), (128, 512, 1)]


@pytest.mark.parametrize("shape", SHAPES)
def test_ensemble_shapes_match_per_system_oracle(shape):
    systems = make_systems(40, lo=3, hi=512, seed=21)
    t_end, eta = 1.0 / 64, 1.0 / 64
    ens = DeviceEnsemble(systems, eta)
    ens.set_shape(*shape)
    assert ens.shape == shape
    ens.evolve(t_end, batch=4)
    t, k, st = ens.state()
    assert np.all(t == t_end)
    off = ens.off
    for s, ps in enumerate(systems):
        ref = {c: v.copy() for c, v in ps.items()}
        steps = oi.evolve(ref, t_end, eta, "ahermite4")
        assert k[s] == len(steps), s
        a, b = int(off[s]), int(off[s + 1])
        for c in ("rx", "ry", "rz", "vx", "vy", "vz"):
            scale = np.abs(ref[c]).max() + 1e-30
            assert np.max(np.abs(st[c][a:b] - ref[c])) <= 1e-6 * scale, (s, c)
    ens.close()


@pytest.mark.parametrize("nt,ib", [(128, 128), (256, 64)])
def test_ensemble_prefetch_is_bit_identical(nt, ib):
    # the double-buffered copy changes when records arrive, not what is
    # computed from them
    systems = make_systems(200, lo=3, hi=512, seed=22)
    out = []
    for pf in (0, 1):
        ens = DeviceEnsemble(systems, 1.0 / 64)
        ens.set_shape(nt, ib, pf)
        ens.evolve(1.0 / 64, batch=4)
        out.append(ens.state())
        ens.close()
    (t0, k0, s0), (t1, k1, s1) = out
    np.testing.assert_array_equal(t0, t1)
    np.testing.assert_array_equal(k0, k1)
    for c in s0:
        np.testing.assert_array_equal(s0[c], s1[c])


def test_ensemble_shape_default_and_rejects():
    import tupan_gb300.lib as lib
    from tupan_gb300 import ensemble as en
    old = en.default_shape()
    try:
        en.set_default_shape(256, 64, 0)
        systems = make_systems(3, lo=3, hi=30, seed=2)
        ens = DeviceEnsemble(systems, 1.0 / 64)
        assert ens.shape == (256, 64, 0)
        for bad in ((64, 128, 1), (128, 96, 1), (128, 128, 2)):
            with pytest.raises(lib.TupanGB300Error):
                ens.set_shape(*bad)
            with pytest.raises(lib.TupanGB300Error):
                en.set_default_shape(*bad)
        ens.evolve(1.0 / 128, batch=2)
        ens.close()
    finally:
        en.set_default_shape(*old)


@pytest.mark.parametrize("shape", [(128, 128, 0), (256, 64, 1)])
def test_ensemble_stage_launch_is_bit_identical(shape):
    # the predictor/corrector as launches of their own or inside the sweeps:
    # the same arithmetic on the same forces
    systems = make_systems(150, lo=3, hi=512, seed=23)
    out = []
    for split in (0, 1):
        ens = DeviceEnsemble(systems, 1.0 / 64)
        ens.set_shape(*shape)
        ens.set_stage(split)
        ens.evolve(1.0 / 64, batch=4)
        out.append(ens.state())
        ens.close()
    (t0, k0, s0), (t1, k1, s1) = out
    np.testing.assert_array_equal(t0, t1)
    np.testing.assert_array_equal(k0, k1)
    for c in s0:
        np.testing.assert_array_equal(s0[c], s1[c])
