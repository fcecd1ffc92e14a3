"""The bounded copy-pipeline wait, made to run out on purpose.

Every sweep that streams j-records through a shared-memory ring waits on an
mbarrier for each bulk copy, with a bounded number of tries.  Setting that
bound to 0 (``set_pipe_spin_limit(0)``) makes every main-loop wait give up at
once, so the error path runs without any fault: the CTA records
DERR_PIPE_TIMEOUT, waits (with the full bound) for its copies still in
flight, and leaves without writing results.  The host sees status 3 with the
error bit, the outputs keep their previous contents, and the next call with
the normal bound is correct.
"""

import ctypes

import numpy as np
import pytest

import oracle
from tupan_gb300 import ics, lib
from tupan_gb300.ensemble import DeviceEnsemble, make_systems

pytestmark = pytest.mark.gpu

NAMES = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")


def _configure(policy, gsplit):
    """policy 0: the double-single split variants; 1: the centred sweep."""
    if policy == 1:
        lib.set_centred(1, -1, gsplit)
    else:
        lib.set_centred(0)
        lib.set_split_config("acc_jerk_kernel", 9, gsplit)


def _restore():
    lib.set_centred(-1, -1, 0)
    lib.set_split_config("acc_jerk_kernel", -1, 0)


def _sweep(torch, ps, n, policy, gsplit):
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(ps[k][:n])).to(dev)
         for k in NAMES}
    out = [torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
           for _ in range(6)]
    ptr = [d[k].data_ptr() for k in NAMES]
    VP = ctypes.c_void_p
    _configure(policy, gsplit)
    try:
        st = lib.load().tupan_gb300_dev_sweep(
            lib.KERNEL_ID["acc_jerk_kernel"], lib.MODE_SPLIT, n,
            (VP * 8)(*ptr), n, (VP * 8)(*ptr), None, 0,
            (VP * 6)(*[o.data_ptr() for o in out]), None, 1)
    finally:
        _restore()
    return st, [o.cpu().numpy() for o in out]


POLICIES = [(0, 1), (0, 4), (1, 1), (1, 4)]


@pytest.mark.parametrize("policy,gsplit", POLICIES)
def test_pipeline_timeout_is_reported_and_recoverable(policy, gsplit):
    torch = pytest.importorskip("torch")
    n = 3000
    ps = ics.plummer(n, eps=1e-4, seed=12)
    old = lib.set_pipe_spin_limit(0)
    try:
        st, out = _sweep(torch, ps, n, policy, gsplit)
    finally:
        lib.set_pipe_spin_limit(old)
    L = lib.load()
    assert st == 3
    assert L.tupan_gb300_last_device_error() & lib.DERR_PIPE_TIMEOUT
    # no sweep CTA and no partial-sum pass wrote an output
    assert all(np.all(np.isnan(o)) for o in out)
    # the context is intact and the normal bound gives a correct answer
    st, out = _sweep(torch, ps, n, policy, gsplit)
    assert st == 0
    want = oracle.run("acc_jerk_kernel", ps, ps)
    g = np.stack(out[:3])
    w = np.stack(want[:3])
    err = np.linalg.norm(g - w, axis=0) / np.linalg.norm(w, axis=0)
    assert np.median(err) <= 1e-7 and err.max() <= 2e-6, (err.max(),
                                                          np.median(err))


def test_ensemble_pipeline_timeout_is_reported():
    systems = make_systems(24, lo=3, hi=200, seed=5)

    def run():
        e = DeviceEnsemble(systems, 1.0 / 64)
        try:
            e.evolve(1.0 / 32)
            return e.state()
        finally:
            e.close()

    t0, k0, s0 = run()
    e = DeviceEnsemble(systems, 1.0 / 64)
    old = lib.set_pipe_spin_limit(0)
    try:
        with pytest.raises(lib.TupanGB300Error, match="status 3"):
            e.evolve(1.0 / 32)
    finally:
        lib.set_pipe_spin_limit(old)
        e.close()
    t1, k1, s1 = run()
    np.testing.assert_array_equal(t1, t0)
    np.testing.assert_array_equal(k1, k0)
    for c in s0:
        np.testing.assert_array_equal(s1[c], s0[c])
