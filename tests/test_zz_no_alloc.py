"""The allocation-free acc_jerk entry point (tupan_gb300_acc_jerk_split_noalloc).

It exists for callers that cannot let the library call cudaMalloc, for
example a host application whose memory manager owns the whole device heap,
or a time-step loop that must not stall on cudaMalloc's device-wide
synchronisation.  The test calls it through the C-ABI on caller-owned device
buffers, twice in a row with different particle sets (its scratch arrays are
shared by every call and keep the previous contents), and checks each result
against the fp64 oracle (the reference's arithmetic) with the bounds of the
SPLIT tests, and against the library's regular SPLIT entry point.  The
second call must leave the device's free memory unchanged.  Sizes above the
stated maximum are refused before anything runs.
"""

import ctypes

import numpy as np
import pytest

import oracle
from tupan_gb300 import ics, lib

pytestmark = pytest.mark.gpu

NAMES = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")
MAX_N = 65536


def _entry():
    L = lib.load("float64")
    f = L.tupan_gb300_acc_jerk_split_noalloc
    f.argtypes = ([ctypes.c_uint64] + [ctypes.c_void_p] * 8
                  + [ctypes.c_uint64] + [ctypes.c_void_p] * 8
                  + [ctypes.c_void_p] * 6 + [ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_uint)])
    f.restype = ctypes.c_int
    return f


def _device(ps, n, torch, dev):
    return {k: torch.from_numpy(np.ascontiguousarray(ps[k][:n])).to(dev)
            for k in NAMES}


def _rel(a, b):
    return np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)


def test_noalloc_matches_oracle_twice():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    f = _entry()
    cases = [(ics.plummer(20000, eps=1e-4, seed=31), 20000, 20000),
             (ics.plummer(MAX_N, eps=1e-4, seed=32), 777, MAX_N)]
    for call, (ps, ni, nj) in enumerate(cases):
        I = _device(ps, ni, torch, dev)
        J = _device(ps, nj, torch, dev)
        out = [torch.full((ni,), float("nan"), dtype=torch.float64, device=dev)
               for _ in range(6)]
        err = ctypes.c_uint(12345)
        args = ([ni] + [I[k].data_ptr() for k in NAMES]
                + [nj] + [J[k].data_ptr() for k in NAMES]
                + [o.data_ptr() for o in out] + [None, ctypes.byref(err)])
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        st = f(*args)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(dev)[0]
        assert st == 0 and err.value == 0
        if call > 0:
            # the static arrays were set up by the first call: nothing more
            # is taken from the device heap
            assert free1 == free0
        got = np.stack([o.cpu().numpy() for o in out])
        assert np.all(np.isfinite(got))

        sub = {k: np.ascontiguousarray(ps[k][:ni]) for k in NAMES}
        js = {k: np.ascontiguousarray(ps[k][:nj]) for k in NAMES}
        want = np.stack(oracle.run("acc_jerk_kernel", sub, js))
        ea = _rel(got[:3], want[:3])
        ej = _rel(got[3:], want[3:])
        assert np.median(ea) <= 1e-7 and ea.max() <= 2e-6, ea.max()
        assert ej.max() <= 1e-4 and np.median(ej) <= 1e-6, (ej.max(),
                                                            np.median(ej))

        want_t = [torch.empty(ni, dtype=torch.float64, device=dev)
                  for _ in range(6)]
        lib.dev_sweep("acc_jerk_kernel", ni, [I[k].data_ptr() for k in NAMES],
                      nj, [J[k].data_ptr() for k in NAMES],
                      [o.data_ptr() for o in want_t], mode=lib.MODE_SPLIT,
                      sync=True)
        lib_out = np.stack([o.cpu().numpy() for o in want_t])
        assert _rel(got[:3], lib_out[:3]).max() <= 2e-6


def test_noalloc_refuses_oversized_requests():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    f = _entry()
    x = torch.zeros(MAX_N + 1, dtype=torch.float64, device=dev)
    p = x.data_ptr()
    err = ctypes.c_uint(0)
    st = f(MAX_N + 1, *([p] * 8), 10, *([p] * 8), *([p] * 6), None,
           ctypes.byref(err))
    assert st == 5
    assert float(x.abs().sum().item()) == 0.0
