"""Sakura sweep with queued Kepler-branch pairs, the batched pair solver and
the learned start (device arrays given as torch tensors or raw pointers)."""

import ctypes

import numpy as np

from . import lib

_VP = ctypes.c_void_p


def _declare(L):
    c = ctypes
    L.tupan_gb300_kepler_set_mlp.argtypes = [_VP] * 7 + [c.c_float]
    L.tupan_gb300_kepler_set_mlp.restype = c.c_int
    L.tupan_gb300_kepler_pairs.argtypes = [
        c.c_uint64, c.c_double, _VP, _VP, _VP, _VP, _VP, _VP, _VP, c.c_int,
        c.c_longlong, _VP]
    L.tupan_gb300_kepler_pairs.restype = c.c_int
    L.tupan_gb300_sakura_queue.argtypes = [
        c.c_uint64, c.POINTER(_VP), c.c_uint64, c.POINTER(_VP), c.c_double,
        c.c_int64, c.POINTER(_VP), c.c_int, c.c_longlong, _VP,
        c.POINTER(c.c_ulonglong), c.POINTER(c.c_longlong), c.c_int]
    L.tupan_gb300_sakura_queue.restype = c.c_int
    L.tupan_gb300_kepler_set_form.argtypes = [c.c_int]
    L.tupan_gb300_kepler_set_form.restype = c.c_int


def _lib():
    L = lib.load("float64")
    if not getattr(L, "_kepler_declared", False):
        _declare(L)
        L._kepler_declared = True
    return L


def _ptr(t):
    return None if t is None else t.data_ptr()


def sakura_queue(ni, i_ptrs, nj, j_ptrs, out_ptrs, dt, flag, use_mlp=False,
                 budget=0, stream=None, histogram=False, mode="exact"):
    """sakura_kernel over device arrays (flag -1 or +1).  Returns the number
    of Kepler-branch pairs and, if asked, the Laguerre-update histogram.
    mode "split": leapfrog-branch pairs in FP32 on double-single positions
    (the Kepler branch stays fp64)."""
    L = _lib()
    ia = (_VP * 8)(*i_ptrs)
    ja = (_VP * 8)(*j_ptrs)
    oa = (_VP * 6)(*out_ptrs)
    nk = ctypes.c_ulonglong()
    hist = (ctypes.c_longlong * 65)() if histogram else None
    st = L.tupan_gb300_sakura_queue(int(ni), ia, int(nj), ja, float(dt),
                                    int(flag), oa, 1 if use_mlp else 0,
                                    int(budget), stream, ctypes.byref(nk),
                                    hist, lib.MODE_SPLIT if mode == "split"
                                    else lib.MODE_EXACT)
    if st:
        raise lib.TupanGB300Error("sakura_queue failed: status %d" % st)
    return nk.value, (np.array(hist[:]) if histogram else None)


def kepler_pairs(n, dt, m, e2, state, out, iters=None, rec_x=None,
                 rec_y=None, use_mlp=False, budget=0, stream=None):
    """Solve n pairs (device tensors); see tupan_gb300_kepler_pairs."""
    st = _lib().tupan_gb300_kepler_pairs(
        int(n), float(dt), _ptr(m), _ptr(e2), _ptr(state), _ptr(out),
        _ptr(iters), _ptr(rec_x), _ptr(rec_y), 1 if use_mlp else 0,
        int(budget), stream)
    if st:
        raise lib.TupanGB300Error("kepler_pairs failed: status %d" % st)


FORMS = {"reference": 0, "shared": 1, "mixed": 2}


def set_form(form):
    """Root-solve form of the pair solver and the Sakura paths: "reference"
    (the reference's structure), "shared" (one cos/sin per Laguerre update,
    bit-identical) or "mixed" (FP32 updates, then FP64 to the reference's
    tolerance).  Returns the previous form's name."""
    old = _lib().tupan_gb300_kepler_set_form(FORMS[form])
    if old < 0:
        raise ValueError(form)
    return {v: k for k, v in FORMS.items()}[old]


def set_mlp(w1, b1, w2, b2, w3, b3, norm, gate=float("-inf")):
    """Install the learned start (device tensors; bf16 weights), used where
    log(|dt| sqrt(m / r^3)) > gate."""
    st = _lib().tupan_gb300_kepler_set_mlp(*[_ptr(t) for t in
                                             (w1, b1, w2, b2, w3, b3, norm)],
                                           float(gate))
    if st:
        raise lib.TupanGB300Error("set_mlp failed")


def clear_mlp():
    _lib().tupan_gb300_kepler_set_mlp(None, None, None, None, None, None,
                                      None, 0.0)


_DP = ctypes.POINTER(ctypes.c_double)


class DeviceSakura(object):
    """Fixed-step Sakura integrator (tupan/integrator/sakura.py:22-50) with
    the particles resident on the GPU and queued Kepler-branch solves."""

    KEYS = ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")

    def __init__(self, ps, mode="exact"):
        L = _lib()
        c = ctypes
        L.tupan_gb300_sakura_set_mode.argtypes = [_VP, c.c_int]
        L.tupan_gb300_sakura_set_mode.restype = c.c_int
        L.tupan_gb300_sakura_create.argtypes = [c.c_uint64] + [_DP] * 8 + [
            c.POINTER(_VP)]
        L.tupan_gb300_sakura_create.restype = c.c_int
        L.tupan_gb300_sakura_evolve.argtypes = [
            _VP, c.c_double, c.c_double, c.c_int, _DP,
            c.POINTER(c.c_longlong), c.POINTER(c.c_longlong),
            c.POINTER(c.c_longlong)]
        L.tupan_gb300_sakura_evolve.restype = c.c_int
        L.tupan_gb300_sakura_get_state.argtypes = [_VP] + [_DP] * 6
        L.tupan_gb300_sakura_get_state.restype = c.c_int
        L.tupan_gb300_sakura_destroy.argtypes = [_VP]
        L.tupan_gb300_sakura_destroy.restype = c.c_int
        self.L = L
        self.n = len(ps["m"])
        arrs = [np.ascontiguousarray(ps[k], dtype=np.float64)
                for k in self.KEYS]
        h = _VP()
        st = L.tupan_gb300_sakura_create(self.n,
                                         *[a.ctypes.data_as(_DP) for a in arrs],
                                         ctypes.byref(h))
        if st:
            raise lib.TupanGB300Error("sakura_create failed: status %d" % st)
        self.h = h
        self.hist = np.zeros(65, np.int64)
        if mode != "exact":
            if L.tupan_gb300_sakura_set_mode(
                    h, lib.MODE_SPLIT if mode == "split" else -1):
                raise ValueError("unexpected mode: %r" % (mode,))

    def evolve(self, tau, t_end, use_mlp=False):
        t = ctypes.c_double()
        k = ctypes.c_longlong()
        nk = ctypes.c_longlong()
        h = (ctypes.c_longlong * 65)()
        st = self.L.tupan_gb300_sakura_evolve(self.h, float(tau), float(t_end),
                                              1 if use_mlp else 0,
                                              ctypes.byref(t), ctypes.byref(k),
                                              ctypes.byref(nk), h)
        if st:
            raise lib.TupanGB300Error("sakura_evolve failed: status %d" % st)
        self.hist += np.array(h[:])
        return t.value, k.value, nk.value

    def state(self):
        out = {c: np.empty(self.n) for c in ("rx", "ry", "rz", "vx", "vy", "vz")}
        st = self.L.tupan_gb300_sakura_get_state(
            self.h, *[out[c].ctypes.data_as(_DP)
                      for c in ("rx", "ry", "rz", "vx", "vy", "vz")])
        if st:
            raise lib.TupanGB300Error("sakura_get_state failed")
        return out

    def close(self):
        if self.h:
            self.L.tupan_gb300_sakura_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
