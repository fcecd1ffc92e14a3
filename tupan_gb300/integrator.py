"""Device-resident integrators on the CUDA library.

``DeviceHermite`` keeps one particle system in HBM and advances it with
tupan's Hermite scheme (tupan/integrator/hermite.py: H2/H4/H6/H8, P(EC)^2,
shared steps; ``adaptive=True`` is tupan's "ahermiteN" with the Tstep kernel
and power-of-two quantisation of tupan/integrator/__init__.py:59-78).  Steps
are replayed from a CUDA graph; the host only reads the time between
batches.  With ``mode="exact"`` a run is bit-identical to tupan's own
integrator on its C backend.
"""

import ctypes

import numpy as np

from . import lib

_DP = ctypes.POINTER(ctypes.c_double)


def _declare(L):
    c = ctypes
    L.tupan_gb300_hermite_create.argtypes = (
        [c.c_uint64, c.c_int, c.c_int, c.c_int, c.c_double] + [_DP] * 8
        + [c.c_longlong, c.POINTER(c.c_void_p)])
    L.tupan_gb300_hermite_create.restype = c.c_int
    L.tupan_gb300_hermite_evolve.argtypes = [
        c.c_void_p, c.c_double, c.c_longlong, c.c_int, _DP,
        c.POINTER(c.c_longlong)]
    L.tupan_gb300_hermite_evolve.restype = c.c_int
    L.tupan_gb300_hermite_get_state.argtypes = [c.c_void_p] + [_DP] * 6
    L.tupan_gb300_hermite_get_state.restype = c.c_int
    L.tupan_gb300_hermite_tau_log.argtypes = [c.c_void_p, _DP, c.c_longlong]
    L.tupan_gb300_hermite_tau_log.restype = c.c_longlong
    L.tupan_gb300_hermite_energy.argtypes = [c.c_void_p, _DP, _DP]
    L.tupan_gb300_hermite_energy.restype = c.c_int
    L.tupan_gb300_hermite_destroy.argtypes = [c.c_void_p]
    L.tupan_gb300_hermite_destroy.restype = c.c_int


def _p(a):
    return a.ctypes.data_as(_DP)


class DeviceHermite(object):
    """One N-body system integrated on the GPU."""

    def __init__(self, ps, eta, order=4, adaptive=True, mode="split",
                 record_steps=0):
        self.L = lib.load("float64")
        _declare(self.L)
        self.n = len(ps["m"])
        self.eta = float(eta)
        arrs = [np.ascontiguousarray(ps[k], dtype=np.float64)
                for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")]
        h = ctypes.c_void_p()
        st = self.L.tupan_gb300_hermite_create(
            self.n, int(order), 1 if adaptive else 0,
            lib.MODE_SPLIT if mode == "split" else lib.MODE_EXACT,
            self.eta, *[_p(a) for a in arrs], int(record_steps),
            ctypes.byref(h))
        if st:
            raise lib.TupanGB300Error("hermite_create failed: status %d" % st)
        self.h = h
        self.time = 0.0
        self.nsteps = 0

    def evolve(self, t_end, max_steps=0, batch=16):
        t = ctypes.c_double()
        k = ctypes.c_longlong()
        st = self.L.tupan_gb300_hermite_evolve(self.h, float(t_end),
                                               int(max_steps), int(batch),
                                               ctypes.byref(t),
                                               ctypes.byref(k))
        if st:
            raise lib.TupanGB300Error("hermite_evolve failed: status %d" % st)
        self.time = t.value
        self.nsteps = k.value
        return self.time

    def state(self):
        out = {k: np.empty(self.n) for k in ("rx", "ry", "rz", "vx", "vy",
                                             "vz")}
        st = self.L.tupan_gb300_hermite_get_state(
            self.h, *[_p(out[k]) for k in ("rx", "ry", "rz", "vx", "vy",
                                           "vz")])
        if st:
            raise lib.TupanGB300Error("hermite_get_state failed")
        return out

    def steps(self, cap=1 << 20):
        buf = np.empty(cap)
        k = self.L.tupan_gb300_hermite_tau_log(self.h, _p(buf), cap)
        return buf[:k].copy()

    def energy(self):
        ke = ctypes.c_double()
        pe = ctypes.c_double()
        st = self.L.tupan_gb300_hermite_energy(self.h, ctypes.byref(ke),
                                               ctypes.byref(pe))
        if st:
            raise lib.TupanGB300Error("hermite_energy failed")
        return ke.value, pe.value

    def close(self):
        if self.h:
            self.L.tupan_gb300_hermite_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _declare_block(L):
    c = ctypes
    L.tupan_gb300_block_create.argtypes = (
        [c.c_uint64, c.c_int, c.c_int, c.c_double, c.c_double] + [_DP] * 8
        + [c.POINTER(c.c_void_p)])
    L.tupan_gb300_block_create.restype = c.c_int
    L.tupan_gb300_block_evolve.argtypes = [
        c.c_void_p, c.c_double, c.c_longlong, _DP, c.POINTER(c.c_longlong),
        c.POINTER(c.c_longlong)]
    L.tupan_gb300_block_evolve.restype = c.c_int
    L.tupan_gb300_block_get_state.argtypes = [c.c_void_p] + [_DP] * 8
    L.tupan_gb300_block_get_state.restype = c.c_int
    L.tupan_gb300_block_destroy.argtypes = [c.c_void_p]
    L.tupan_gb300_block_destroy.restype = c.c_int
    L.tupan_gb300_block_set_graphs.argtypes = [c.c_void_p, c.c_int]
    L.tupan_gb300_block_set_graphs.restype = c.c_int
    L.tupan_gb300_block_launch_mode.argtypes = [c.c_void_p]
    L.tupan_gb300_block_launch_mode.restype = c.c_int


class DeviceBlockHermite(object):
    """Hermite (order 4, 6 or 8) with individual power-of-two block steps,
    device resident; see csrc/blockstep.cu for the scheme."""

    def __init__(self, ps, eta, dt_max, order=4, mode="split", graphs=True):
        """graphs: launch batches of block steps as one CUDA graph (active
        set sized on the device); False: read the active count back each
        step and launch for it."""
        self.L = lib.load("float64")
        _declare_block(self.L)
        self.n = len(ps["m"])
        arrs = [np.ascontiguousarray(ps[k], dtype=np.float64)
                for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")]
        h = ctypes.c_void_p()
        st = self.L.tupan_gb300_block_create(
            self.n, int(order),
            lib.MODE_SPLIT if mode == "split" else lib.MODE_EXACT,
            float(eta), float(dt_max), *[_p(a) for a in arrs],
            ctypes.byref(h))
        if st:
            raise lib.TupanGB300Error("block_create failed: status %d" % st)
        self.h = h
        self.time = 0.0
        self.nsteps = 0
        self.active = 0
        self.L.tupan_gb300_block_set_graphs(h, 1 if graphs else 0)

    @property
    def launch_mode(self):
        """"graphs" or "host" (the path the evolution takes)."""
        return "graphs" if self.L.tupan_gb300_block_launch_mode(self.h) == 1 \
            else "host"

    def evolve(self, t_end, max_steps=0):
        t = ctypes.c_double()
        k = ctypes.c_longlong()
        a = ctypes.c_longlong()
        st = self.L.tupan_gb300_block_evolve(self.h, float(t_end),
                                             int(max_steps), ctypes.byref(t),
                                             ctypes.byref(k), ctypes.byref(a))
        if st:
            raise lib.TupanGB300Error("block_evolve failed: status %d" % st)
        self.time, self.nsteps, self.active = t.value, k.value, a.value
        return self.time

    def state(self):
        keys = ("rx", "ry", "rz", "vx", "vy", "vz", "t", "dt")
        out = {k: np.empty(self.n) for k in keys}
        st = self.L.tupan_gb300_block_get_state(self.h,
                                                *[_p(out[k]) for k in keys])
        if st:
            raise lib.TupanGB300Error("block_get_state failed")
        return out

    def close(self):
        if self.h:
            self.L.tupan_gb300_block_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _declare_sia(L):
    c = ctypes
    lp = c.POINTER(c.c_longlong)
    L.tupan_gb300_sia_create.argtypes = (
        [c.c_uint64, c.c_char_p, c.c_double, c.c_int] + [_DP] * 8
        + [c.POINTER(c.c_void_p)])
    L.tupan_gb300_sia_create.restype = c.c_int
    L.tupan_gb300_sia_evolve.argtypes = [c.c_void_p, c.c_double, c.c_longlong,
                                         _DP, lp, _DP, c.c_longlong]
    L.tupan_gb300_sia_evolve.restype = c.c_int
    L.tupan_gb300_sia_get_state.argtypes = ([c.c_void_p, lp] + [_DP] * 7
                                            + [lp, _DP])
    L.tupan_gb300_sia_get_state.restype = c.c_int
    L.tupan_gb300_sia_stats.argtypes = [c.c_void_p, lp]
    L.tupan_gb300_sia_stats.restype = c.c_int
    L.tupan_gb300_sia_set_subtree.argtypes = [c.c_void_p, c.c_int]
    L.tupan_gb300_sia_set_subtree.restype = c.c_int
    L.tupan_gb300_sia_destroy.argtypes = [c.c_void_p]
    L.tupan_gb300_sia_destroy.restype = c.c_int


SIA_METHODS = tuple("sia%s%s.%s" % (s, m, k)
                    for s in ("21", "22", "43", "44", "45", "46", "67", "69")
                    for m in "sah" for k in ("dkd", "kdk"))


class DeviceSIA(object):
    """tupan's SIA integrators (tupan/integrator/sia.py; methods
    ``sia21s.dkd`` .. ``sia69h.kdk``) with the particles in HBM; see
    csrc/sia.cu.  The particle order changes at every split like the
    reference's; ``state()`` returns it with each particle's ``id``.
    Newtonian only."""

    def __init__(self, ps, method, eta, mode="exact"):
        if method not in SIA_METHODS:
            raise ValueError("unexpected SIA method: %r" % (method,))
        self.L = lib.load("float64")
        _declare_sia(self.L)
        self.n = len(ps["m"])
        arrs = [np.ascontiguousarray(ps[k], dtype=np.float64)
                for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")]
        h = ctypes.c_void_p()
        st = self.L.tupan_gb300_sia_create(
            self.n, method.encode(), float(eta),
            lib.MODE_SPLIT if mode == "split" else lib.MODE_EXACT,
            *[_p(a) for a in arrs], ctypes.byref(h))
        if st:
            raise lib.TupanGB300Error("sia_create failed: status %d" % st)
        self.h = h
        self.time = 0.0

    def evolve(self, t_end, max_steps=0):
        """Base steps until |t| >= t_end (or max_steps); returns the time
        after each step taken by this call."""
        cap = int(max_steps) if max_steps else 1 << 16
        log = np.zeros(cap)
        t = ctypes.c_double()
        k = ctypes.c_longlong()
        st = self.L.tupan_gb300_sia_evolve(self.h, float(t_end),
                                           int(max_steps), ctypes.byref(t),
                                           ctypes.byref(k), _p(log), cap)
        if st:
            raise lib.TupanGB300Error("sia_evolve failed: status %d" % st)
        self.time = t.value
        return log[:min(k.value, cap)].copy()

    def state(self):
        out = {k: np.empty(self.n) for k in
               ("rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep")}
        out["id"] = np.empty(self.n, dtype=np.int64)
        out["nstep"] = np.empty(self.n, dtype=np.int64)
        lp = ctypes.POINTER(ctypes.c_longlong)
        st = self.L.tupan_gb300_sia_get_state(
            self.h, out["id"].ctypes.data_as(lp),
            *[_p(out[k]) for k in ("rx", "ry", "rz", "vx", "vy", "vz",
                                   "time")],
            out["nstep"].ctypes.data_as(lp), _p(out["tstep"]))
        if st:
            raise lib.TupanGB300Error("sia_get_state failed")
        return out

    def set_subtree(self, max_n):
        """Subsystems of at most ``max_n`` (<= 128) particles run their
        whole recursion in one CTA; 0 drives every level from the host.
        Both give the same bits."""
        old = self.L.tupan_gb300_sia_set_subtree(self.h, int(max_n))
        if old < 0:
            raise ValueError("max_n must be in 0..128")
        return old

    def stats(self):
        s = np.zeros(9, dtype=np.int64)
        self.L.tupan_gb300_sia_stats(
            self.h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        return dict(zip(("recursions", "kepler", "sweeps", "partitions",
                         "max_depth", "steps", "subtrees", "subtree_us",
                         "interactions"), (int(x) for x in s)))

    def close(self):
        if self.h:
            self.L.tupan_gb300_sia_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _declare_nreg(L):
    c = ctypes
    L.tupan_gb300_nreg_create.argtypes = (
        [c.c_uint64, c.c_int, c.c_double] + [_DP] * 8
        + [c.POINTER(c.c_void_p)])
    L.tupan_gb300_nreg_create.restype = c.c_int
    L.tupan_gb300_nreg_evolve.argtypes = [
        c.c_void_p, c.c_double, c.c_longlong, _DP, c.POINTER(c.c_longlong),
        _DP, c.c_longlong]
    L.tupan_gb300_nreg_evolve.restype = c.c_int
    L.tupan_gb300_nreg_get_state.argtypes = [c.c_void_p] + [_DP] * 7
    L.tupan_gb300_nreg_get_state.restype = c.c_int
    L.tupan_gb300_nreg_destroy.argtypes = [c.c_void_p]
    L.tupan_gb300_nreg_destroy.restype = c.c_int


class DeviceNreg(object):
    """tupan's regularised-time integrators ``nreg`` and ``anreg``
    (tupan/integrator/nreg.py) with the particles in HBM; see csrc/nreg.cu.
    EXACT sweeps and numpy's summation order: bit-identical to the
    reference's runs."""

    def __init__(self, ps, method, eta):
        if method not in ("nreg", "anreg"):
            raise ValueError("unexpected NREG method: %r" % (method,))
        self.L = lib.load("float64")
        _declare_nreg(self.L)
        self.n = len(ps["m"])
        arrs = [np.ascontiguousarray(ps[k], dtype=np.float64)
                for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")]
        h = ctypes.c_void_p()
        st = self.L.tupan_gb300_nreg_create(
            self.n, 1 if method == "anreg" else 0, float(eta),
            *[_p(a) for a in arrs], ctypes.byref(h))
        if st:
            raise lib.TupanGB300Error("nreg_create failed: status %d" % st)
        self.h = h

    def evolve(self, t_end, max_steps=0):
        cap = int(max_steps) if max_steps else 1 << 16
        log = np.zeros(cap)
        t = ctypes.c_double()
        k = ctypes.c_longlong()
        st = self.L.tupan_gb300_nreg_evolve(self.h, float(t_end),
                                            int(max_steps), ctypes.byref(t),
                                            ctypes.byref(k), _p(log), cap)
        if st:
            raise lib.TupanGB300Error("nreg_evolve failed: status %d" % st)
        return log[:min(k.value, cap)].copy()

    def state(self):
        out = {k: np.empty(self.n) for k in
               ("rx", "ry", "rz", "vx", "vy", "vz")}
        sc = np.zeros(5)
        st = self.L.tupan_gb300_nreg_get_state(
            self.h, *[_p(out[k]) for k in ("rx", "ry", "rz", "vx", "vy",
                                           "vz")], _p(sc))
        if st:
            raise lib.TupanGB300Error("nreg_get_state failed")
        out.update(zip(("W", "U", "S", "E0", "t"), (float(x) for x in sc)))
        return out

    def close(self):
        if self.h:
            self.L.tupan_gb300_nreg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
