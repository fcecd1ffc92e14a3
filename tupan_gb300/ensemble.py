"""Ensembles of independent N-body systems on one GPU (csrc/ensemble.cu):
each system has its own shared adaptive Hermite-4 step.  Batched mode: every
force evaluation of the ensemble is one persistent batched SPLIT launch;
persistent mode: one CTA steps one whole system at a time."""

import ctypes

import numpy as np

from . import ics, lib

_DP = ctypes.POINTER(ctypes.c_double)
_KEYS = ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")


def _declare(L):
    c = ctypes
    L.tupan_gb300_ensemble_create.argtypes = (
        [c.c_uint, c.POINTER(c.c_uint64), c.c_double] + [_DP] * 8
        + [c.POINTER(c.c_void_p)])
    L.tupan_gb300_ensemble_create.restype = c.c_int
    L.tupan_gb300_ensemble_evolve.argtypes = [c.c_void_p, c.c_double, c.c_int,
                                              c.POINTER(c.c_longlong)]
    L.tupan_gb300_ensemble_evolve.restype = c.c_int
    L.tupan_gb300_ensemble_energy.argtypes = [c.c_void_p, _DP, _DP]
    L.tupan_gb300_ensemble_energy.restype = c.c_int
    L.tupan_gb300_ensemble_get.argtypes = [c.c_void_p, _DP,
                                           c.POINTER(c.c_longlong)] + [_DP] * 6
    L.tupan_gb300_ensemble_get.restype = c.c_int
    L.tupan_gb300_ensemble_destroy.argtypes = [c.c_void_p]
    L.tupan_gb300_ensemble_destroy.restype = c.c_int
    L.tupan_gb300_ensemble_set_mode.argtypes = [c.c_void_p, c.c_int, c.c_int,
                                                c.c_int]
    L.tupan_gb300_ensemble_set_mode.restype = c.c_int
    L.tupan_gb300_ensemble_set_shape.argtypes = [c.c_void_p, c.c_int, c.c_int,
                                                 c.c_int]
    L.tupan_gb300_ensemble_set_shape.restype = c.c_int
    L.tupan_gb300_ensemble_get_shape.argtypes = [c.c_void_p] + [
        c.POINTER(c.c_int)] * 3
    L.tupan_gb300_ensemble_get_shape.restype = c.c_int
    L.tupan_gb300_ensemble_set_stage.argtypes = [c.c_void_p, c.c_int]
    L.tupan_gb300_ensemble_set_stage.restype = c.c_int


def set_default_shape(nt, ib, prefetch):
    """Launch shape of ensembles created later (see DeviceEnsemble.set_shape)."""
    L = lib.load("float64")
    _declare(L)
    if L.tupan_gb300_ensemble_set_shape(None, int(nt), int(ib), int(prefetch)):
        raise lib.TupanGB300Error("bad ensemble shape %r" % ((nt, ib, prefetch),))


def default_shape():
    L = lib.load("float64")
    _declare(L)
    v = [ctypes.c_int() for _ in range(3)]
    L.tupan_gb300_ensemble_get_shape(None, *[ctypes.byref(x) for x in v])
    return tuple(x.value for x in v)


def make_systems(count, lo=3, hi=512, eps=1e-4, seed=1):
    """Seeded ensemble: sizes uniform in [lo, hi], equal masses per system,
    each a Plummer sphere in N-body units."""
    sizes = ics.ensemble_sizes(count, lo, hi, seed)
    return [ics.plummer(int(n), eps=eps, seed=seed * 100003 + k)
            for k, n in enumerate(sizes)]


class DeviceEnsemble(object):
    def __init__(self, systems, eta):
        self.L = lib.load("float64")
        _declare(self.L)
        self.sizes = np.array([len(s["m"]) for s in systems], np.uint64)
        self.off = np.concatenate([[0], np.cumsum(self.sizes)]).astype(
            np.uint64)
        cat = {k: np.ascontiguousarray(np.concatenate([s[k] for s in systems]))
               for k in _KEYS}
        h = ctypes.c_void_p()
        st = self.L.tupan_gb300_ensemble_create(
            len(systems), self.off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            float(eta), *[cat[k].ctypes.data_as(_DP) for k in _KEYS],
            ctypes.byref(h))
        if st:
            raise lib.TupanGB300Error("ensemble_create failed: status %d" % st)
        self.h = h
        self.n_sys = len(systems)
        self.n = int(self.off[-1])

    def set_mode(self, mode, steps_per_launch=1024, switch_below=0):
        """"batched": every step of all systems as five launches (graph of
        `batch` steps); "persistent": one CTA per system for up to
        steps_per_launch steps per launch, handing the last systems (fewer
        than switch_below) to the batched mode."""
        m = {"batched": 0, "persistent": 1}[mode]
        st = self.L.tupan_gb300_ensemble_set_mode(
            self.h, m, int(steps_per_launch), int(switch_below))
        if st:
            raise lib.TupanGB300Error("ensemble_set_mode failed: status %d"
                                      % st)

    def set_shape(self, nt, ib, prefetch=1):
        """Batched sweep launch shape: nt threads per CTA (128 or 256), ib
        the full i-block of a work item (32..512), prefetch 1 to overlap the
        next item's record copy with the current item."""
        st = self.L.tupan_gb300_ensemble_set_shape(self.h, int(nt), int(ib),
                                                   int(prefetch))
        if st:
            raise lib.TupanGB300Error("ensemble_set_shape failed: status %d"
                                      % st)

    def set_stage(self, split):
        """1: each AccJerk sweep's predictor/corrector as a launch of its
        own; 0 (default, faster): inside the sweep (bit-identical results)."""
        st = self.L.tupan_gb300_ensemble_set_stage(self.h, int(split))
        if st:
            raise lib.TupanGB300Error("ensemble_set_stage failed: status %d"
                                      % st)

    @property
    def shape(self):
        v = [ctypes.c_int() for _ in range(3)]
        self.L.tupan_gb300_ensemble_get_shape(self.h,
                                              *[ctypes.byref(x) for x in v])
        return tuple(x.value for x in v)

    def evolve(self, t_end, batch=8):
        mx = ctypes.c_longlong()
        st = self.L.tupan_gb300_ensemble_evolve(self.h, float(t_end),
                                                int(batch), ctypes.byref(mx))
        if st:
            raise lib.TupanGB300Error("ensemble_evolve failed: status %d" % st)
        return mx.value

    def energies(self):
        ke = np.empty(self.n_sys)
        pe = np.empty(self.n_sys)
        st = self.L.tupan_gb300_ensemble_energy(self.h, ke.ctypes.data_as(_DP),
                                                pe.ctypes.data_as(_DP))
        if st:
            raise lib.TupanGB300Error("ensemble_energy failed")
        return ke, pe

    def state(self):
        t = np.empty(self.n_sys)
        k = np.empty(self.n_sys, np.int64)
        out = {c: np.empty(self.n) for c in ("rx", "ry", "rz", "vx", "vy", "vz")}
        st = self.L.tupan_gb300_ensemble_get(
            self.h, t.ctypes.data_as(_DP),
            k.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
            *[out[c].ctypes.data_as(_DP) for c in ("rx", "ry", "rz", "vx",
                                                   "vy", "vz")])
        if st:
            raise lib.TupanGB300Error("ensemble_get failed")
        return t, k, out

    def close(self):
        if self.h:
            self.L.tupan_gb300_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
