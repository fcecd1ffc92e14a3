"""ctypes loader of the in-tree CUDA libraries.

``libtupan_gb300.so`` exports the float64 prototypes of tupan's
``libtupan.h`` and ``libtupan_gb300_sp.so`` the float32 ones, plus the
``tupan_gb300_*`` extension entry points.  Loading fails loudly when a
library is missing: there is no CPU fallback.
"""

import ctypes
import os
import threading

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIBNAMES = {"float64": "libtupan_gb300.so", "float32": "libtupan_gb300_sp.so"}

# Kernel ids of the C-ABI (tg::KernelId), in libtupan.h order.
KERNEL_ID = {name: k for k, name in enumerate(abi.KERNEL_NAMES)}

MODE_EXACT = 0
MODE_SPLIT = 1

DERR_PIPE_TIMEOUT = 1
DERR_KEPLER_BUDGET = 2

_lock = threading.Lock()
_libs = {}


class TupanGB300Error(RuntimeError):
    """A CUDA or argument error reported by the library."""


def library_path(prec="float64"):
    return os.path.join(HERE, LIBNAMES[prec])


def _declare(L):
    c = ctypes
    L.tupan_gb300_last_error.restype = c.c_int
    L.tupan_gb300_last_error_message.restype = c.c_char_p
    L.tupan_gb300_last_device_error.restype = c.c_uint
    L.tupan_gb300_set_mode.argtypes = [c.c_int]
    L.tupan_gb300_set_mode.restype = c.c_int
    L.tupan_gb300_get_mode.restype = c.c_int
    L.tupan_gb300_set_kepler_budget.argtypes = [c.c_longlong]
    L.tupan_gb300_set_kepler_budget.restype = c.c_longlong
    L.tupan_gb300_set_split_config.argtypes = [c.c_int, c.c_int, c.c_int]
    L.tupan_gb300_set_split_config.restype = c.c_int
    L.tupan_gb300_set_tuned.argtypes = [c.c_int, c.c_uint64, c.c_uint64,
                                        c.c_int, c.c_int]
    L.tupan_gb300_set_tuned.restype = c.c_int
    L.tupan_gb300_split_choice.argtypes = [c.c_int, c.c_uint64, c.c_uint64,
                                           c.POINTER(c.c_int),
                                           c.POINTER(c.c_int)]
    L.tupan_gb300_split_choice.restype = c.c_int
    L.tupan_gb300_split_variants.restype = c.c_int
    L.tupan_gb300_split_variant_info.argtypes = [c.c_int] + [
        c.POINTER(c.c_int)] * 3
    L.tupan_gb300_split_variant_info.restype = None
    L.tupan_gb300_dev_sweep.argtypes = [
        c.c_int, c.c_int, c.c_uint64, c.POINTER(c.c_void_p), c.c_uint64,
        c.POINTER(c.c_void_p), c.POINTER(c.c_double), c.c_int64,
        c.POINTER(c.c_void_p), c.c_void_p, c.c_int]
    L.tupan_gb300_dev_sweep.restype = c.c_int
    L.tupan_gb300_kernel_arity.argtypes = [c.c_int, c.POINTER(c.c_int),
                                           c.POINTER(c.c_int)]
    L.tupan_gb300_kernel_arity.restype = c.c_int
    L.tupan_gb300_device_sms.restype = c.c_int
    L.tupan_gb300_real_bits.restype = c.c_int
    L.tupan_gb300_set_centred.argtypes = [c.c_int, c.c_int, c.c_int]
    L.tupan_gb300_set_centred.restype = c.c_int
    L.tupan_gb300_set_centred_mid.argtypes = [c.c_double]
    L.tupan_gb300_set_centred_mid.restype = c.c_double
    L.tupan_gb300_sweep_plan.argtypes = [c.c_int, c.c_uint64, c.c_uint64] + [
        c.POINTER(c.c_int)] * 3
    L.tupan_gb300_sweep_plan.restype = c.c_int
    L.tupan_gb300_set_pipe_spin_limit.argtypes = [c.c_uint]
    L.tupan_gb300_set_pipe_spin_limit.restype = c.c_uint
    L.tupan_gb300_device_name.argtypes = [c.c_char_p, c.c_int]
    L.tupan_gb300_device_name.restype = c.c_int


def load(prec="float64"):
    """The CUDA library for ``prec``; raises if it was not built."""
    with _lock:
        if prec not in _libs:
            path = library_path(prec)
            if not os.path.exists(path):
                raise TupanGB300Error(
                    "CUDA library %s is not built; run "
                    "`python -m tupan_gb300.build` (there is no CPU "
                    "fallback)" % path)
            L = ctypes.CDLL(path)
            _declare(L)
            _libs[prec] = L
            fresh = prec == "float64"
        else:
            fresh = False
    if fresh:
        _apply_tuning()
    return _libs[prec]


def _apply_tuning():
    """This GPU's saved autotuner entries (split sweep and block-step level
    shapes, the ensemble shape), once per process; TUPAN_GB300_NO_TUNING=1
    keeps the built-in choices."""
    if os.environ.get("TUPAN_GB300_NO_TUNING"):
        return
    if device_name() is None:
        return
    from . import autotune
    try:
        autotune.apply_saved(strict=False)
    except (OSError, ValueError) as exc:      # an unreadable table
        import warnings
        warnings.warn("tuning table not applied: %s" % exc)


def device_name():
    """Name of the current CUDA device, or None without one."""
    buf = ctypes.create_string_buffer(256)
    if load("float64").tupan_gb300_device_name(buf, 256):
        return None
    return buf.value.decode()


def check(prec="float64"):
    """Raise TupanGB300Error if the last call on ``prec``'s library failed."""
    L = load(prec)
    st = L.tupan_gb300_last_error()
    if st:
        msg = L.tupan_gb300_last_error_message().decode(errors="replace")
        raise TupanGB300Error("status %d: %s" % (st, msg))


def set_mode(mode, prec="float64"):
    """Select EXACT (0) or SPLIT (1) arithmetic; returns the previous mode."""
    if isinstance(mode, str):
        mode = {"exact": MODE_EXACT, "split": MODE_SPLIT}[mode]
    return load(prec).tupan_gb300_set_mode(int(mode))


def get_mode(prec="float64"):
    return load(prec).tupan_gb300_get_mode()


def set_kepler_budget(budget, prec="float64"):
    return load(prec).tupan_gb300_set_kepler_budget(int(budget))


def split_choice(kernel, ni, nj):
    L = load("float64")
    v = ctypes.c_int()
    g = ctypes.c_int()
    st = L.tupan_gb300_split_choice(KERNEL_ID[kernel], ni, nj,
                                    ctypes.byref(v), ctypes.byref(g))
    if st:
        check()
    return v.value, g.value


def split_variants():
    L = load("float64")
    out = []
    for v in range(L.tupan_gb300_split_variants()):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.tupan_gb300_split_variant_info(v, ctypes.byref(a), ctypes.byref(b),
                                         ctypes.byref(c))
        out.append({"ni_per_thread": a.value, "jsplit": b.value,
                    "threads": c.value})
    return out


def set_centred(policy=-1, shape=-1, gsplit=0, prec="float64"):
    """Centred SPLIT sweeps (Phi/Acc/AccJerk): policy -1 automatic, 0 never,
    1 always; shape below 0 / gsplit at most 0: automatic."""
    st = load(prec).tupan_gb300_set_centred(int(policy), int(shape),
                                            int(gsplit))
    if st:
        raise TupanGB300Error("bad centred config")


def set_centred_mid(reach, prec="float64"):
    """Mid-tile reach of the centred sweeps in tile radii (<= 1.25: none);
    returns the previous reach."""
    prev = load(prec).tupan_gb300_set_centred_mid(float(reach))
    if prev < 0:
        raise TupanGB300Error("bad mid-tile reach %r" % (reach,))
    return prev


def sweep_plan(kernel, ni, nj):
    """(path, config, gsplit) of a SPLIT sweep: path 1 = centred (config =
    launch shape), 0 = split variants (config = variant)."""
    L = load("float64")
    p, c, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    st = L.tupan_gb300_sweep_plan(KERNEL_ID[kernel], int(ni), int(nj),
                                  ctypes.byref(p), ctypes.byref(c),
                                  ctypes.byref(g))
    if st:
        check()
    return p.value, c.value, g.value


def set_pipe_spin_limit(limit, prec="float64"):
    """Tries of each main-loop copy-barrier wait before DERR_PIPE_TIMEOUT
    (default 2**20); returns the previous limit."""
    return load(prec).tupan_gb300_set_pipe_spin_limit(int(limit))


def set_split_config(kernel, variant, gsplit=1):
    st = load("float64").tupan_gb300_set_split_config(
        KERNEL_ID[kernel], int(variant), int(gsplit))
    if st:
        raise TupanGB300Error("bad split config")


def set_tuned(kernel, ni, nj, variant, gsplit):
    st = load("float64").tupan_gb300_set_tuned(
        KERNEL_ID[kernel], int(ni), int(nj), int(variant), int(gsplit))
    if st:
        raise TupanGB300Error("bad tuned config")


def bind(name, prec="float64"):
    """The libtupan.h entry point ``name`` with its argtypes set."""
    return abi.bind(load(prec), name, prec)


def dev_sweep(kernel, ni, i_ptrs, nj, j_ptrs, out_ptrs, scal=(), iscal=0,
              mode=-1, stream=None, sync=False, prec="float64"):
    """One sweep over device arrays given as integer device addresses."""
    L = load(prec)
    k = KERNEL_ID[kernel]
    VP = ctypes.c_void_p
    ia = (VP * len(i_ptrs))(*i_ptrs)
    ja = (VP * len(j_ptrs))(*j_ptrs) if j_ptrs is not None else None
    oa = (VP * len(out_ptrs))(*out_ptrs)
    sc = (ctypes.c_double * 8)(*(list(scal) + [0.0] * (8 - len(scal))))
    st = L.tupan_gb300_dev_sweep(k, int(mode), int(ni), ia, int(nj), ja, sc,
                                 int(iscal), oa, stream, 1 if sync else 0)
    if st:
        check(prec)
    return st
