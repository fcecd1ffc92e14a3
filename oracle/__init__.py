"""CPU oracle for the tupan kernel layer -- TEST INFRASTRUCTURE ONLY.

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  The product library never links or
calls it, and it is never the thing being measured except as the CPU
baseline.

Two checkers live here:

* ``liboracle.so`` / ``liboracle_sp.so`` -- a plain-C restatement
  (``oracle.c``) of the reference kernels, built with ``make -C oracle``.
  It is pinned against the reference's own outputs by the golden fixtures in
  ``tests/golden`` and, where the reference sources are present, against the
  reference compiled directly from them (``_ref/``, ``make -C oracle ref``).
* ``_ref/libtupan_ref{,_sp}.so`` -- the reference kernels themselves,
  compiled from their own source files.  Only present where those sources
  exist.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

from tupan_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
_LOCK = threading.Lock()
_LIBS = {}


def reference_root():
    """The reference tree: $TUPAN_REFERENCE, else the one the recipe
    (oracle/Makefile) names.  None when it is not present."""
    root = os.environ.get("TUPAN_REFERENCE")
    if not root:
        try:
            root = subprocess.run(["make", "-s", "-C", HERE, "print-reference"],
                                  stdout=subprocess.PIPE,
                                  stderr=subprocess.DEVNULL, text=True,
                                  check=True).stdout.strip()
        except (OSError, subprocess.CalledProcessError):
            return None
    return root if root and os.path.isdir(os.path.join(root, "tupan")) \
        else None


def build(ref=False):
    """Compile the oracle (and, if asked and available, the reference)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if ref:
        root = reference_root()
        if root:
            subprocess.check_call(["make", "-s", "-C", HERE, "ref",
                                   "TUPAN_REFERENCE=" + root])


def _load(path):
    with _LOCK:
        if path not in _LIBS:
            _LIBS[path] = ctypes.CDLL(path)
        return _LIBS[path]


def lib(prec="float64"):
    name = "liboracle.so" if prec == "float64" else "liboracle_sp.so"
    path = os.path.join(HERE, name)
    if not os.path.exists(path):
        build()
    return _load(path)


def ref_available(prec="float64"):
    name = "libtupan_ref.so" if prec == "float64" else "libtupan_ref_sp.so"
    return os.path.exists(os.path.join(HERE, "_ref", name))


def ref_lib(prec="float64"):
    name = "libtupan_ref.so" if prec == "float64" else "libtupan_ref_sp.so"
    return _load(os.path.join(HERE, "_ref", name))


def _symbol(name, prec):
    return ("oracle_" if prec == "float64" else "oracle_sp_") + name


def set_threads(n, prec="float64"):
    sym = "oracle_set_threads" if prec == "float64" else "oracle_sp_set_threads"
    getattr(lib(prec), sym)(ctypes.c_int(int(n)))


def max_threads(prec="float64"):
    sym = "oracle_max_threads" if prec == "float64" else "oracle_sp_max_threads"
    fn = getattr(lib(prec), sym)
    fn.restype = ctypes.c_int
    return int(fn())


def run(name, ips, jps=None, scalars=None, prec="float64", out=None):
    """Run oracle kernel ``name`` on attribute dicts; returns the outputs."""
    fn = abi.bind(lib(prec), name, prec, symbol=_symbol(name, prec))
    vals = abi.make_args(name, prec, ips, jps, scalars, out)
    abi.call(fn, name, prec, vals)
    return abi.outputs(name, vals)


def run_ref(name, ips, jps=None, scalars=None, prec="float64", out=None):
    """Run the reference kernel compiled from its own sources."""
    fn = abi.bind(ref_lib(prec), name, prec)
    vals = abi.make_args(name, prec, ips, jps, scalars, out)
    abi.call(fn, name, prec, vals)
    return abi.outputs(name, vals)


def kepler_pairs(dt, m, e2, states):
    """Full universal-Kepler solve (with the reference's retry and energy
    check) of n independent pairs.  ``states``: (n, 6) relative r, v.
    Returns (new states, Laguerre iterations, single-step solves)."""
    L = lib("float64")
    fn = L.oracle_kepler_pairs
    dp = ctypes.POINTER(ctypes.c_double)
    lp = ctypes.POINTER(ctypes.c_long)
    fn.argtypes = [ctypes.c_long, ctypes.c_double, dp, dp, dp, dp, lp, lp]
    n = len(m)
    m = np.ascontiguousarray(m, dtype=np.float64)
    e2 = np.ascontiguousarray(e2, dtype=np.float64)
    st = np.ascontiguousarray(states, dtype=np.float64).reshape(n, 6)
    out = np.empty_like(st)
    it = np.zeros(n, dtype=np.int64)
    so = np.zeros(n, dtype=np.int64)
    fn(n, dt, m.ctypes.data_as(dp), e2.ctypes.data_as(dp),
       st.ctypes.data_as(dp), out.ctypes.data_as(dp),
       it.ctypes.data_as(lp), so.ctypes.data_as(lp))
    return out, it, so


def kepler_root(dt, m, e2, states, s_start=None):
    """One Laguerre solve per pair from ``s_start`` (NaN: plain guess).
    Returns (status, iterations, root, plain guess)."""
    L = lib("float64")
    fn = L.oracle_kepler_root
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    fn.argtypes = [ctypes.c_long, ctypes.c_double, dp, dp, dp, dp, dp, dp,
                   ip, ip]
    n = len(m)
    m = np.ascontiguousarray(m, dtype=np.float64)
    e2 = np.ascontiguousarray(e2, dtype=np.float64)
    st = np.ascontiguousarray(states, dtype=np.float64).reshape(n, 6)
    root = np.empty(n)
    plain = np.empty(n)
    status = np.zeros(n, dtype=np.int32)
    iters = np.zeros(n, dtype=np.int32)
    sp = None
    if s_start is not None:
        s_start = np.ascontiguousarray(s_start, dtype=np.float64)
        sp = s_start.ctypes.data_as(dp)
    fn(n, dt, m.ctypes.data_as(dp), e2.ctypes.data_as(dp),
       st.ctypes.data_as(dp), sp, root.ctypes.data_as(dp),
       plain.ctypes.data_as(dp), status.ctypes.data_as(ip),
       iters.ctypes.data_as(ip))
    return status, iters, root, plain
