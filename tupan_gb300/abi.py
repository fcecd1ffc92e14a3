"""Argument tables of the tupan kernel ABI.

Each entry lists the arguments of one C entry point in call order, exactly as
tupan declares them in ``tupan/lib/src/libtupan.h:2-246`` and marshals them in
``tupan/lib/extensions.py`` (``Phi.set_args`` :118-137 ... ``Kepler.set_args``
:638-651).  Kinds:

``uint``  particle count (``UINT``: uint64 for float64, uint32 for float32)
``int``   integer scalar (``INT``)
``real``  floating scalar (``REAL``)
``in``    ``const REAL *`` particle attribute
``out``   ``REAL *`` result array, overwritten completely

The same table drives the ctypes bindings of the CUDA library, of the CPU
oracle and of the reference build, so the three are called identically.
"""

import ctypes
from collections import OrderedDict

import numpy as np

_POS = ("rx", "ry", "rz")
_VEL = ("vx", "vy", "vz")
_ACC = ("ax", "ay", "az")
_JRK = ("jx", "jy", "jz")


def _side(prefix, attrs):
    return [("in", prefix + a) for a in attrs]


_MRE = ("m",) + _POS + ("e2",)
_MREV = _MRE + _VEL

SIGNATURES = OrderedDict()

SIGNATURES["phi_kernel"] = (
    [("uint", "ni")] + _side("i", _MRE) + [("uint", "nj")] + _side("j", _MRE)
    + [("out", "iphi")])

SIGNATURES["acc_kernel"] = (
    [("uint", "ni")] + _side("i", _MRE) + [("uint", "nj")] + _side("j", _MRE)
    + [("out", "iax"), ("out", "iay"), ("out", "iaz")])

SIGNATURES["acc_jerk_kernel"] = (
    [("uint", "ni")] + _side("i", _MREV) + [("uint", "nj")]
    + _side("j", _MREV)
    + [("out", n) for n in ("iax", "iay", "iaz", "ijx", "ijy", "ijz")])

SIGNATURES["snap_crackle_kernel"] = (
    [("uint", "ni")] + _side("i", _MREV + _ACC + _JRK) + [("uint", "nj")]
    + _side("j", _MREV + _ACC + _JRK)
    + [("out", n) for n in ("isx", "isy", "isz", "icx", "icy", "icz")])

SIGNATURES["tstep_kernel"] = (
    [("uint", "ni")] + _side("i", _MREV) + [("uint", "nj")]
    + _side("j", _MREV) + [("real", "eta")]
    + [("out", "idt_a"), ("out", "idt_b")])

SIGNATURES["pnacc_kernel"] = (
    [("uint", "ni")] + _side("i", _MREV) + [("uint", "nj")]
    + _side("j", _MREV) + [("uint", "order")]
    + [("real", "inv%d" % k) for k in range(1, 8)]
    + [("out", "ipnax"), ("out", "ipnay"), ("out", "ipnaz")])

SIGNATURES["nreg_Xkernel"] = (
    [("uint", "ni")] + _side("i", _MREV) + [("uint", "nj")]
    + _side("j", _MREV) + [("real", "dt")]
    + [("out", n) for n in ("idrx", "idry", "idrz", "iax", "iay", "iaz",
                            "iu")])

SIGNATURES["nreg_Vkernel"] = (
    [("uint", "ni")] + _side("i", ("m",) + _VEL + _ACC) + [("uint", "nj")]
    + _side("j", ("m",) + _VEL + _ACC) + [("real", "dt")]
    + [("out", n) for n in ("idvx", "idvy", "idvz", "ik")])

SIGNATURES["sakura_kernel"] = (
    [("uint", "ni")] + _side("i", _MREV) + [("uint", "nj")]
    + _side("j", _MREV) + [("real", "dt"), ("int", "flag")]
    + [("out", n) for n in ("idrx", "idry", "idrz", "idvx", "idvy", "idvz")])

SIGNATURES["kepler_solver_kernel"] = (
    _side("i", _MREV) + [("real", "dt")]
    + [("out", n) for n in ("ir1x", "ir1y", "ir1z", "iv1x", "iv1y", "iv1z")])

KERNEL_NAMES = tuple(SIGNATURES)

# Result attribute names registered on the i-particles by each extension
# (tupan/lib/extensions.py:123-132, :185-198, ..., :645-646).
OUTPUT_ATTRS = {
    "phi_kernel": ("phi",),
    "acc_kernel": ("ax", "ay", "az"),
    "acc_jerk_kernel": ("ax", "ay", "az", "jx", "jy", "jz"),
    "snap_crackle_kernel": ("sx", "sy", "sz", "cx", "cy", "cz"),
    "tstep_kernel": ("tstep", "tstepij"),
    "pnacc_kernel": ("pnax", "pnay", "pnaz"),
    "nreg_Xkernel": ("mrx", "mry", "mrz", "ax", "ay", "az", "u"),
    "nreg_Vkernel": ("mvx", "mvy", "mvz", "mk"),
    "sakura_kernel": ("drx", "dry", "drz", "dvx", "dvy", "dvz"),
    "kepler_solver_kernel": ("rx", "ry", "rz", "vx", "vy", "vz"),
}


def ctypes_for(prec):
    """(uint, int, real) ctypes for a precision name, as
    ``tupan/lib/cffi_backend.py:35-36`` and ``tupan/lib/utils/ctype.py:16-18``.
    """
    if prec == "float64":
        return ctypes.c_uint64, ctypes.c_int64, ctypes.c_double
    if prec == "float32":
        return ctypes.c_uint32, ctypes.c_int32, ctypes.c_float
    raise ValueError("unsupported precision: %r" % (prec,))


def numpy_real(prec):
    return np.dtype(np.float64) if prec == "float64" else np.dtype(np.float32)


def argtypes(name, prec):
    cu, ci, cr = ctypes_for(prec)
    rp = ctypes.POINTER(cr)
    kinds = {"uint": cu, "int": ci, "real": cr, "in": rp, "out": rp}
    return [kinds[k] for (k, _) in SIGNATURES[name]]


def bind(cdll, name, prec, symbol=None):
    """Return the ctypes function for ``name`` with argtypes set."""
    fn = getattr(cdll, symbol or name)
    fn.argtypes = argtypes(name, prec)
    fn.restype = None
    return fn


def as_real_pointer(arr, prec):
    """Pointer to a contiguous REAL array; refuses silent copies."""
    dt = numpy_real(prec)
    if not isinstance(arr, np.ndarray):
        raise TypeError("expected a numpy array, got %r" % type(arr))
    if arr.dtype != dt:
        raise TypeError("expected dtype %s, got %s" % (dt, arr.dtype))
    if not arr.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    _, _, cr = ctypes_for(prec)
    return arr.ctypes.data_as(ctypes.POINTER(cr))


def call(fn, name, prec, values):
    """Call a bound entry point with a dict ``values`` keyed by the table's
    argument names.  Arrays are passed by pointer; scalars by value."""
    cu, ci, cr = ctypes_for(prec)
    args = []
    for kind, arg in SIGNATURES[name]:
        v = values[arg]
        if kind in ("in", "out"):
            args.append(as_real_pointer(v, prec))
        elif kind == "uint":
            args.append(cu(int(v)))
        elif kind == "int":
            args.append(ci(int(v)))
        else:
            args.append(cr(float(v)))
    fn(*args)


def make_args(name, prec, ips, jps=None, scalars=None, out=None):
    """Build the argument dict from two attribute dicts.

    ``ips``/``jps`` map attribute names (m, rx, ..., jz) to arrays; ``out``
    optionally gives preallocated outputs keyed by output argument names.
    """
    jps = ips if jps is None else jps
    scalars = scalars or {}
    dt = numpy_real(prec)
    vals = {}
    ni = len(ips["m"])
    nj = len(jps["m"])
    for kind, arg in SIGNATURES[name]:
        if kind == "uint" and arg in ("ni", "nj"):
            vals[arg] = ni if arg == "ni" else nj
        elif kind == "in":
            side = ips if arg[0] == "i" else jps
            vals[arg] = side[arg[1:]]
        elif kind == "out":
            if out is not None and arg in out:
                vals[arg] = out[arg]
            else:
                n = 2 if name == "kepler_solver_kernel" else ni
                vals[arg] = np.zeros(n, dtype=dt)
        else:
            vals[arg] = scalars[arg]
    return vals


def outputs(name, vals):
    return tuple(vals[arg] for (kind, arg) in SIGNATURES[name]
                 if kind == "out")
