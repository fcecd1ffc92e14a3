"""High-level extension objects on the CUDA backend.

Mirrors ``tupan/lib/extensions.py``: ``get_kernel(name, backend, prec)``
(:63-76), the ``Clight`` holder (:30-60), one class per kernel with
``set_args(ips, jps, *args)``, ``run()``, ``get_result()`` and
``calc(ips, jps, *args)`` (:84-97), and module-level singletons (:654-666).
``ips``/``jps`` are particle sets with the attributes tupan's
``ParticleSystem`` has (``n``, ``mass``, ``eps2``, ``rx`` ... ``jz``) and
``register_auxiliary_attribute``; results are written into auxiliary
attributes of ``ips`` named as in the reference (``phi``, ``ax`` ...).

Singletons are created on first use rather than at import, so importing this
module does not need a GPU.
"""

import os
import sys

from . import abi
from .backend import CUDAKernel

__all__ = ["Phi", "Acc", "AccJerk", "SnapCrackle", "Tstep", "PNAcc",
           "Sakura", "NREG_X", "NREG_V", "Kepler", "Clight", "get_kernel",
           "clight"]

# particle attribute read for each ABI argument suffix
_ATTR = {"m": "mass", "e2": "eps2"}


class Clight(object):
    """PN order and inverse powers of the speed of light
    (tupan/lib/extensions.py:30-60)."""

    def __init__(self):
        self._pn_order = 0
        self._clight = None
        for k in range(1, 8):
            setattr(self, "inv%d" % k, 0.0)

    @property
    def pn_order(self):
        return self._pn_order

    @pn_order.setter
    def pn_order(self, value):
        self._pn_order = int(value)

    @property
    def clight(self):
        return self._clight

    @clight.setter
    def clight(self, value):
        self._clight = float(value)
        self.inv1 = 1.0 / self._clight
        self.inv2 = self.inv1 ** 2
        self.inv3 = self.inv1 ** 3
        self.inv4 = self.inv1 ** 4
        self.inv5 = self.inv1 ** 5
        self.inv6 = self.inv1 ** 6
        self.inv7 = self.inv1 ** 7


def get_kernel(name, backend, prec):
    """Kernel object for ``name``; ``backend`` must be "CUDA" here (the C and
    CL backends live in tupan itself, see tupan_gb300.shim)."""
    if backend != "CUDA":
        raise ValueError("Inappropriate 'backend': {}. Supported values: "
                         "['CUDA']".format(backend))
    return CUDAKernel(prec, name)


def prepare_args(args, argtypes):
    return [argtype(arg) for (arg, argtype) in zip(args, argtypes)]


class AbstractExtension(object):
    """Argument marshalling driven by the ABI table (tupan_gb300.abi)."""

    kernel_name = None
    scalar_names = ()

    def __init__(self, backend, prec):
        self.kernel = get_kernel(self.kernel_name, backend, prec)
        self.prec = prec
        cty = self.kernel.cty
        kinds = {"uint": cty.c_uint, "int": cty.c_int, "real": cty.c_real,
                 "in": cty.c_real_p, "out": cty.c_real_p}
        sig = abi.SIGNATURES[self.kernel_name]
        self.argtypes = tuple(kinds[k] for (k, _) in sig if k != "out")
        self.restypes = tuple(kinds[k] for (k, _) in sig if k == "out")

    def _scalars(self, args):
        return dict(zip(self.scalar_names, args))

    def set_args(self, ips, jps, *args):
        name = self.kernel_name
        self.kernel.set_gsize(ips.n, jps.n)
        outs = abi.OUTPUT_ATTRS[name]
        for attr in outs:
            if attr not in ips.__dict__:
                ips.register_auxiliary_attribute(attr, "real")
        scal = self._scalars(args)
        inargs = []
        for kind, arg in abi.SIGNATURES[name]:
            if kind == "out":
                continue
            if arg in ("ni", "nj"):
                inargs.append(ips.n if arg == "ni" else jps.n)
            elif kind == "in":
                side = ips if arg[0] == "i" else jps
                inargs.append(getattr(side, _ATTR.get(arg[1:], arg[1:])))
            else:
                inargs.append(scal[arg])
        self._inargs = tuple(inargs)
        self._outargs = tuple(getattr(ips, a) for a in outs)
        self.inargs = prepare_args(self._inargs, self.argtypes)
        self.outargs = prepare_args(self._outargs, self.restypes)
        self.kernel.set_args(self.inargs + self.outargs)

    def run(self):
        self.kernel.run()

    def get_result(self):
        return self.kernel.map_buffers(self._outargs, self.outargs)

    def calc(self, ips, jps, *args):
        self.set_args(ips, jps, *args)
        self.run()
        return self.get_result()


class Phi(AbstractExtension):
    kernel_name = "phi_kernel"


class Acc(AbstractExtension):
    kernel_name = "acc_kernel"


class AccJerk(AbstractExtension):
    kernel_name = "acc_jerk_kernel"


class SnapCrackle(AbstractExtension):
    kernel_name = "snap_crackle_kernel"


class Tstep(AbstractExtension):
    kernel_name = "tstep_kernel"
    scalar_names = ("eta",)


class PNAcc(AbstractExtension):
    kernel_name = "pnacc_kernel"

    def _scalars(self, args):
        c = clight
        d = {"order": c.pn_order}
        for k in range(1, 8):
            d["inv%d" % k] = getattr(c, "inv%d" % k)
        return d


class Sakura(AbstractExtension):
    kernel_name = "sakura_kernel"
    scalar_names = ("dt", "flag")


class NREG_X(AbstractExtension):
    kernel_name = "nreg_Xkernel"
    scalar_names = ("dt",)


class NREG_V(AbstractExtension):
    kernel_name = "nreg_Vkernel"
    scalar_names = ("dt",)


class Kepler(AbstractExtension):
    """Two-body solver writing the new state into ``ips`` in place
    (tupan/lib/extensions.py:618-651)."""
    kernel_name = "kepler_solver_kernel"
    scalar_names = ("dt",)

    def set_args(self, ips, jps, *args):
        scal = self._scalars(args)
        inargs = []
        for kind, arg in abi.SIGNATURES[self.kernel_name]:
            if kind == "in":
                inargs.append(getattr(ips, _ATTR.get(arg[1:], arg[1:])))
            elif kind == "real":
                inargs.append(scal[arg])
        self._inargs = tuple(inargs)
        self._outargs = (ips.rx, ips.ry, ips.rz, ips.vx, ips.vy, ips.vz)
        self.inargs = prepare_args(self._inargs, self.argtypes)
        self.outargs = prepare_args(self._outargs, self.restypes)
        self.kernel.set_args(self.inargs + self.outargs)


clight = Clight()

_SINGLETONS = {"phi": Phi, "acc": Acc, "acc_jerk": AccJerk,
               "snap_crackle": SnapCrackle, "tstep": Tstep, "pnacc": PNAcc,
               "sakura": Sakura, "nreg_x": NREG_X, "nreg_v": NREG_V,
               "kepler": Kepler}

backend = "CUDA"


def _prec():
    return "float32" if "--use_sp" in sys.argv else "float64"


def __getattr__(name):
    # Module singletons (extensions.py:656-666), built on first access.
    if name in _SINGLETONS:
        obj = _SINGLETONS[name](backend, _prec())
        globals()[name] = obj
        return obj
    raise AttributeError(name)
