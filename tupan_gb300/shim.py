"""Install the CUDA backend into an importable tupan.

tupan picks its backend once, at import of ``tupan.lib.extensions``
(``backend = "CL" if "--use_cl" in sys.argv else "C"``, extensions.py:654),
and builds every kernel singleton then (:656-666); ``get_kernel`` accepts
only "C" and "CL" (:63-76).  ``install()`` wraps ``get_kernel`` so that the
backend name "CUDA" resolves to ``tupan_gb300.backend.CUDAKernel`` and
rebuilds the ten singletons on it.  Integrators and particles look the
singletons up at call time (e.g. ``extensions.acc_jerk.calc`` in
particles/body.py:349-354, ``extensions.sakura.calc`` in
integrator/sakura.py:30), so everything above the kernels runs unchanged.

Call it before the first force evaluation, e.g. at the top of a driver
script or when ``--use_cuda`` is in ``sys.argv``::

    from tupan_gb300 import shim
    shim.install()               # or shim.install(mode="split")
"""

import sys

from . import lib
from .backend import CUDAKernel

SINGLETONS = (("phi", "Phi"), ("acc", "Acc"), ("acc_jerk", "AccJerk"),
              ("snap_crackle", "SnapCrackle"), ("tstep", "Tstep"),
              ("pnacc", "PNAcc"), ("sakura", "Sakura"), ("nreg_x", "NREG_X"),
              ("nreg_v", "NREG_V"), ("kepler", "Kepler"))


def install(mode=None, extensions=None):
    """Route tupan's kernel singletons to the CUDA library.

    ``mode``: None keeps the library mode (EXACT unless TUPAN_GB300_MODE
    says otherwise), "exact" or "split".  ``extensions``: the tupan
    extensions module (imported if omitted).  Returns that module.
    """
    if extensions is None:
        from tupan.lib import extensions
    ext = extensions
    if getattr(ext, "_tupan_gb300_installed", False):
        if mode is not None:
            lib.set_mode(mode)
        return ext
    original = ext.get_kernel

    def get_kernel(name, backend, prec):
        if backend == "CUDA":
            return CUDAKernel(prec, name)
        return original(name, backend, prec)

    ext.get_kernel = get_kernel
    ext.backend = "CUDA"
    from tupan.lib.utils import ctype
    for attr, cls in SINGLETONS:
        setattr(ext, attr, getattr(ext, cls)("CUDA", ctype.prec))
    ext._tupan_gb300_installed = True
    if mode is not None:
        lib.set_mode(mode)
    return ext


def install_if_requested(argv=None):
    """``install()`` when ``--use_cuda`` is on the command line, the way
    tupan reads ``--use_cl`` (extensions.py:654)."""
    argv = sys.argv if argv is None else argv
    if "--use_cuda" in argv:
        return install(mode="split" if "--cuda_split" in argv else None)
    return None
