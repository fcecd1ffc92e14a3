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

On a host where tupan's C backend cannot be built (no cffi or no C
compiler), importing ``tupan.lib.extensions`` fails, because it builds its
ten singletons on the C backend at import (extensions.py:654-666).
``install(before_import=True)``, called before anything imports tupan's
extensions, registers this library's kernel class as tupan's C kernel class
(the module ``tupan.lib.cffi_backend``, which ``get_kernel`` imports for the
"C" backend, extensions.py:65-66), so that the import builds the singletons
on the GPU and never compiles C.
"""

import sys
import types

from . import lib
from .backend import CUDAKernel


def _register_kernel_module():
    """Stand in for tupan.lib.cffi_backend: its CKernel is CUDAKernel."""
    import tupan.lib  # noqa: F401  (the package, not its extensions)
    name = "tupan.lib.cffi_backend"
    if name in sys.modules:
        raise RuntimeError("tupan's C backend is already imported; call "
                           "install(before_import=True) before importing "
                           "tupan.lib.extensions")
    mod = types.ModuleType(name)
    mod.CKernel = CUDAKernel
    mod.__doc__ = ("tupan_gb300: tupan's C kernel class routed to the CUDA "
                   "library")
    sys.modules[name] = mod
    sys.modules["tupan.lib"].cffi_backend = mod

SINGLETONS = (("phi", "Phi"), ("acc", "Acc"), ("acc_jerk", "AccJerk"),
              ("snap_crackle", "SnapCrackle"), ("tstep", "Tstep"),
              ("pnacc", "PNAcc"), ("sakura", "Sakura"), ("nreg_x", "NREG_X"),
              ("nreg_v", "NREG_V"), ("kepler", "Kepler"))


def install(mode=None, extensions=None, before_import=False):
    """Route tupan's kernel singletons to the CUDA library.

    ``mode``: None keeps the library mode (EXACT unless TUPAN_GB300_MODE
    says otherwise), "exact" or "split".  ``extensions``: the tupan
    extensions module (imported if omitted).  ``before_import``: tupan's
    extensions are not imported yet and its C backend is not to be built
    (see the module docstring).  Returns the extensions module.
    """
    if before_import and extensions is None and \
            "tupan.lib.extensions" not in sys.modules:
        _register_kernel_module()
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
