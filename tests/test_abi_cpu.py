"""Host-side checks that need no GPU: the libraries load and export every
symbol the public header declares; the ABI tables agree with the header;
the Python facade behaves like tupan's (tupan/lib/extensions.py)."""

import ctypes
import os
import re

import numpy as np
import pytest

from tupan_gb300 import abi, backend, extensions, lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tupan_gb300.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
    skip = {"if", "defined"}
    return sorted({n for n in names if n not in skip})


@pytest.fixture(scope="module")
def built():
    for prec in ("float64", "float32"):
        if not os.path.exists(lib.library_path(prec)):
            from tupan_gb300 import build
            build.build()
    return True


def float64_only():
    """Header functions the float32 library does not export: the sections
    marked 'libtupan_gb300.so only' (device drivers, Sakura/Kepler queue,
    learned-start training, ensembles) and the no-alloc sweep."""
    prefixes = ("tupan_gb300_hermite_", "tupan_gb300_block_",
                "tupan_gb300_sakura_", "tupan_gb300_kepler_",
                "tupan_gb300_mlp_", "tupan_gb300_ensemble_",
                "tupan_gb300_sia_", "tupan_gb300_nreg_")
    return {n for n in header_functions()
            if n.startswith(prefixes) or n.endswith("_noalloc")}


def test_float64_library_exports_nothing_undeclared(built):
    """Every tupan_gb300_* function the float64 library exports is declared
    in the header."""
    import subprocess
    path = lib.library_path("float64")
    try:
        out = subprocess.run(["nm", "-D", "--defined-only", path],
                             capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("nm not available")
    exported = {ln.split()[-1] for ln in out.splitlines()
                if len(ln.split()) == 3 and ln.split()[1] == "T"}
    ours = {n for n in exported if n.startswith("tupan_gb300_")}
    extra = sorted(ours - set(header_functions()))
    assert not extra, extra


@pytest.mark.parametrize("prec", ["float64", "float32"])
def test_library_exports_every_header_symbol(built, prec):
    L = ctypes.CDLL(lib.library_path(prec))
    skip = float64_only() if prec == "float32" else set()
    missing = [n for n in header_functions()
               if n not in skip and not hasattr(L, n)]
    assert not missing, missing


def test_header_declares_all_reference_kernels():
    names = header_functions()
    for k in abi.KERNEL_NAMES:
        assert k in names


def test_header_argument_counts_match_abi_table():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for name, sig in abi.SIGNATURES.items():
        m = re.search(r"\b%s\s*\((.*?)\);" % name, text, flags=re.S)
        assert m, name
        nargs = len([a for a in m.group(1).split(",") if a.strip()])
        assert nargs == len(sig), (name, nargs, len(sig))


@pytest.mark.parametrize("prec", ["float64", "float32"])
def test_precision_of_library(built, prec):
    L = lib.load(prec)
    assert L.tupan_gb300_real_bits() == (64 if prec == "float64" else 32)


def test_mode_switch_without_device(built):
    old = lib.set_mode("split")
    assert lib.get_mode() == lib.MODE_SPLIT
    lib.set_mode(old)
    # float32 library has no SPLIT mode: the request is ignored
    L = lib.load("float32")
    prev = L.tupan_gb300_set_mode(1)
    assert L.tupan_gb300_get_mode() == 0
    L.tupan_gb300_set_mode(prev)


def test_kernel_arity_table(built):
    L = lib.load("float64")
    for name, k in lib.KERNEL_ID.items():
        a, b = ctypes.c_int(), ctypes.c_int()
        assert L.tupan_gb300_kernel_arity(k, ctypes.byref(a), ctypes.byref(b)) == 0
        sig = abi.SIGNATURES[name]
        n_in = len([1 for (kind, arg) in sig if kind == "in" and arg[0] == "i"])
        n_out = len([1 for (kind, _) in sig if kind == "out"])
        assert (a.value, b.value) == (n_in, n_out), name


def test_get_kernel_rejects_unknown_backend():
    # tupan/lib/extensions.py:69-71 raises ValueError on a bad backend
    with pytest.raises(ValueError):
        extensions.get_kernel("acc_kernel", "OpenGL", "float64")


def test_cty_converters_refuse_wrong_arrays(built):
    k = backend.CUDAKernel("float64", "acc_kernel")
    with pytest.raises(TypeError):
        k.cty.c_real_p(np.zeros(4, dtype=np.float32))
    with pytest.raises(ValueError):
        k.cty.c_real_p(np.zeros((4, 2))[:, 0])
    p = k.cty.c_real_p(np.zeros(4))
    assert isinstance(p, ctypes.POINTER(ctypes.c_double))
    assert k.cty.c_uint(5) == 5


def test_set_args_start_offset(built):
    k = backend.CUDAKernel("float64", "phi_kernel")
    k.set_args([1, 2, 3])
    k.set_args([9], start=1)
    assert k.args == [1, 9, 3]


def test_error_status_without_device(built):
    # No GPU here: a call must fail loudly through the error status, never
    # compute on the CPU.
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    n = 4
    ps = {k: np.ones(n) for k in ("m", "rx", "ry", "rz", "e2")}
    fn = lib.bind("phi_kernel")
    vals = abi.make_args("phi_kernel", "float64", ps, ps)
    vals["iphi"][:] = 12345.0
    abi.call(fn, "phi_kernel", "float64", vals)
    assert lib.load().tupan_gb300_last_error() != 0
    with pytest.raises(lib.TupanGB300Error):
        lib.check()
    assert np.all(vals["iphi"] == 12345.0)
