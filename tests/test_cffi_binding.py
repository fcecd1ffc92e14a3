"""The cffi binding a tupan maintainer would add: cdef the reference's own
libtupan.h (as tupan/lib/cffi_backend.py:31-87 does) with the float64 and
float32 typedefs and dlopen this library in its place.  Every one of the
ten prototypes must resolve.  Runs where the reference sources exist; no
call is made, so no GPU is needed."""

import os

import pytest

import oracle
from tupan_gb300 import lib

cffi = pytest.importorskip("cffi")

_ROOT = oracle.reference_root()
REF_H = os.path.join(_ROOT or "", "tupan", "lib", "src", "libtupan.h")
NAMES = ("phi_kernel", "acc_kernel", "acc_jerk_kernel", "snap_crackle_kernel",
         "tstep_kernel", "pnacc_kernel", "nreg_Xkernel", "nreg_Vkernel",
         "sakura_kernel", "kepler_solver_kernel")
TYPES = {"float64": "typedef int64_t INT; typedef uint64_t UINT; "
                    "typedef double REAL;\n",
         "float32": "typedef int32_t INT; typedef uint32_t UINT; "
                    "typedef float REAL;\n"}


@pytest.mark.parametrize("prec", ["float64", "float32"])
def test_reference_header_binds_to_this_library(prec):
    if not os.path.exists(REF_H):
        pytest.skip("reference sources not present")
    path = lib.library_path(prec)
    if not os.path.exists(path):
        pytest.skip("library not built")
    src = open(REF_H).read().replace("restrict", "")
    ffi = cffi.FFI()
    ffi.cdef(TYPES[prec] + src)
    L = ffi.dlopen(path)
    for name in NAMES:
        fn = getattr(L, name)
        assert ffi.typeof(fn).kind == "function", name
    ffi.cdef("int tupan_gb300_last_error(void);")
    assert L.tupan_gb300_last_error() in range(0, 16)
