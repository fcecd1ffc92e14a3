"""The CUDA backend object behind tupan's extension facade.

``CUDAKernel(prec, name)`` has the surface of tupan's ``CKernel``
(``tupan/lib/cffi_backend.py:90-126``) and ``CLKernel``
(``tupan/lib/opencl_backend.py:104-171``): ``cty`` converters, ``set_gsize``,
``set_args(args, start=0)``, ``run`` and ``map_buffers``.  Arrays are passed
to the C-ABI by pointer without copies (like the C backend); the library
stages them to the GPU, runs the sweep and writes the results back into the
output arrays before ``run`` returns, so ``map_buffers`` is the identity.
"""

import ctypes
from collections import namedtuple

import numpy as np

from . import abi, lib

Types = namedtuple("Types", ["c_int", "c_int_p", "c_uint", "c_uint_p",
                             "c_real", "c_real_p"])


class CUDAKernel(object):
    """One libtupan.h entry point of the CUDA library."""

    def __init__(self, prec, name):
        if name not in abi.SIGNATURES:
            raise ValueError("unknown kernel %r" % (name,))
        self.prec = prec
        self.name = name
        self.kernel = lib.bind(name, prec)
        cu, ci, cr = abi.ctypes_for(prec)
        real = abi.numpy_real(prec)
        ityp = np.dtype(np.int64 if prec == "float64" else np.int32)
        utyp = np.dtype(np.uint64 if prec == "float64" else np.uint32)

        def ptr(dtype, ctype):
            def conv(x):
                if not isinstance(x, np.ndarray) or x.dtype != dtype:
                    raise TypeError("%s: expected a %s numpy array"
                                    % (name, dtype))
                if not x.flags["C_CONTIGUOUS"]:
                    raise ValueError("%s: array must be C-contiguous" % name)
                return x.ctypes.data_as(ctypes.POINTER(ctype))
            return conv

        self.cty = Types(c_int=lambda x: x,
                         c_int_p=ptr(ityp, ci),
                         c_uint=lambda x: x,
                         c_uint_p=ptr(utyp, cu),
                         c_real=lambda x: x,
                         c_real_p=ptr(real, cr))
        self.args = []

    def set_gsize(self, ni, nj):
        # The library picks its own launch geometry (autotuned split sweeps).
        pass

    def allocate_local_memory(self, numbufs, sctype):
        return []

    def set_args(self, args, start=0):
        args = list(args)
        if start == 0:
            self.args = args
        else:
            self.args[start:start + len(args)] = args

    def map_buffers(self, arrays, buffers):
        return arrays

    def run(self):
        self.kernel(*self.args)
        lib.check(self.prec)
