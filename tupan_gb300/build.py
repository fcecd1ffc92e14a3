"""Build the CUDA libraries in-tree with nvcc for sm_103a (GB300).

Produces ``tupan_gb300/libtupan_gb300.so`` (float64 ABI) and
``tupan_gb300/libtupan_gb300_sp.so`` (float32 ABI).  Object files go to
``tupan_gb300/_build``.  Translation units compile in parallel; the exact-
mode kernels are compiled with ``-fmad=false`` so that a*b+c is rounded twice
like the reference C.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17",
                 "-Xcompiler", "-fPIC,-fvisibility=hidden,-O2",
                 "-Xptxas", "-warn-spills"]

LIB64 = os.path.join(HERE, "libtupan_gb300.so")
LIB32 = os.path.join(HERE, "libtupan_gb300_sp.so")

# object -> (source, extra flags)
UNITS = {
    "exact.o": ("exact.cu", ["-fmad=false"]),
    "split.o": ("split.cu", []),
    "csweep.o": ("csweep.cu", []),
    "abi64.o": ("abi.cu", ["-DTG_ABI_FLOAT64"]),
    "abi32.o": ("abi.cu", ["-DTG_ABI_FLOAT32"]),
    "microbench.o": ("microbench.cu", []),
    "driver.o": ("driver.cu", ["-fmad=false"]),
    "blockstep.o": ("blockstep.cu", ["-fmad=false"]),
    "sakura.o": ("sakura.cu", ["-fmad=false"]),
    "mlp.o": ("mlp.cu", []),
    "ensemble.o": ("ensemble.cu", ["-fmad=false"]),
    "noalloc.o": ("noalloc.cu", []),
    "sia.o": ("sia.cu", ["-fmad=false"]),
    "nreg.o": ("nreg.cu", ["-fmad=false"]),
}
LINKS = {
    LIB64: ["exact.o", "split.o", "csweep.o", "abi64.o", "microbench.o", "driver.o",
            "blockstep.o", "sakura.o", "mlp.o", "ensemble.o",
            "noalloc.o", "sia.o", "nreg.o"],
    LIB32: ["exact.o", "split.o", "csweep.o", "abi32.o", "microbench.o"],
}


def nvcc():
    cand = [os.environ.get("NVCC"),
            os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                         "bin", "nvcc"),
            shutil.which("nvcc")]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found (set NVCC or CUDA_HOME)")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cuh")]


def build(force=False, verbose=False, jobs=4):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    todo = []
    for obj, (src, extra) in UNITS.items():
        o = os.path.join(OUT, obj)
        s = os.path.join(SRC, src)
        if force or _stale(o, [s, __file__] + hdrs):
            todo.append([cc] + COMMON + extra + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for cmd, r in ex.map(run, todo):
            if r.returncode != 0:
                sys.stderr.write(r.stdout)
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
            if verbose and r.stdout.strip():
                print(r.stdout)
    for lib, objs in LINKS.items():
        deps = [os.path.join(OUT, o) for o in objs]
        if force or _stale(lib, deps):
            cmd = [cc] + ARCH + ["-shared", "-o", lib] + deps
            r = subprocess.run(cmd, stdout=subprocess.PIPE,
                               stderr=subprocess.STDOUT, text=True)
            if r.returncode != 0:
                sys.stderr.write(r.stdout)
                raise RuntimeError("link failed: " + " ".join(cmd))
    return LIB64, LIB32


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
