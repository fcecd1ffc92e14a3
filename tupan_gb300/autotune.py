"""Measured autotuning of the SPLIT sweep launch shape.

For a kernel and a size (ni, nj), ``tune`` times every compiled variant (i
per thread, lanes per i, threads per block) with a set of grid j-splits on
synthetic Plummer data, picks the fastest and records it in the library's
table for the same power-of-two size bucket (``tupan_gb300_set_tuned``).
Without an entry the library uses its occupancy model (waves x work per
CTA).  ``save``/``load`` keep the table in a JSON file next to this module,
keyed by GPU name; ``load`` runs on import of ``tupan_gb300.autotune``'s
``apply_saved`` so a tuned machine starts tuned.
"""

import json
import os

import numpy as np

from . import abi, ics, lib

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning.json")
GSPLITS = (1, 2, 4, 8, 16, 32)


def _device_name():
    import torch
    return torch.cuda.get_device_name(0)


def tune(kernel, ni, nj, reps=3, gsplits=GSPLITS, record=True):
    """Time all (variant, gsplit) candidates; returns the sorted results
    [(seconds, variant, gsplit), ...] and records the best."""
    import torch
    dev = torch.device("cuda")
    ps = ics.plummer(max(ni, nj), eps=1e-4, seed=17)
    names = [arg[1:] for (kind, arg) in abi.SIGNATURES[kernel]
             if kind == "in" and arg[0] == "i"]
    # attributes a Plummer sphere lacks (a, j for snap_crackle) are zero:
    # the timing does not depend on their values
    data = {k: torch.from_numpy(np.ascontiguousarray(
                ps[k] if k in ps else np.zeros(len(ps["m"])))).to(dev)
            for k in names}
    ip = [data[k].data_ptr() for k in names]
    nout = len([1 for (kind, _) in abi.SIGNATURES[kernel] if kind == "out"])
    outs = [torch.empty(ni, dtype=torch.float64, device=dev)
            for _ in range(nout)]
    op = [o.data_ptr() for o in outs]
    scal = [1.0 / 64] if kernel == "tstep_kernel" else []
    stream = torch.cuda.Stream(dev)
    results = []
    nv = len(lib.split_variants())
    try:
        for v in range(nv):
            for g in gsplits:
                if g > 1 and (nj + 255) // 256 < g:
                    continue
                try:
                    lib.set_split_config(kernel, v, g)
                except lib.TupanGB300Error:
                    break          # variant not compiled for this kernel
                with torch.cuda.stream(stream):
                    lib.dev_sweep(kernel, ni, ip, nj, ip, op, scal=scal,
                                  mode=lib.MODE_SPLIT,
                                  stream=stream.cuda_stream)
                    best = float("inf")
                    for _ in range(reps):
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        lib.dev_sweep(kernel, ni, ip, nj, ip, op, scal=scal,
                                      mode=lib.MODE_SPLIT,
                                      stream=stream.cuda_stream)
                        e1.record(stream)
                        stream.synchronize()
                        best = min(best, e0.elapsed_time(e1) / 1e3)
                results.append((best, v, g))
    finally:
        lib.set_split_config(kernel, -1, 0)
    results.sort()
    if record:
        _, v, g = results[0]
        lib.set_tuned(kernel, ni, nj, v, g)
    return results


def tune_sizes(kernels=("acc_kernel", "acc_jerk_kernel"),
               sizes=((262144, 262144),), reps=3):
    table = {}
    for k in kernels:
        for (ni, nj) in sizes:
            res = tune(k, ni, nj, reps=reps)
            t, v, g = res[0]
            table["%s|%d|%d" % (k, ni, nj)] = {"variant": v, "gsplit": g,
                                               "seconds": t}
    return table


def save(table, path=TABLE):
    allt = {}
    if os.path.exists(path):
        with open(path) as f:
            allt = json.load(f)
    allt.setdefault(_device_name(), {}).update(table)
    with open(path, "w") as f:
        json.dump(allt, f, indent=1, sort_keys=True)


def apply_saved(path=TABLE):
    """Record the saved entries of this GPU in the library's table."""
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        allt = json.load(f)
    entries = allt.get(_device_name(), {})
    for key, e in entries.items():
        k, ni, nj = key.split("|")
        lib.set_tuned(k, int(ni), int(nj), e["variant"], e["gsplit"])
    return len(entries)


if __name__ == "__main__":
    import sys
    t = tune_sizes()
    print(json.dumps(t))
    if "--save" in sys.argv:
        save(t)
