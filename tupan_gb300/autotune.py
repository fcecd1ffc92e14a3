"""Measured autotuning of the launch shapes.

* SPLIT sweeps: for a kernel and a size (ni, nj), ``tune`` times every
  compiled variant (i per thread, lanes per i, threads per block) with a set
  of grid j-splits on synthetic Plummer data, picks the fastest and records
  it in the library's table for the same power-of-two size bucket
  (``tupan_gb300_set_tuned``).  Without an entry the library uses its
  occupancy model (waves x work per CTA).
* Block steps: ``tune_block`` runs ``tune`` for every active-set level
  (ni = 1, 2, 4, ... N against all N) of each kernel a block step sweeps;
  the captured level graphs take their sweep shapes from those entries.
* Ensembles: ``tune_ensemble`` times the batched sweep's CTA size, full
  i-block and prefetch on the ensemble workload (systems of N ~ U[3, 512])
  and sets the library's default shape.

``save`` keeps the entries in ``tuning.json`` next to this module, keyed by
GPU name; ``apply_saved`` puts this GPU's entries into the library, which
``lib.load`` does once per process (unless ``TUPAN_GB300_NO_TUNING`` is set),
so a tuned machine starts tuned.
"""

import json
import os

import numpy as np

from . import abi, ics, lib

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning.json")
GSPLITS = (1, 2, 4, 8, 16, 32)


def _device_name():
    return lib.device_name()


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
    # the variant table is what is timed: keep the centred path out
    lib.set_centred(0)
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
        lib.set_centred(-1)
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


BLOCK_KERNELS = {4: ("acc_jerk_kernel", "tstep_kernel"),
                 6: ("acc_jerk_kernel", "snap_crackle_kernel", "tstep_kernel")}


def tune_block(n=65536, order=6, reps=3, gsplits=GSPLITS):
    """Sweep shapes of the block-step levels: every kernel of a block step of
    `order` at ni = 2^L (L = 0 .. log2 N) against all n."""
    table = {}
    ni = 1
    while ni <= n:
        for k in BLOCK_KERNELS[order]:
            res = tune(k, ni, n, reps=reps, gsplits=gsplits)
            t, v, g = res[0]
            table["%s|%d|%d" % (k, ni, n)] = {"variant": v, "gsplit": g,
                                              "seconds": t}
        ni *= 2
    return table


ENSEMBLE_SHAPES = tuple((nt, ib, pf) for nt in (128, 256)
                        for ib in (64, 128, 256) for pf in (0, 1))


def tune_ensemble(systems=4096, t_end=1.0 / 64, eta=1.0 / 64,
                  shapes=ENSEMBLE_SHAPES, record=True):
    """Time an ensemble evolution (warm-up to t_end / 8, then timed to
    t_end) for every batched sweep shape; returns [(seconds, shape), ...]
    sorted, and sets the fastest as the library's default shape."""
    import time
    from .ensemble import DeviceEnsemble, make_systems, set_default_shape
    syss = make_systems(systems, seed=1)
    results = []
    for sh in shapes:
        ens = DeviceEnsemble(syss, eta)
        try:
            ens.set_shape(*sh)
            ens.evolve(t_end / 8, batch=16)
            t0 = time.perf_counter()
            ens.evolve(t_end, batch=16)
            results.append((time.perf_counter() - t0, tuple(sh)))
        finally:
            ens.close()
    results.sort()
    if record:
        set_default_shape(*results[0][1])
    return results


def ensemble_entry(results, systems):
    t, (nt, ib, pf) = results[0]
    return {"ensemble|%d" % systems: {"nt": nt, "ib": ib, "prefetch": pf,
                                      "seconds": t}}


def save(table, path=TABLE):
    allt = {}
    if os.path.exists(path):
        with open(path) as f:
            allt = json.load(f)
    allt.setdefault(_device_name(), {}).update(table)
    with open(path, "w") as f:
        json.dump(allt, f, indent=1, sort_keys=True)


def apply_saved(path=TABLE, strict=True):
    """Record the saved entries of this GPU in the library's table; returns
    how many were taken.  strict: a malformed or unusable entry raises;
    otherwise it is skipped with a warning (the library's load does this, so
    a stale table never makes the library unusable)."""
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        allt = json.load(f)
    entries = allt.get(_device_name(), {})
    ens = []
    taken = 0
    for key, e in entries.items():
        try:
            parts = key.split("|")
            if parts[0] == "ensemble":
                ens.append((int(parts[1]), e))
                continue
            k, ni, nj = parts
            lib.set_tuned(k, int(ni), int(nj), e["variant"], e["gsplit"])
            taken += 1
        except (ValueError, KeyError, lib.TupanGB300Error) as exc:
            if strict:
                raise
            import warnings
            warnings.warn("tuning entry %r skipped: %s" % (key, exc))
    if ens:
        # the entry measured on the most systems sets the default shape
        from .ensemble import set_default_shape
        e = max(ens, key=lambda x: x[0])[1]
        try:
            set_default_shape(e["nt"], e["ib"], e["prefetch"])
            taken += len(ens)
        except (KeyError, lib.TupanGB300Error) as exc:
            if strict:
                raise
            import warnings
            warnings.warn("ensemble tuning entry skipped: %s" % exc)
    return taken


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--what", default="sweep,block,ensemble")
    ap.add_argument("--n", type=int, default=65536, help="block-step N")
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--systems", type=int, default=4096)
    ap.add_argument("--save", action="store_true")
    ap.add_argument("--out", default=TABLE, help="table file for --save")
    a = ap.parse_args(argv)
    what = a.what.split(",")
    table = {}
    if "sweep" in what:
        table.update(tune_sizes())
    if "block" in what:
        table.update(tune_block(a.n, a.order))
    if "ensemble" in what:
        res = tune_ensemble(a.systems)
        print(json.dumps({"ensemble_results": [[t, list(sh)]
                                               for t, sh in res]}))
        table.update(ensemble_entry(res, a.systems))
    print(json.dumps(table, sort_keys=True))
    if a.save:
        save(table, a.out)


if __name__ == "__main__":
    main()
