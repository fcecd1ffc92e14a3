"""Run one pairwise sweep of a given size on device-resident data, for
profiling (ncu) and timing: ``python -m tupan_gb300.profile_case --kernel
acc_jerk_kernel --ni 77824 --nj 4194304 --mode split --reps 2``.

Particles are a seeded Plummer sphere of nj bodies (the first ni are the
i-particles).  Each repetition launches the library's sweep once; the time
of each is printed with CUDA events.

``--kernel hermite_step --nj N --order 4`` instead creates the device
Hermite driver on N particles and takes `--reps` adaptive shared steps
(each: Tstep sweep, state copy, forces, predictor, two forces + corrector
passes), so the fp64 predictor and corrector can be profiled at sizes whose
arrays exceed L2.
"""

import argparse
import json

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", default="acc_jerk_kernel")
    ap.add_argument("--ni", type=int, default=77824)
    ap.add_argument("--nj", type=int, default=4194304)
    ap.add_argument("--mode", default="split", choices=["split", "exact"])
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--variant", type=int, default=-1)
    ap.add_argument("--gsplit", type=int, default=0)
    ap.add_argument("--order", type=int, default=4)
    ap.add_argument("--path", default="auto",
                    choices=["auto", "centred", "split"],
                    help="SPLIT sweeps: the automatic choice, the centred "
                         "kernels or the double-single split variants")
    a = ap.parse_args(argv)

    if a.kernel == "hermite_step":
        return hermite_steps(a)

    import torch
    from . import abi, ics, lib

    dev = torch.device("cuda", 0)
    ps = ics.plummer(a.nj, eps=1e-4, seed=3)
    names = [arg[1:] for (kind, arg) in abi.SIGNATURES[a.kernel]
             if kind == "in" and arg[0] == "i"]
    d = {k: torch.from_numpy(np.ascontiguousarray(ps[k])).to(dev)
         for k in names}
    nout = len([1 for (kind, _) in abi.SIGNATURES[a.kernel] if kind == "out"])
    outs = [torch.empty(a.ni, dtype=torch.float64, device=dev)
            for _ in range(nout)]
    ptr = [d[k].data_ptr() for k in names]
    mode = lib.MODE_SPLIT if a.mode == "split" else lib.MODE_EXACT
    if a.variant >= 0:
        lib.set_split_config(a.kernel, a.variant, max(1, a.gsplit))
    lib.set_centred({"auto": -1, "centred": 1, "split": 0}[a.path], -1,
                    a.gsplit if a.path == "centred" else 0)
    scal = [1.0 / 64] if a.kernel in ("tstep_kernel", "nreg_Xkernel",
                                      "nreg_Vkernel") else []
    st = torch.cuda.Stream(dev)
    times = []
    with torch.cuda.stream(st):
        for _ in range(a.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            lib.dev_sweep(a.kernel, a.ni, ptr, a.nj, ptr,
                          [o.data_ptr() for o in outs], scal=scal, mode=mode,
                          stream=st.cuda_stream)
            e1.record(st)
            st.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    lib.check()
    path, cfg, g = lib.sweep_plan(a.kernel, a.ni, a.nj)
    lib.set_centred(-1, -1, 0)
    best = min(times)
    print(json.dumps({"kernel": a.kernel, "mode": a.mode, "ni": a.ni,
                      "nj": a.nj, "times_s": times,
                      "gint_s": a.ni * a.nj / best / 1e9,
                      "path": "centred" if path == 1 else "split",
                      "config": cfg, "gsplit": g}))


def hermite_steps(a):
    import time
    from . import ics
    from .integrator import DeviceHermite
    ps = ics.plummer(a.nj, eps=1e-4, seed=3)
    h = DeviceHermite(ps, 1.0 / 64, order=a.order, adaptive=True,
                      mode=a.mode)
    times = []
    for k in range(a.reps):
        t0 = time.perf_counter()
        h.evolve(1.0, max_steps=1, batch=1)
        times.append(time.perf_counter() - t0)
    h.close()
    print(json.dumps({"kernel": "hermite_step", "mode": a.mode,
                      "n": a.nj, "order": a.order, "steps": a.reps,
                      "times_s": times}))


if __name__ == "__main__":
    main()
