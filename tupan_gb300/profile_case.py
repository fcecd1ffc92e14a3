"""Run one pairwise sweep of a given size on device-resident data, for
profiling (ncu) and timing: ``python -m tupan_gb300.profile_case --kernel
acc_jerk_kernel --ni 77824 --nj 4194304 --mode split --reps 2``.

Particles are a seeded Plummer sphere of nj bodies (the first ni are the
i-particles).  Each repetition launches the library's sweep once; the time
of each is printed with CUDA events.
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
    a = ap.parse_args(argv)

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
    v, g = lib.split_choice(a.kernel, a.ni, a.nj)
    best = min(times)
    print(json.dumps({"kernel": a.kernel, "mode": a.mode, "ni": a.ni,
                      "nj": a.nj, "times_s": times,
                      "gint_s": a.ni * a.nj / best / 1e9,
                      "variant": v, "gsplit": g}))


if __name__ == "__main__":
    main()
