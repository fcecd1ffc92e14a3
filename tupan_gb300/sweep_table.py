"""Single force-evaluation sweeps at several N: Acc and AccJerk of all i
against all j on equal-mass Plummer spheres (eps = 1e-4), SPLIT mode on the
whole sphere and the fp64 EXACT mode on an i-subset, with the SPLIT error
against the fp64 EXACT sweep (bit-identical to the reference's fp64 kernel)
on a random i-subset.

    python -m tupan_gb300.sweep_table --n 16384 65536 262144 1048576

Prints one JSON line per N: Gint/s of each sweep, the fraction of the FP32
FMA rate measured in the same run (at the reference's 20 and 42 flop per
interaction), the EXACT rate, and the max and median |da|/|a| of the SPLIT
AccJerk sweep.
"""

import argparse
import ctypes
import json

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, nargs="+",
                    default=[16384, 65536, 262144, 1048576])
    ap.add_argument("--reps", type=int, default=3)
    # EXACT i-subset: two CTAs of 128 i per SM, so the fp64 sweep fills the
    # GPU (smaller subsets leave SMs idle and understate the fp64 rate)
    ap.add_argument("--exact-ni", type=int, default=2 * 152 * 128)
    ap.add_argument("--check-ni", type=int, default=128)
    a = ap.parse_args(argv)

    import torch
    from . import ics, lib

    L = lib.load()
    L.tupan_gb300_fp32_peak_tflops.restype = ctypes.c_double
    L.tupan_gb300_fp32_peak_tflops.argtypes = [ctypes.c_int, ctypes.c_int]
    peak = float(L.tupan_gb300_fp32_peak_tflops(20000, 5))
    names = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")
    stream = torch.cuda.current_stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(a.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        return best

    for n in a.n:
        ps = ics.plummer(n, eps=1e-4, seed=n)
        d = {k: torch.from_numpy(np.ascontiguousarray(ps[k])).cuda()
             for k in names}
        p5 = [d[k].data_ptr() for k in names[:5]]
        p8 = [d[k].data_ptr() for k in names]
        acc = [torch.empty(n, dtype=torch.float64, device="cuda")
               for _ in range(3)]
        aj = [torch.empty(n, dtype=torch.float64, device="cuda")
              for _ in range(6)]

        def sweep(kernel, ni, ptrs, outs, mode):
            lib.dev_sweep(kernel, ni, ptrs, n, ptrs,
                          [t.data_ptr() for t in outs], mode=mode,
                          stream=stream.cuda_stream)

        t_acc = timed(lambda: sweep("acc_kernel", n, p5, acc, lib.MODE_SPLIT))
        t_aj = timed(lambda: sweep("acc_jerk_kernel", n, p8, aj,
                                   lib.MODE_SPLIT))
        ni = min(n, a.exact_ni)
        t_aj64 = timed(lambda: sweep("acc_jerk_kernel", ni, p8, aj,
                                     lib.MODE_EXACT))
        sweep("acc_jerk_kernel", n, p8, aj, lib.MODE_SPLIT)
        torch.cuda.synchronize()
        # reference: the fp64 EXACT sweep (bit-identical to the reference's
        # fp64 kernel) of a random i-subset against all j
        idx = np.sort(np.random.default_rng(0).choice(n, a.check_ni,
                                                      replace=False))
        d_idx = torch.from_numpy(idx).cuda()
        sub = [d[k].index_select(0, d_idx).contiguous() for k in names]
        ex = [torch.empty(len(idx), dtype=torch.float64, device="cuda")
              for _ in range(6)]
        lib.dev_sweep("acc_jerk_kernel", len(idx),
                      [t.data_ptr() for t in sub], n, p8,
                      [t.data_ptr() for t in ex], mode=lib.MODE_EXACT,
                      stream=stream.cuda_stream)
        torch.cuda.synchronize()
        want = [t.cpu().numpy() for t in ex]
        got = [t.cpu().numpy()[idx] for t in aj]
        ga, wa = np.stack(got[:3]), np.stack(want[:3])
        rel = np.linalg.norm(ga - wa, axis=0) / np.linalg.norm(wa, axis=0)
        gi_acc = n * n / t_acc / 1e9
        gi_aj = n * n / t_aj / 1e9
        path, cfg, gsp = lib.sweep_plan("acc_jerk_kernel", n, n)
        print(json.dumps({
            "n": n, "acc_gints": gi_acc, "acc_jerk_gints": gi_aj,
            "path": "centred" if path == 1 else "split variants",
            "config": cfg, "gsplit": gsp,
            "acc_frac_fp32": gi_acc * 20 / 1e3 / peak,
            "acc_jerk_frac_fp32": gi_aj * 42 / 1e3 / peak,
            "fp64_exact_acc_jerk_gints": ni * n / t_aj64 / 1e9,
            "split_over_exact": gi_aj / (ni * n / t_aj64 / 1e9),
            "acc_rel_err_max": float(rel.max()),
            "acc_rel_err_median": float(np.median(rel)),
            "check_ni": int(a.check_ni), "fp32_peak_tflops": peak}),
            flush=True)
        del d, acc, aj
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
