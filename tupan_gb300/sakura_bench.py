"""Time one Sakura sweep of a Salpeter Plummer sphere (eps = 0) on the GPU:
the EXACT in-order kernel, the queued Kepler path, plain and learned start.

    python -m tupan_gb300.sakura_bench --n 4096 --dt 0.001953125 --reps 5
    python -m tupan_gb300.sakura_bench --integrate --tau 0.00390625 --t-end 0.25

Prints one JSON line: pair evaluations per second of each path, the number
of Kepler-branch solves per sweep, Kepler solves per second of the queue's
solve kernel alone (plain and learned start) and the Laguerre iteration
histograms.
"""

import argparse
import json
import os

import numpy as np


def integrate(a):
    """The Sakura integrator on the device (N = a.n Salpeter Plummer sphere,
    eps = 0, fixed step tau to t_end): EXACT sweeps with the plain Kepler
    start, EXACT with the learned start, and SPLIT sweeps.  Wall time,
    Kepler solves and their rate, mean Laguerre updates, and the largest
    difference of each final state from the first, relative to the
    coordinate scale."""
    import time
    import torch
    from . import ics, learned
    from .kepler import DeviceSakura
    ps = ics.plummer(a.n, eps=0.0, seed=11, masses="salpeter")
    res = {"n": a.n, "tau": a.tau, "t_end": a.t_end}
    finals = {}
    net = learned.LearnedStart.load(a.weights or learned.WEIGHTS)
    runs = (("plain", False, "exact"), ("learned", True, "exact"),
            ("split", False, "split"))
    for label, use, mode in runs:
        if use:
            net.install()
        else:
            from .kepler import clear_mlp
            clear_mlp()
        d = DeviceSakura(ps, mode=mode)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t, steps, nk = d.evolve(a.tau, a.t_end, use_mlp=use)
        wall = time.perf_counter() - t0
        h = d.hist.copy()
        finals[label] = d.state()
        d.close()
        res[label] = {"steps": int(steps), "wall_s": wall,
                      "kepler_solves": int(nk),
                      "kepler_solves_per_s": nk / wall,
                      "mean_updates": float((np.arange(65) * h).sum() /
                                            max(h.sum(), 1))}
    from .kepler import clear_mlp
    clear_mlp()
    for other in ("learned", "split"):
        diff = 0.0
        for c in ("rx", "ry", "rz", "vx", "vy", "vz"):
            scale = np.abs(finals["plain"][c]).max()
            diff = max(diff, float(np.abs(finals["plain"][c] -
                                          finals[other][c]).max() / scale))
        res["max_state_diff_over_scale_" + other] = diff
    res["split_over_plain_wall"] = (res["plain"]["wall_s"] /
                                    res["split"]["wall_s"])
    res["learned_over_plain_wall"] = (res["plain"]["wall_s"] /
                                      res["learned"]["wall_s"])
    print(json.dumps(res))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--integrate", action="store_true",
                    help="run the Sakura integrator (plain and learned)")
    ap.add_argument("--tau", type=float, default=1.0 / 256)
    ap.add_argument("--t-end", type=float, default=0.25)
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--dt", type=float, default=1.0 / 512)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--weights", default=None)
    a = ap.parse_args(argv)
    if a.integrate:
        return integrate(a)

    import torch
    from . import ics, lib, learned
    from . import kepler as kp

    n = a.n
    ps = ics.plummer(n, eps=0.0, seed=11, masses="salpeter")
    names = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")
    d = {k: torch.from_numpy(np.ascontiguousarray(ps[k])).cuda() for k in names}
    ptr = [d[k].data_ptr() for k in names]
    out = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(6)]
    optr = [o.data_ptr() for o in out]
    res = {"n": n, "dt": a.dt}

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(a.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return min(ts)

    t_exact = timed(lambda: lib.dev_sweep(
        "sakura_kernel", n, ptr, n, ptr, optr, scal=[a.dt], iscal=-1,
        mode=lib.MODE_EXACT, sync=True))
    res["exact_pairs_per_s"] = n * n / t_exact
    nk, hist = kp.sakura_queue(n, ptr, n, ptr, optr, a.dt, -1,
                               histogram=True)
    t_queue = timed(lambda: kp.sakura_queue(n, ptr, n, ptr, optr, a.dt, -1))
    res["queue_pairs_per_s"] = n * n / t_queue
    t_split = timed(lambda: kp.sakura_queue(n, ptr, n, ptr, optr, a.dt, -1,
                                            mode="split"))
    res["queue_split_pairs_per_s"] = n * n / t_split
    res["kepler_pairs"] = int(nk)
    res["hist_plain"] = hist[:12].tolist()
    res["mean_iters_plain"] = float((np.arange(65) * hist).sum() / max(nk, 1))

    # the solve kernel alone on the same pairs (plain and learned start)
    st, m, e2 = learned.kepler_pair_states(n, 11, a.dt, flag=-1)
    npair = len(m)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    sm, se, ss = T(m), T(e2), T(st)
    o = torch.zeros((npair, 6), dtype=torch.float64, device="cuda")
    it = torch.zeros(npair, dtype=torch.int32, device="cuda")
    t_plain = timed(lambda: kp.kepler_pairs(npair, a.dt, sm, se, ss, o,
                                            iters=it))
    res["kepler_solves_per_s_plain"] = npair / t_plain
    res["mean_iters_pairs_plain"] = float(it.float().mean().item())
    w = a.weights or learned.WEIGHTS
    if os.path.exists(w):
        net = learned.LearnedStart.load(w)
        net.install()
        t_learn = timed(lambda: kp.kepler_pairs(npair, a.dt, sm, se, ss, o,
                                                iters=it, use_mlp=True))
        res["kepler_solves_per_s_learned"] = npair / t_learn
        res["mean_iters_pairs_learned"] = float(it.float().mean().item())
        res["learned_speedup"] = t_plain / t_learn
        kp.clear_mlp()
    print(json.dumps(res))


if __name__ == "__main__":
    main()
