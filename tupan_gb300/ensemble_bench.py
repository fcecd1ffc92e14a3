"""Config-4 shape on the GPU: an ensemble of independent Plummer systems with
N uniform in [3, 512] (seeded), equal masses, eps = 1e-4, Hermite-4 shared
adaptive steps (eta = 1/64), SPLIT forces, advanced together.

    python -m tupan_gb300.ensemble_bench --systems 4096 --t-end 0.0625

Prints one JSON line: systems per second (systems advanced to t_end per wall
second), the largest step count, and the distribution of per-system fp64
energy errors.
"""

import argparse
import json
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=4096)
    ap.add_argument("--t-end", type=float, default=1.0 / 16)
    ap.add_argument("--eta", type=float, default=1.0 / 64)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--mode", default="batched",
                    choices=["batched", "persistent"])
    ap.add_argument("--steps-per-launch", type=int, default=1024)
    ap.add_argument("--switch-below", type=int, default=0)
    ap.add_argument("--shape", default="",
                    help="batched sweep shape nt,ib,prefetch (default: the "
                         "library's, tuned where a table is saved)")
    ap.add_argument("--stage", type=int, default=0,
                    help="1: predictor/corrector as launches of their own; "
                         "0: inside the sweeps")
    a = ap.parse_args(argv)
    from .ensemble import DeviceEnsemble, make_systems
    t0 = time.perf_counter()
    systems = make_systems(a.systems, seed=1)
    ens = DeviceEnsemble(systems, a.eta)
    ens.set_mode(a.mode, a.steps_per_launch, a.switch_below)
    if a.shape:
        ens.set_shape(*[int(x) for x in a.shape.split(",")])
    ens.set_stage(a.stage)
    shape = ens.shape
    ke0, pe0 = ens.energies()
    t1 = time.perf_counter()
    mx = ens.evolve(a.t_end, batch=a.batch)
    t2 = time.perf_counter()
    ke1, pe1 = ens.energies()
    t, k, _ = ens.state()
    ens.close()
    de = np.abs(((ke1 + pe1) - (ke0 + pe0)) / -pe0)
    print(json.dumps({
        "systems": a.systems, "particles": int(ens.n), "t_end": a.t_end,
        "mode": a.mode, "steps_per_launch": a.steps_per_launch,
        "switch_below": a.switch_below, "shape": list(shape),
        "stage": a.stage,
        "wall_s": t2 - t1, "setup_s": t1 - t0,
        "systems_per_s": a.systems / (t2 - t1),
        "max_steps": int(mx), "mean_steps": float(k.mean()),
        "all_at_t_end": bool(np.all(t == a.t_end)),
        "dE_over_E_median": float(np.median(de)),
        "dE_over_E_p99": float(np.quantile(de, 0.99)),
        "dE_over_E_max": float(de.max())}))


if __name__ == "__main__":
    main()
