"""Config-3 shape on the GPU: Hermite 6/8 with individual power-of-two block
steps on a Salpeter Plummer sphere (masses [0.1, 100], M = 1, eps = 1e-4,
eta = 1/32), SPLIT forces and FP64 predictor/corrector.

    python -m tupan_gb300.blockstep_bench --n 65536 --order 6 --t-end 0.0078125

Prints one JSON line: block steps, active-particle updates, force
interactions per second (each block step evaluates acc/jerk (+snap/crackle)
twice and Tstep once for the active set against all N), the distribution of
active-set sizes and the fp64 energy error.
"""

import argparse
import json
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--t-end", type=float, default=1.0 / 128)
    ap.add_argument("--eta", type=float, default=1.0 / 32)
    ap.add_argument("--dt-max", type=float, default=1.0 / 32)
    ap.add_argument("--mode", default="split")
    ap.add_argument("--launch", default="graphs", choices=["graphs", "host"])
    a = ap.parse_args(argv)

    from . import ics
    from .integrator import DeviceBlockHermite, DeviceHermite

    ps = ics.plummer(a.n, eps=1e-4, seed=3, masses="salpeter")
    e0 = DeviceHermite(ps, a.eta, order=4, adaptive=False, mode="exact")
    k0, p0 = e0.energy()
    e0.close()
    t0 = time.perf_counter()
    b = DeviceBlockHermite(ps, a.eta, a.dt_max, order=a.order, mode=a.mode,
                           graphs=a.launch == "graphs")
    t1 = time.perf_counter()
    b.evolve(a.t_end)
    t2 = time.perf_counter()
    st = b.state()
    launch = b.launch_mode
    b.close()
    fin = dict(ps)
    fin.update({k: st[k] for k in ("rx", "ry", "rz", "vx", "vy", "vz")})
    e1 = DeviceHermite(fin, a.eta, order=4, adaptive=False, mode="exact")
    k1, p1 = e1.energy()
    e1.close()
    sweeps = 3 if a.order == 4 else 5        # acc_jerk x2 (+ snap x2) + tstep
    res = {"n": a.n, "order": a.order, "mode": a.mode, "t_end": a.t_end,
           "launch": launch,
           "time": b.time, "block_steps": b.nsteps,
           "active_updates": b.active,
           "mean_active": b.active / max(b.nsteps, 1),
           "wall_s": t2 - t1, "init_s": t1 - t0,
           "block_steps_per_s": b.nsteps / (t2 - t1),
           "updates_per_s": b.active / (t2 - t1),
           "gint_per_s": sweeps * b.active * a.n / (t2 - t1) / 1e9,
           "dE_over_E": ((k1 + p1) - (k0 + p0)) / -p0,
           "synchronised": bool(np.all(st["t"] == b.time))}
    print(json.dumps(res))


if __name__ == "__main__":
    main()
