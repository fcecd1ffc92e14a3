"""Device SIA on a Plummer sphere: wall time per base step and the
recursion statistics.

    python -m tupan_gb300.sia_bench --n 65536 --method sia21h.dkd --steps 2

Prints one JSON line: base steps, wall time, steps/s, recursion calls,
sweeps, partitions, deepest level, Kepler solves, the pair interactions
summed over all levels (and their rate) and the fp64 energy error (EXACT
Phi on the device).
"""

import argparse
import json
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--method", default="sia21h.dkd")
    ap.add_argument("--eta", type=float, default=1.0 / 64)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--mode", default="split", choices=["split", "exact"])
    ap.add_argument("--masses", default="salpeter")
    a = ap.parse_args(argv)

    from . import ics
    from .integrator import DeviceHermite, DeviceSIA

    ps = ics.plummer(a.n, eps=1e-4, seed=3, masses=a.masses)
    e = DeviceHermite(ps, a.eta, order=4, adaptive=False, mode="exact")
    k0, p0 = e.energy()
    e.close()
    d = DeviceSIA(ps, a.method, a.eta, mode=a.mode)
    t0 = time.perf_counter()
    times = d.evolve(1e9, max_steps=a.steps)
    t1 = time.perf_counter()
    st = d.state()
    stats = d.stats()
    d.close()
    fin = {k: ps[k][st["id"]] for k in ("m", "e2")}
    fin.update({k: st[k] for k in ("rx", "ry", "rz", "vx", "vy", "vz")})
    e = DeviceHermite(fin, a.eta, order=4, adaptive=False, mode="exact")
    k1, p1 = e.energy()
    e.close()
    res = {"n": a.n, "method": a.method, "mode": a.mode, "eta": a.eta,
           "t": float(times[-1]) if len(times) else 0.0,
           "base_steps": len(times), "wall_s": t1 - t0,
           "steps_per_s": len(times) / (t1 - t0),
           "dE_over_E": ((k1 + p1) - (k0 + p0)) / abs(k0 + p0)}
    res.update(stats)
    res["gint_per_s"] = stats["interactions"] / (t1 - t0) / 1e9
    print(json.dumps(res))


if __name__ == "__main__":
    main()
