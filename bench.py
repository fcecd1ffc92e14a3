"""Benchmark: Acc + AccJerk force sweeps at N = 262144 in SPLIT mode.

One step = one Acc sweep and one AccJerk sweep of all N i-particles against
all N j-particles of a seeded Plummer sphere (equal masses, eps = 1e-4),
i.e. 2 N^2 pairwise interactions (at this size both take the centred
kernels: Morton-ordered particles, tile-centred records).  ``value`` is
interactions per second with the particles resident in HBM (device-pointer
entry point, CUDA events on the launching stream, L2 flushed between
steps).  ``e2e`` is the same metric through the reference-facing plugin
object (``extensions.Acc`` / ``AccJerk`` ``.calc(ps, ps)`` on ordinary
pageable numpy arrays -> ``CUDAKernel.run`` -> the ``acc_kernel`` /
``acc_jerk_kernel`` C-ABI), copies included.  The roofline line covers the
dominant kernel, the AccJerk sweep, against the FP32 FMA throughput measured
in the same run.  The FP64 (EXACT) path's rate is measured on an i-subset
(the cost is exactly linear in ni) for the SPLIT / FP64 ratio.

``--impl reference`` times the CPU restatement of the reference kernels
(bit-identical to them) on all host cores over a bounded i-subset of the
same workload.

Multi-GPU (torchrun): every rank runs the same sweep on its own GPU
(replicas; the sweep has no exchange), value = all ranks' interactions over
the slowest rank's time.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("Gint/s at N=256k FP32-split vs fp64 (same GPU, |da|/|a|<=1e-6); "
          "Kepler solves/s")
FLOPS_ACC = 20      # acc_kernel_common.h:38
FLOPS_ACC_JERK = 42  # acc_jerk_kernel_common.h:56


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=262144)
    # fp64 EXACT i-subset: two CTAs of 128 i per SM fill the GPU (the cost
    # is linear in ni; a smaller subset would leave SMs idle)
    p.add_argument("--fp64-ni", type=int, default=2 * 152 * 128)
    p.add_argument("--cpu-ni", type=int, default=32768)
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler(object):
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def slowest_rank(times, world, device=None):
    """Max over ranks of each per-step time (replicas: the job finishes with
    its slowest rank).  Works on any process group backend (nccl, gloo)."""
    if world <= 1:
        return list(times)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(times), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_rate(interactions_per_rank, world, t_step):
    """Whole-job Gint/s: every rank sweeps its own replica."""
    return world * interactions_per_rank / t_step / 1e9


def roofline_traffic():
    """dram bytes per AccJerk launch of the bench's kernel from the committed
    ncu summary (the centred sweep at N = 262144)."""
    path = os.path.join(ROOT, "profiles", "acc_jerk_centred_n262144.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def achieved_aj(n, t_aj):
    """AccJerk TFLOP/s at the reference's 42 flop per interaction."""
    return n * n * FLOPS_ACC_JERK / t_aj / 1e12


def nominal_fp32_tflops(sms, sm_mhz):
    """SMs x 128 FP32 lanes x 2 flop per FMA x SM clock, in TFLOP/s."""
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12


def cpu_baseline(n, ni, ps, single_ni=None):
    """Oracle (bit-identical restatement of the reference C kernels) on all
    host threads over ni i-particles x all n j-particles, both kernels; and
    on one thread, as the reference ships (single-threaded C), over
    single_ni i-particles (default ni / 16, about the same wall time)."""
    import oracle
    threads = oracle.max_threads()

    def timed(k):
        sub = {a: np.ascontiguousarray(v[:k]) for a, v in ps.items()}
        t0 = time.perf_counter()
        oracle.run("acc_kernel", sub, ps)
        oracle.run("acc_jerk_kernel", sub, ps)
        return time.perf_counter() - t0

    dt = timed(ni)
    k1 = max(1, single_ni if single_ni is not None else ni // 16)
    oracle.set_threads(1)
    try:
        dt1 = timed(k1)
    finally:
        oracle.set_threads(threads)
    return {"value": 2.0 * ni * n / dt / 1e9, "unit": "Gint/s",
            "cores": threads, "kind": "port",
            "sample": "acc + acc_jerk, ni=%d x nj=%d of the N=%d Plummer "
                      "sphere (%.1f s)" % (ni, n, n, dt),
            "single_core": {"value": 2.0 * k1 * n / dt1 / 1e9,
                            "unit": "Gint/s", "cores": 1,
                            "sample": "ni=%d x nj=%d (%.1f s)" % (k1, n, dt1)}}


def kepler_long_step(long_dt, res, kp, learned, best, dl, n8, bufs):
    """Solves per second of every root-solve form, plain and learned start,
    on the Kepler-branch pairs at the long step dl (into long_dt)."""
    s8m, s8e, s8s, o8, i8 = bufs
    for form in ("reference", "shared", "mixed"):
        for mlp in (False, True):
            if mlp and res.get("solves_per_s_learned") is None:
                continue
            if mlp:
                learned.LearnedStart.load().install()
            old_form = kp.set_form(form)
            try:
                t = best(lambda: kp.kepler_pairs(n8, dl, s8m, s8e, s8s, o8,
                                                 iters=i8, use_mlp=mlp))
            finally:
                kp.set_form(old_form)
                if mlp:
                    kp.clear_mlp()
            tag = ("learned_" if mlp else "") + form
            long_dt["solves_per_s_%s" % tag] = n8 / t
            long_dt["mean_fp64_updates_%s" % tag] = float(
                i8.float().mean().item())
    if long_dt.get("solves_per_s_learned_mixed"):
        long_dt["learned_mixed_over_plain_reference"] = (
            long_dt["solves_per_s_learned_mixed"]
            / long_dt["solves_per_s_reference"])


def kepler_solves(torch, stream):
    """Second half of the metric: universal-Kepler pair solves per second on
    the Kepler-branch pairs of a Sakura sweep (Salpeter Plummer N = 4096,
    eps = 0, dt = 1/512: the config-5 half step; and dt = 1/8), plain first
    guess and learned start, and the queued Sakura sweep's pair rate."""
    import numpy as np
    from tupan_gb300 import ics, learned
    from tupan_gb300 import kepler as kp
    from tupan_gb300.lib import TupanGB300Error
    dt = 1.0 / 512
    st, m, e2 = learned.kepler_pair_states(4096, 11, dt, flag=-1)
    n = len(m)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    sm, se, ss = T(m), T(e2), T(st)
    out = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    it = torch.zeros(n, dtype=torch.int32, device="cuda")

    def best(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return min(ts)

    res = {"pairs": n, "dt": dt}
    # the three root-solve forms (reference structure; one cos/sin per
    # Laguerre update, bit-identical; FP32 then FP64 updates), plain start
    for form in ("reference", "shared", "mixed"):
        old_form = kp.set_form(form)
        try:
            t = best(lambda: kp.kepler_pairs(n, dt, sm, se, ss, out,
                                             iters=it))
        finally:
            kp.set_form(old_form)
        res["solves_per_s_%s" % form] = n / t
        res["mean_fp64_updates_%s" % form] = float(it.float().mean().item())
    res["solves_per_s_plain"] = res["solves_per_s_reference"]
    res["mean_iters_plain"] = res["mean_fp64_updates_reference"]
    try:
        net = learned.LearnedStart.load()
        net.install()
        for form in ("reference", "mixed"):
            old_form = kp.set_form(form)
            try:
                t = best(lambda: kp.kepler_pairs(n, dt, sm, se, ss, out,
                                                 iters=it, use_mlp=True))
            finally:
                kp.set_form(old_form)
            res["solves_per_s_learned_%s" % form] = n / t
            res["mean_fp64_updates_learned_%s" % form] = float(
                it.float().mean().item())
        res["solves_per_s_learned"] = res["solves_per_s_learned_reference"]
        res["learned_gate"] = net.gate
        kp.clear_mlp()
    except (OSError, KeyError):
        res["solves_per_s_learned"] = None
    if res.get("solves_per_s_learned_mixed"):
        res["learned_mixed_over_plain_reference"] = (
            res["solves_per_s_learned_mixed"] / res["solves_per_s_reference"])
        res["learned_mixed_over_plain_shared"] = (
            res["solves_per_s_learned_mixed"] / res["solves_per_s_shared"])
    # a long step: the Kepler-branch pairs of the same sphere at dt = 1/8
    # (longer arcs, more Laguerre updates), every form, plain and learned
    dl = 1.0 / 8
    st8, m8, e28 = learned.kepler_pair_states(4096, 11, dl, flag=-1)
    n8 = len(m8)
    s8m, s8e, s8s = T(m8), T(e28), T(st8)
    o8 = torch.zeros((n8, 6), dtype=torch.float64, device="cuda")
    i8 = torch.zeros(n8, dtype=torch.int32, device="cuda")
    long_dt = {"pairs": n8, "dt": dl}
    try:
        kepler_long_step(long_dt, res, kp, learned, best, dl, n8,
                         (s8m, s8e, s8s, o8, i8))
    except TupanGB300Error as exc:
        long_dt["error"] = str(exc)
    res["dt_1_8"] = long_dt
    ps = ics.plummer(4096, eps=0.0, seed=11, masses="salpeter")
    names = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")
    d = {k: T(ps[k]) for k in names}
    p = [d[k].data_ptr() for k in names]
    o = [torch.zeros(4096, dtype=torch.float64, device="cuda")
         for _ in range(6)]
    op = [x.data_ptr() for x in o]
    t = best(lambda: kp.sakura_queue(4096, p, 4096, p, op, dt, -1))
    res["sakura_pairs_per_s"] = 4096 * 4096 / t
    old_form = kp.set_form("mixed")
    try:
        t = best(lambda: kp.sakura_queue(4096, p, 4096, p, op, dt, -1))
    finally:
        kp.set_form(old_form)
    res["sakura_pairs_per_s_mixed"] = 4096 * 4096 / t
    return res


def noalloc_rate(torch, dev, ps, stream):
    """The allocation-free acc_jerk entry at its largest size (65536 i
    against 65536 j of the sphere's first particles), interactions/s."""
    import ctypes
    from tupan_gb300 import lib
    L = lib.load()
    f = L.tupan_gb300_acc_jerk_split_noalloc
    f.argtypes = ([ctypes.c_uint64] + [ctypes.c_void_p] * 8
                  + [ctypes.c_uint64] + [ctypes.c_void_p] * 8
                  + [ctypes.c_void_p] * 6 + [ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_uint)])
    f.restype = ctypes.c_int
    n = min(65536, len(ps["m"]))
    names = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")
    d = [torch.from_numpy(np.ascontiguousarray(ps[k][:n])).to(dev)
         for k in names]
    o = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(6)]
    args = ([n] + [x.data_ptr() for x in d] + [n] + [x.data_ptr() for x in d]
            + [x.data_ptr() for x in o] + [stream, None])
    f(*args)
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        st = f(*args)
        b.record()
        torch.cuda.synchronize()
        if st:
            return None
        ts.append(a.elapsed_time(b) / 1e3)
    return {"n": n, "gints": n * n / min(ts) / 1e9}


def reference_step(ps, sub):
    """One Acc + AccJerk sweep of the i-subset `sub` against all of `ps` on
    the host: the reference kernels compiled from their own sources
    (oracle/_ref, single-threaded C as shipped) fanned out over i-ranges on
    every host thread where they are built, else the oracle port (the same
    arithmetic bit for bit) on its own threads.  Returns (step, kind,
    threads)."""
    import oracle
    threads = oracle.max_threads()
    if not oracle.ref_available():
        def step():
            oracle.run("acc_kernel", sub, ps)
            oracle.run("acc_jerk_kernel", sub, ps)
        return step, "port", threads
    from concurrent.futures import ThreadPoolExecutor
    ni = len(sub["m"])
    cuts = np.linspace(0, ni, threads + 1).astype(int)
    chunks = [{k: np.ascontiguousarray(v[a:b]) for k, v in sub.items()}
              for a, b in zip(cuts[:-1], cuts[1:]) if b > a]
    pool = ThreadPoolExecutor(max_workers=len(chunks))

    def step():
        # ctypes releases the GIL for the duration of each C call
        jobs = [pool.submit(oracle.run_ref, name, c, ps)
                for name in ("acc_kernel", "acc_jerk_kernel") for c in chunks]
        for j in jobs:
            j.result()
    return step, "reference", len(chunks)


def run_reference(args):
    """--impl reference: the reference kernels' CPU path on all host
    threads (reference_step)."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    from tupan_gb300 import ics
    n = args.n
    ps = ics.plummer(n, eps=1e-4, seed=1)
    ni = args.cpu_ni
    sub = {k: np.ascontiguousarray(v[:ni]) for k, v in ps.items()}
    step, kind, threads = reference_step(ps, sub)
    warm, _, _ = reference_step(
        ps, {k: np.ascontiguousarray(v[:64]) for k, v in sub.items()})
    warm()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    val = 2.0 * ni * n / t / 1e9
    line = {"metric": METRIC, "value": val, "unit": "Gint/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic Plummer sphere (seeded)",
            "config": {"workload": "acc+acc_jerk sweep, Plummer N=%d eps=1e-4"
                                   % n, "sample_ni": ni, "n": n},
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": "Gint/s", "cores": threads,
                             "kind": kind,
                             "sample": "ni=%d x nj=%d per step" % (ni, n)},
            "e2e": {"value": val, "unit": "Gint/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    import torch.distributed as dist
    from tupan_gb300 import ics, lib

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    n = args.n
    ps = ics.plummer(n, eps=1e-4, seed=1 + rank)
    names8 = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")
    d_in = {k: torch.from_numpy(ps[k]).to(dev) for k in names8}
    d_acc = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(3)]
    d_aj = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(6)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32,
                        device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    p5 = [d_in[k].data_ptr() for k in names8[:5]]
    p8 = [d_in[k].data_ptr() for k in names8]

    def step(mode=lib.MODE_SPLIT, ni=n):
        lib.dev_sweep("acc_kernel", ni, p5, n, p5,
                      [t.data_ptr() for t in d_acc], mode=mode, stream=sh)
        lib.dev_sweep("acc_jerk_kernel", ni, p8, n, p8,
                      [t.data_ptr() for t in d_aj], mode=mode, stream=sh)

    # --- device-resident timing (value) -----------------------------------
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = lib.load().tupan_gb300_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))                 # evict L2 between steps
        a, b, c = ev[k]
        a.record(stream)
        lib.dev_sweep("acc_kernel", n, p5, n, p5,
                      [t.data_ptr() for t in d_acc], mode=lib.MODE_SPLIT,
                      stream=sh)
        b.record(stream)
        lib.dev_sweep("acc_jerk_kernel", n, p8, n, p8,
                      [t.data_ptr() for t in d_aj], mode=lib.MODE_SPLIT,
                      stream=sh)
        c.record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    if world > 1:
        dist.barrier()
    launches = lib.load().tupan_gb300_launch_count() - launches0
    t_acc = sum(e[0].elapsed_time(e[1]) for e in ev) / 1e3 / args.steps
    t_aj = sum(e[1].elapsed_time(e[2]) for e in ev) / 1e3 / args.steps
    t_step, t_acc, t_aj = slowest_rank([t_acc + t_aj, t_acc, t_aj], world,
                                       dev)
    inter = 2.0 * n * n
    value = job_rate(inter, world, t_step)

    # --- end to end through the drop-in plugin object (tupan's extension
    # surface: Acc / AccJerk .calc -> CUDAKernel.run -> acc_kernel /
    # acc_jerk_kernel C-ABI) on ordinary pageable numpy arrays, as tupan's
    # ParticleSystem holds them; right after the device-timed steps so both
    # see the same clocks --------------------------------------------------
    from tupan_gb300 import extensions
    from tupan_gb300.particles import Bodies
    bodies = Bodies(ps)
    x_acc = extensions.Acc("CUDA", "float64")
    x_aj = extensions.AccJerk("CUDA", "float64")
    old_mode = lib.set_mode(lib.MODE_SPLIT)

    def host_step():
        x_acc.calc(bodies, bodies)
        x_aj.calc(bodies, bodies)

    host_step()
    e2e_clocks = ClockSampler(local)
    e2e_clocks.start()
    t0 = time.perf_counter()
    ksteps = max(1, min(args.steps, 3))
    for _ in range(ksteps):
        host_step()
    t_e2e = (time.perf_counter() - t0) / ksteps
    e2e_clk = e2e_clocks.stop()
    lib.set_mode(old_mode)
    h2d = 8 * n * (5 + 8)
    d2h = 8 * n * (3 + 6)
    e2e_val = world * inter / t_e2e / 1e9

    # accuracy of this run's AccJerk against the fp64 EXACT sweep (the
    # product's fp64 path, bit-identical to the reference's fp64 kernel) of
    # an i-subset against all j
    acc_err = None
    wa = None
    idx = np.sort(np.random.default_rng(0).choice(n, 128, replace=False))
    if rank == 0:
        d_idx = torch.from_numpy(idx).to(dev)
        d_sub = {k: d_in[k].index_select(0, d_idx).contiguous()
                 for k in names8}
        d_ex = [torch.empty(len(idx), dtype=torch.float64, device=dev)
                for _ in range(6)]
        lib.dev_sweep("acc_jerk_kernel", len(idx),
                      [d_sub[k].data_ptr() for k in names8], n, p8,
                      [t.data_ptr() for t in d_ex], mode=lib.MODE_EXACT,
                      stream=sh)
        torch.cuda.synchronize()
        wa = np.stack([t.cpu().numpy() for t in d_ex[:3]])
        got = [t.cpu().numpy()[idx] for t in d_aj]
        ga = np.stack(got[:3])
        rel = np.linalg.norm(ga - wa, axis=0) / np.linalg.norm(wa, axis=0)
        acc_err = {"max": float(rel.max()), "median": float(np.median(rel)),
                   "sample_i": int(len(idx)),
                   "reference": "fp64 EXACT sweep of the same i against all j"}

    # --- the same sweeps with the Newton step after rsqrt (the variant the
    # default replaces: 9 -> 5, 10 -> 7, 11 -> 0), for comparison ----------
    newton = None
    v_def, g_def = lib.split_choice("acc_jerk_kernel", n, n)
    v_nr = {9: 5, 10: 7, 11: 0}.get(v_def)
    if rank == 0 and v_nr is not None:
        for name in ("acc_kernel", "acc_jerk_kernel"):
            lib.set_split_config(name, v_nr, g_def)
        lib.set_centred(0)
        try:
            step()
            f0, f1, f2 = (torch.cuda.Event(enable_timing=True)
                          for _ in range(3))
            flush.fill_(0.5)
            f0.record(stream)
            lib.dev_sweep("acc_kernel", n, p5, n, p5,
                          [t.data_ptr() for t in d_acc], mode=lib.MODE_SPLIT,
                          stream=sh)
            f1.record(stream)
            lib.dev_sweep("acc_jerk_kernel", n, p8, n, p8,
                          [t.data_ptr() for t in d_aj], mode=lib.MODE_SPLIT,
                          stream=sh)
            f2.record(stream)
            torch.cuda.synchronize()
        finally:
            for name in ("acc_kernel", "acc_jerk_kernel"):
                lib.set_split_config(name, -1, 0)
            lib.set_centred(-1, -1, 0)
        got = [t.cpu().numpy()[idx] for t in d_aj]
        rel = (np.linalg.norm(np.stack(got[:3]) - wa, axis=0) /
               np.linalg.norm(wa, axis=0))
        newton = {"variant": v_nr, "gsplit": g_def,
                  "acc_split_gints": n * n / (f0.elapsed_time(f1) / 1e3) / 1e9,
                  "acc_jerk_split_gints":
                      n * n / (f1.elapsed_time(f2) / 1e3) / 1e9,
                  "acc_rel_err_vs_fp64": {
                      "max": float(rel.max()),
                      "median": float(np.median(rel))}}

    # --- the same sweeps on the double-single split variants (the path
    # the centred kernels replace at this size), for comparison ------------
    variants_cmp = None
    if rank == 0:
        lib.set_centred(0)
        try:
            step()
            f0, f1, f2 = (torch.cuda.Event(enable_timing=True)
                          for _ in range(3))
            flush.fill_(0.25)
            f0.record(stream)
            lib.dev_sweep("acc_kernel", n, p5, n, p5,
                          [t.data_ptr() for t in d_acc], mode=lib.MODE_SPLIT,
                          stream=sh)
            f1.record(stream)
            lib.dev_sweep("acc_jerk_kernel", n, p8, n, p8,
                          [t.data_ptr() for t in d_aj], mode=lib.MODE_SPLIT,
                          stream=sh)
            f2.record(stream)
            torch.cuda.synchronize()
            v_sv, g_sv = lib.split_choice("acc_jerk_kernel", n, n)
        finally:
            lib.set_centred(-1, -1, 0)
        variants_cmp = {
            "variant": v_sv, "gsplit": g_sv,
            "acc_split_gints": n * n / (f0.elapsed_time(f1) / 1e3) / 1e9,
            "acc_jerk_split_gints": n * n / (f1.elapsed_time(f2) / 1e3) / 1e9}

    # --- the centred sweeps without mid tiles (every tile beyond 1.25 R on
    # the one-operation far difference): faster, less accurate on particles
    # whose net force is a near-cancelling sum ---------------------------
    mid_off = None
    if rank == 0:
        prev_mid = lib.set_centred_mid(0.0)
        try:
            step()
            f0, f1, f2 = (torch.cuda.Event(enable_timing=True)
                          for _ in range(3))
            flush.fill_(0.125)
            f0.record(stream)
            lib.dev_sweep("acc_kernel", n, p5, n, p5,
                          [t.data_ptr() for t in d_acc], mode=lib.MODE_SPLIT,
                          stream=sh)
            f1.record(stream)
            lib.dev_sweep("acc_jerk_kernel", n, p8, n, p8,
                          [t.data_ptr() for t in d_aj], mode=lib.MODE_SPLIT,
                          stream=sh)
            f2.record(stream)
            torch.cuda.synchronize()
        finally:
            lib.set_centred_mid(prev_mid)
        t_mo = f1.elapsed_time(f2) / 1e3
        mid_off = {
            "mid_reach": 0.0, "default_mid_reach": prev_mid,
            "acc_split_gints": n * n / (f0.elapsed_time(f1) / 1e3) / 1e9,
            "acc_jerk_split_gints": n * n / t_mo / 1e9,
            "acc_jerk_tflops": achieved_aj(n, t_mo)}

    # --- FP64 EXACT path on an i-subset (linear in ni) ---------------------
    ni64 = min(args.fp64_ni, n)
    step(lib.MODE_EXACT, ni64)     # warm
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    lib.dev_sweep("acc_kernel", ni64, p5, n, p5,
                  [t.data_ptr() for t in d_acc], mode=lib.MODE_EXACT,
                  stream=sh)
    e1.record(stream)
    lib.dev_sweep("acc_jerk_kernel", ni64, p8, n, p8,
                  [t.data_ptr() for t in d_aj], mode=lib.MODE_EXACT,
                  stream=sh)
    e2.record(stream)
    torch.cuda.synchronize()
    t64 = (e0.elapsed_time(e2)) / 1e3
    fp64_gints = 2.0 * ni64 * n / t64 / 1e9
    fp64_aj_gints = ni64 * n / (e1.elapsed_time(e2) / 1e3) / 1e9

    # --- FP32 FMA throughput measured now (roofline denominator) ----------
    peak = lib.load()
    import ctypes
    peak.tupan_gb300_fp32_peak_tflops.restype = ctypes.c_double
    peak.tupan_gb300_fp32_peak_tflops.argtypes = [ctypes.c_int, ctypes.c_int]
    fp32_peak = float(peak.tupan_gb300_fp32_peak_tflops(20000, 5))
    # the same peak derived from the SM count and the SM clock sampled under
    # load, as a cross-check of the measured one
    nominal = None
    try:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        mhz = float(clk.get("sm_mhz") or clk.get("sm_max_mhz"))
        tf = nominal_fp32_tflops(sms, mhz)
        nominal = {"value": tf, "unit": "TFLOP/s", "sms": sms,
                   "sm_mhz": mhz, "frac": achieved_aj(n, t_aj) / tf,
                   "formula": "SMs x 128 lanes x 2 flop x SM clock"}
    except Exception:
        nominal = None
    if mid_off is not None and nominal is not None:
        mid_off["acc_jerk_frac_nominal"] = (mid_off["acc_jerk_tflops"]
                                            / nominal["value"])

    kepler = kepler_solves(torch, stream) if rank == 0 else None
    noalloc = noalloc_rate(torch, dev, ps, sh) if rank == 0 else None

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    cpu = None if args.no_cpu else cpu_baseline(n, args.cpu_ni, ps)
    achieved = n * n * FLOPS_ACC_JERK / t_aj / 1e12
    traffic = roofline_traffic()
    path_aj, cfg_aj, g_aj = lib.sweep_plan("acc_jerk_kernel", n, n)
    cur_mid = lib.set_centred_mid(3.0)
    lib.set_centred_mid(cur_mid)
    kname = ("ct_sweep<CtAccJerk> (centred, shape %d)" % cfg_aj
             if path_aj == 1 else
             "split_sweep<AccJerkS> variant %d" % cfg_aj)
    line = {
        "metric": METRIC, "value": value, "unit": "Gint/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-split",
        "data": "synthetic Plummer sphere (seeded, equal masses)",
        "config": {"workload": "acc + acc_jerk sweep, all i vs all j, Plummer "
                               "N=%d eps=1e-4, SPLIT mode" % n,
                   "n": n, "interactions_per_step": inter,
                   "l2": "flushed between steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "acc_jerk_path": "centred" if path_aj == 1 else "split",
                   "acc_jerk_config": cfg_aj, "acc_jerk_gsplit": g_aj,
                   "centred_mid_reach": cur_mid},
        "kernels": {"acc_split_gints": n * n / t_acc / 1e9,
                    "acc_jerk_split_gints": n * n / t_aj / 1e9,
                    "fp64_exact_gints": fp64_gints,
                    "fp64_exact_acc_jerk_gints": fp64_aj_gints,
                    "fp64_sample_ni": ni64,
                    "split_over_fp64": (inter / t_step) / (2.0 * ni64 * n / t64),
                    "acc_rel_err_vs_fp64": acc_err,
                    "newton_form": newton,
                    "split_variants_path": variants_cmp,
                    "centred_mid_off": mid_off,
                    "noalloc_acc_jerk": noalloc},
        "roofline": {"bound": "fp32",
                     "kernel": kname,
                     "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "flops_per_interaction": FLOPS_ACC_JERK,
                     "peak_source": "FP32 FMA-chain kernel measured in this "
                                    "run (MEASURED_PEAKS.json has no FP32 "
                                    "figure)",
                     "peak_nominal": nominal,
                     "traffic": traffic},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "Gint/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "tupan_gb300.extensions Acc/AccJerk .calc(ps, ps) -> "
                        "CUDAKernel.run -> acc_kernel / acc_jerk_kernel C-ABI, "
                        "pageable numpy arrays, SPLIT mode",
                "ms_per_step": t_e2e * 1e3, "clocks": e2e_clk},
        "kepler": kepler,
        "gpu_launches": int(launches),
        "clocks": clk,
        "wall_s_timed": t_wall,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
