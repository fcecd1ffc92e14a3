"""Learned first guess for the universal-variable Kepler solver.

A 4 -> 64 -> 64 -> 1 MLP (SiLU, bf16 weights, FP32 accumulation) predicts
log(root / plain guess) for a pair solve from log r, log |v|,
r.v / (r |v|) and log(|dt| sqrt(m / r^3)).  The solver starts from
plain_guess * exp(prediction) and iterates to the unchanged 2^-42 tolerance
(universal_kepler_solver.h:251), so converged states do not change; only the
number of Laguerre updates can.

Training data are pair states that take the Kepler branch in Sakura sweeps
of Salpeter Plummer spheres, with the roots the plain solver converges to
(``tupan_gb300_kepler_pairs`` records them).  Training runs on the GPU with
the library's own forward/backward and Adam kernels (``csrc/mlp.cu``).
"""

import ctypes
import os

import numpy as np

from . import ics, lib
from . import kepler as kp

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "kepler_start.npz")
IN, H = 4, 64
N_PARAM = H * IN + H + H * H + H + H + 1
_VP = ctypes.c_void_p


def _declare(L):
    c = ctypes
    L.tupan_gb300_mlp_param_count.restype = c.c_int
    L.tupan_gb300_mlp_round.argtypes = [_VP] * 5 + [_VP]
    L.tupan_gb300_mlp_round.restype = c.c_int
    L.tupan_gb300_mlp_grad.argtypes = [_VP, _VP, _VP, _VP, c.c_uint64,
                                       c.c_float, _VP, _VP, _VP]
    L.tupan_gb300_mlp_grad.restype = c.c_int
    L.tupan_gb300_mlp_adam.argtypes = [_VP, _VP, _VP, _VP, c.c_float, c.c_int,
                                       _VP]
    L.tupan_gb300_mlp_adam.restype = c.c_int


def _lib():
    L = lib.load("float64")
    if not getattr(L, "_mlp_declared", False):
        _declare(L)
        L._mlp_declared = True
    assert L.tupan_gb300_mlp_param_count() == N_PARAM
    return L


def kepler_pair_states(n_bodies=4096, seed=1, dt=1.0 / 512, eps=0.0,
                       flag=-1):
    """Relative states (r, v), total masses and softenings of all pairs of a
    Salpeter Plummer sphere that take the Kepler branch of a Sakura sweep
    with the given flag (sakura_kernel_common.h:111-117, :151-164)."""
    ps = ics.plummer(n_bodies, eps=eps, seed=seed, masses="salpeter")
    r = np.stack([ps["rx"], ps["ry"], ps["rz"]], 1)
    v = np.stack([ps["vx"], ps["vy"], ps["vz"]], 1)
    m, e2 = ps["m"], ps["e2"]
    out_s, out_m, out_e = [], [], []
    for i0 in range(0, n_bodies, 256):
        ii = np.arange(i0, min(n_bodies, i0 + 256))
        dr = r[ii, None, :] - r[None, :, :]
        dv = v[ii, None, :] - v[None, :, :]
        if flag == -1:
            dr = dr - dv * dt
        mm = m[ii, None] + m[None, :]
        r2 = (dr * dr).sum(-1)
        v2 = (dv * dv).sum(-1)
        with np.errstate(divide="ignore", invalid="ignore"):
            R = 64 * (mm / v2)
            kep = ~(r2 > R * R)
        kep &= r2 > 0
        a, b = np.nonzero(kep)
        out_s.append(np.concatenate([dr[a, b], dv[a, b]], 1))
        out_m.append(mm[a, b])
        out_e.append(e2[ii][a] + e2[b])
    return (np.concatenate(out_s), np.concatenate(out_m),
            np.concatenate(out_e))


class LearnedStart(object):
    """Parameters, optimiser state and device buffers of the network."""

    def __init__(self, seed=0):
        import torch
        self.torch = torch
        self.L = _lib()
        dev = torch.device("cuda")
        rng = np.random.default_rng(seed)
        p = np.zeros(N_PARAM, np.float32)
        o = 0
        p[o:o + H * IN] = rng.normal(0, np.sqrt(1.0 / IN), H * IN)
        o += H * IN + H
        p[o:o + H * H] = rng.normal(0, np.sqrt(1.0 / H), H * H)
        o += H * H + H
        p[o:o + H] = rng.normal(0, np.sqrt(1.0 / H), H) * 0.1
        self.params = torch.from_numpy(p).to(dev)
        f32 = lambda n: torch.zeros(n, dtype=torch.float32, device=dev)
        self.m, self.v, self.grad = f32(N_PARAM), f32(N_PARAM), f32(N_PARAM)
        self.rw = f32(N_PARAM)
        self.loss = f32(1)
        self.norm = f32(8)
        self.norm[4:] = 1.0
        bf = lambda n: torch.zeros(n, dtype=torch.bfloat16, device=dev)
        self.w1, self.w2, self.w3 = bf(H * IN), bf(H * H), bf(H)
        self.gate = float("-inf")
        self.steps = 0
        self._round()

    def _round(self):
        st = self.L.tupan_gb300_mlp_round(
            self.params.data_ptr(), self.w1.data_ptr(), self.w2.data_ptr(),
            self.w3.data_ptr(), self.rw.data_ptr(), None)
        if st:
            raise lib.TupanGB300Error("mlp_round failed")

    def set_norm(self, X):
        X = np.asarray(X, np.float64)
        mu = X.mean(0)
        sd = X.std(0) + 1e-6
        self.norm.copy_(self.torch.from_numpy(
            np.concatenate([mu, 1.0 / sd]).astype(np.float32)))

    def gradient(self, X, Y):
        """Gradient of the mean squared error on (X, Y) (device tensors);
        returns (grad copy on host, mean squared error)."""
        n = X.shape[0]
        self.grad.zero_()
        self.loss.zero_()
        st = self.L.tupan_gb300_mlp_grad(
            self.rw.data_ptr(), self.norm.data_ptr(), X.data_ptr(),
            Y.data_ptr(), n, 1.0 / n, self.grad.data_ptr(),
            self.loss.data_ptr(), None)
        if st:
            raise lib.TupanGB300Error("mlp_grad failed")
        self.torch.cuda.synchronize()
        return self.grad.cpu().numpy().copy(), float(self.loss.item()) / n

    def fit(self, X, Y, epochs=20, batch=8192, lr=3e-3, seed=0):
        """Adam on mini-batches; X (n x 4) and Y (n) host or device arrays.
        Returns the mean squared error of each epoch."""
        torch = self.torch
        X = torch.as_tensor(np.asarray(X, np.float32)).cuda()
        Y = torch.as_tensor(np.asarray(Y, np.float32)).cuda()
        self.set_norm(X.cpu().numpy())
        n = X.shape[0]
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, device="cuda", generator=gen)
            tot = 0.0
            self.loss.zero_()
            for b0 in range(0, n, batch):
                idx = perm[b0:b0 + batch]
                xb = X[idx].contiguous()
                yb = Y[idx].contiguous()
                nb = xb.shape[0]
                self._round()
                st = self.L.tupan_gb300_mlp_grad(
                    self.rw.data_ptr(), self.norm.data_ptr(), xb.data_ptr(),
                    yb.data_ptr(), nb, 1.0 / nb, self.grad.data_ptr(),
                    self.loss.data_ptr(), None)
                self.steps += 1
                st |= self.L.tupan_gb300_mlp_adam(
                    self.params.data_ptr(), self.m.data_ptr(),
                    self.v.data_ptr(), self.grad.data_ptr(), lr, self.steps,
                    None)
                if st:
                    raise lib.TupanGB300Error("mlp training step failed")
            torch.cuda.synchronize()
            hist.append(float(self.loss.item()) / n)
        self._round()
        return hist

    def install(self):
        self._round()
        b1 = self.rw[H * IN:H * IN + H].contiguous()
        o2 = H * IN + H + H * H
        self._b2 = self.rw[o2:o2 + H].contiguous()
        self._b3 = self.rw[N_PARAM - 1:N_PARAM].contiguous()
        self._b1 = b1
        kp.set_mlp(self.w1, self._b1, self.w2, self._b2, self.w3, self._b3,
                   self.norm, self.gate)

    def fit_gate(self, X, iters_plain, iters_learned, cost):
        """Gate on feature 3, log(|dt| sqrt(m/r^3)), that maximises the
        updates saved net of the network's cost: the start is used where
        the feature exceeds the gate, and there each solve saves
        iters_plain - iters_learned updates and pays `cost` update
        equivalents for evaluating the network.  +inf (never) if no
        threshold saves anything."""
        f = np.asarray(X, np.float64)[:, 3]
        gain = (np.asarray(iters_plain, np.float64)
                - np.asarray(iters_learned, np.float64) - cost)
        order = np.argsort(-f, kind="stable")
        cum = np.cumsum(gain[order])
        k = int(np.argmax(cum))
        if cum[k] <= 0:
            self.gate = float("inf")
        else:
            lo = f[order[k + 1]] if k + 1 < len(f) else f[order[k]] - 1.0
            self.gate = float(0.5 * (f[order[k]] + lo))
        return self.gate

    def set_gate(self, X, iters, excess=0.1):
        """Gate on feature 3, log(|dt| sqrt(m/r^3)): the lowest value above
        which the plain guess averages more than 2 + excess updates."""
        f = np.asarray(X)[:, 3]
        it = np.asarray(iters, np.float64)
        edges = np.quantile(f, np.linspace(0, 1, 41))
        gate = float("inf")
        for a, b in zip(edges[:-1][::-1], edges[1:][::-1]):
            sel = (f >= a) & (f <= b)
            if sel.any() and it[sel].mean() > 2.0 + excess:
                gate = float(a)
            else:
                break
        self.gate = gate
        return gate

    def save(self, path=WEIGHTS):
        np.savez(path, params=self.params.cpu().numpy(),
                 norm=self.norm.cpu().numpy(), gate=np.float64(self.gate))

    @classmethod
    def load(cls, path=WEIGHTS):
        obj = cls()
        z = np.load(path)
        obj.params.copy_(obj.torch.from_numpy(z["params"]))
        obj.norm.copy_(obj.torch.from_numpy(z["norm"]))
        obj.gate = float(z["gate"]) if "gate" in z.files else float("-inf")
        obj._round()
        return obj


def training_set(dts=(1.0 / 512,), seeds=range(1, 9), n_bodies=4096,
                 flags=(-1, 1), keep_pairs=False):
    """(X, Y, iterations) of Kepler-branch pairs solved by the plain solver
    on the GPU; Y = log(root / plain guess).  keep_pairs: also the list of
    (dt, states, m, e2) batches the samples came from."""
    import torch
    Xs, Ys, Is, batches = [], [], [], []
    for dt in dts:
        for seed in seeds:
            for flag in flags:
                st, m, e2 = kepler_pair_states(n_bodies, seed, dt, flag=flag)
                n = len(m)
                T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
                out = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
                rx = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
                ry = torch.zeros(n, dtype=torch.float32, device="cuda")
                it = torch.zeros(n, dtype=torch.int32, device="cuda")
                kp.kepler_pairs(n, dt, T(m), T(e2), T(st), out, iters=it,
                                rec_x=rx, rec_y=ry)
                Xs.append(rx.cpu().numpy())
                Ys.append(ry.cpu().numpy())
                Is.append(it.cpu().numpy())
                if keep_pairs:
                    batches.append((dt, st, m, e2))
    out = (np.concatenate(Xs), np.concatenate(Ys), np.concatenate(Is))
    return out + (batches,) if keep_pairs else out


def solve_batches(batches, use_mlp):
    """Per-pair Laguerre updates and the solve time of every batch, plain or
    with the installed network."""
    import torch
    its, secs, updates = [], 0.0, 0
    for dt, st, m, e2 in batches:
        n = len(m)
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        sm, se, ss = T(m), T(e2), T(st)
        out = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
        it = torch.zeros(n, dtype=torch.int32, device="cuda")
        kp.kepler_pairs(n, dt, sm, se, ss, out, iters=it, use_mlp=use_mlp)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        kp.kepler_pairs(n, dt, sm, se, ss, out, iters=it, use_mlp=use_mlp)
        e1.record()
        torch.cuda.synchronize()
        secs += e0.elapsed_time(e1) / 1e3
        a = it.cpu().numpy()
        its.append(a)
        updates += int(a.sum())
    return np.concatenate(its), secs, updates


def evaluate(net, dt, seeds=(101,), n_bodies=4096):
    """Mean Laguerre updates per Kepler-branch pair solve, plain and with
    the learned start, and the largest difference of the converged states
    relative to each pair's coordinate scale."""
    import torch
    res = {"dt": dt, "pairs": 0}
    its = {"plain": [], "learned": []}
    secs = {"plain": 0.0, "learned": 0.0}
    worst = 0.0
    for seed in seeds:
        for flag in (-1, 1):
            st, m, e2 = kepler_pair_states(n_bodies, seed, dt, flag=flag)
            n = len(m)
            T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
            outs = {}
            for key, use in (("plain", False), ("learned", True)):
                out = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
                it = torch.zeros(n, dtype=torch.int32, device="cuda")
                sm, se, ss = T(m), T(e2), T(st)
                kp.kepler_pairs(n, dt, sm, se, ss, out, iters=it, use_mlp=use)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                kp.kepler_pairs(n, dt, sm, se, ss, out, iters=it, use_mlp=use)
                e1.record()
                torch.cuda.synchronize()
                secs[key] += e0.elapsed_time(e1) / 1e3
                outs[key] = out.cpu().numpy()
                its[key].append(it.cpu().numpy())
            scale = np.abs(st).max(axis=1)
            d = np.abs(outs["plain"] - outs["learned"]).max(axis=1) / scale
            worst = max(worst, float(d.max()))
            res["pairs"] += n
    for key in its:
        a = np.concatenate(its[key])
        res["mean_iters_" + key] = float(a.mean())
        res["hist_" + key] = np.bincount(np.minimum(a, 10),
                                         minlength=11).tolist()
    res["max_state_diff_rel"] = worst
    res["solves_per_s_plain"] = res["pairs"] / secs["plain"]
    res["solves_per_s_learned"] = res["pairs"] / secs["learned"]
    res["speedup"] = secs["plain"] / secs["learned"]
    return res


def main(argv=None):
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--dts", default="0.001953125,0.0078125,0.03125,0.125")
    ap.add_argument("--seeds", type=int, default=6)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args(argv)
    dts = [float(x) for x in a.dts.split(",")]
    t0 = time.time()
    X, Y, I, batches = training_set(dts=dts, seeds=range(1, a.seeds + 1),
                                    keep_pairs=True)
    ok = np.isfinite(Y)
    t1 = time.time()
    net = LearnedStart(seed=0)
    hist = net.fit(X[ok], Y[ok], epochs=a.epochs)
    t2 = time.time()
    # gate from measured costs: the network on every solve against the
    # plain start, on the training pairs
    net.gate = float("-inf")
    net.install()
    it_l, t_l, u_l = solve_batches(batches, True)
    kp.clear_mlp()
    it_p, t_p, u_p = solve_batches(batches, False)
    per_update = t_p / max(u_p, 1)
    cost = max(0.0, (t_l - per_update * u_l) / per_update / len(it_l))
    net.fit_gate(X, it_p, it_l, cost)
    net.save(a.out)
    net.install()
    evals = [evaluate(net, dt) for dt in dts]
    gate = net.gate
    net.gate = float("-inf")          # the network on every solve
    net.install()
    evals_all = [evaluate(net, dt) for dt in dts]
    net.gate = gate
    kp.clear_mlp()
    print(json.dumps({"samples": int(ok.sum()), "data_s": t1 - t0,
                      "train_s": t2 - t1, "gate": net.gate,
                      "network_cost_updates": cost, "loss": hist,
                      "eval": evals, "eval_everywhere": evals_all}))


if __name__ == "__main__":
    main()
