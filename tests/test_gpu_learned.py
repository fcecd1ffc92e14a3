"""Learned Kepler start: GPU forward/backward against the numpy oracle,
training, and solves that converge to the same states."""

import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_oracle():
    torch = pytest.importorskip("torch")
    from tupan_gb300.learned import LearnedStart
    rng = np.random.default_rng(4)
    n = 1000
    X = rng.normal(size=(n, 4)).astype(np.float32) * [1, 2, 0.5, 3]
    Y = rng.normal(size=n).astype(np.float32)
    Y[::97] = np.nan                       # failed solves carry no loss
    net = LearnedStart(seed=3)
    net.set_norm(X)
    g_gpu, loss_gpu = net.gradient(torch.from_numpy(X).cuda(),
                                   torch.from_numpy(Y).cuda())
    rw = net.rw.cpu().numpy().astype(np.float64)
    norm = net.norm.cpu().numpy().astype(np.float64)
    g_ref, sse = omlp.grad(rw, norm, X, Y, 1.0 / n)
    assert abs(loss_gpu - sse / n) <= 1e-4 * (sse / n)
    scale = np.abs(g_ref).max()
    assert np.max(np.abs(g_gpu - g_ref)) <= 2e-4 * scale
    # per-block sums: relative agreement on the large entries
    big = np.abs(g_ref) > 1e-2 * scale
    assert np.max(np.abs(g_gpu - g_ref)[big] / np.abs(g_ref)[big]) < 1e-3


def test_training_and_learned_start_keep_converged_states():
    torch = pytest.importorskip("torch")
    from tupan_gb300 import kepler as kp
    from tupan_gb300.learned import LearnedStart, evaluate, training_set
    dt = 1.0 / 8
    X, Y = training_set(dts=(dt,), seeds=range(1, 3), n_bodies=2048)
    ok = np.isfinite(Y)
    assert ok.mean() > 0.99
    net = LearnedStart(seed=1)
    hist = net.fit(X[ok], Y[ok], epochs=8, batch=4096)
    assert hist[-1] < 0.5 * hist[0]
    net.install()
    try:
        r = evaluate(net, dt, seeds=(77,), n_bodies=2048)
    finally:
        kp.clear_mlp()
    print(r)
    # the stopping rule is unchanged: converged states agree to round-off
    assert r["max_state_diff_rel"] <= 1e-11
    # and the learned start does not cost iterations where the plain guess
    # already needs more than the minimum of two
    assert r["mean_iters_learned"] <= r["mean_iters_plain"]
