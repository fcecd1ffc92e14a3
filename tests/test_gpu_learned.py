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
    X = (rng.normal(size=(n, 4)) * [1, 2, 0.5, 3]).astype(np.float32)
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


def test_training_reduces_loss():
    pytest.importorskip("torch")
    from tupan_gb300.learned import LearnedStart, training_set
    X, Y, _ = training_set(dts=(1.0 / 8,), seeds=(1,), n_bodies=2048)
    ok = np.isfinite(Y)
    assert ok.mean() > 0.99
    net = LearnedStart(seed=1)
    hist = net.fit(X[ok], Y[ok], epochs=6, batch=4096)
    assert hist[-1] < 0.6 * hist[0], hist


def test_trained_start_keeps_states_and_cuts_the_iteration_tail():
    """What the trained network (trained on the GPU by
    `python -m tupan_gb300.learned`, shipped as kepler_start.npz) gains over
    the plain first guess dt/r when it starts every solve: converged states
    are unchanged (same stopping rule), and where the plain guess needs more
    than two Laguerre updates (larger dt) the mean count and the tail of
    long solves drop.  At dt = 1/512 both need the minimum of two updates
    for >99% of pairs."""
    pytest.importorskip("torch")
    from tupan_gb300 import kepler as kp
    from tupan_gb300.learned import LearnedStart, evaluate
    net = LearnedStart.load()
    net.gate = float("-inf")
    net.install()
    try:
        big = evaluate(net, 1.0 / 8, seeds=(77,), n_bodies=2048)
        small = evaluate(net, 1.0 / 512, seeds=(77,), n_bodies=2048)
    finally:
        kp.clear_mlp()
    print(big)
    print(small)
    for r in (big, small):
        assert r["max_state_diff_rel"] <= 1e-11
    tail = lambda h: sum(h[5:])
    assert big["mean_iters_learned"] < big["mean_iters_plain"]
    assert tail(big["hist_learned"]) < 0.5 * tail(big["hist_plain"])
    # where the plain guess is already at the two-update minimum the network
    # can only lose a little
    assert small["mean_iters_learned"] <= small["mean_iters_plain"] + 0.05


def test_shipped_gate_uses_the_network_where_it_pays():
    """The shipped gate (fitted from the measured cost of evaluating the
    network against the Laguerre updates it saves) keeps the plain guess
    where that is already at the two-update minimum and uses the network at
    long steps: no extra updates at dt = 1/512, a halved tail of long
    solves at dt = 1/8, states unchanged.  (Solve rates: the training
    report of `python -m tupan_gb300.learned`.)"""
    pytest.importorskip("torch")
    from tupan_gb300 import kepler as kp
    from tupan_gb300.learned import LearnedStart, evaluate
    net = LearnedStart.load()
    assert net.gate > float("-inf")
    net.install()
    try:
        rs = [evaluate(net, dt, seeds=(78,), n_bodies=2048)
              for dt in (1.0 / 512, 1.0 / 8)]
    finally:
        kp.clear_mlp()
    for r in rs:
        print(r["dt"], r["speedup"], r["mean_iters_plain"],
              r["mean_iters_learned"])
        assert r["max_state_diff_rel"] <= 1e-11
        assert r["mean_iters_learned"] <= r["mean_iters_plain"] + 0.005
    tail = lambda h: sum(h[5:])
    assert tail(rs[1]["hist_learned"]) < 0.5 * tail(rs[1]["hist_plain"])


@pytest.mark.parametrize("bias", [12.0, -12.0])
def test_bad_network_falls_back_to_the_plain_guess(bias):
    """A network whose guess is far off (its output bias set to +-12: starts
    e^12 times too large or too small) costs iterations but never the
    result: a start outside the trust region around the plain guess is not
    taken, and a solve from the learned start that has not converged after
    KEPLER_LEARNED_MAXITER updates is redone from the plain guess, so the
    converged states stay those of the plain solver."""
    pytest.importorskip("torch")
    from tupan_gb300 import kepler as kp
    from tupan_gb300.learned import LearnedStart, evaluate
    net = LearnedStart(seed=3)
    net.params[-1] = bias
    net._round()
    net.gate = float("-inf")
    net.install()
    try:
        r = evaluate(net, 1.0 / 512, seeds=(78,), n_bodies=1024)
    finally:
        kp.clear_mlp()
    print(r)
    assert r["pairs"] > 0
    assert r["max_state_diff_rel"] <= 1e-11
    # a far-off start never saves updates
    assert r["mean_iters_learned"] >= r["mean_iters_plain"]
