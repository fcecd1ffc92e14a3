"""Forms of the universal-Kepler root solve (tg_kepler.cuh).

* "shared" evaluates cos/sin (cosh/sinh) once per Laguerre update instead of
  once per Stumpff function: the same operations on the same values, so the
  results must be bit-identical to the reference form.
* "mixed" iterates in FP32, then takes FP64 Laguerre updates until the
  reference's 2^-42 tolerance is met (or predicted to be met by the next
  update).  Its final states must agree with the oracle's full solve (the
  reference's arithmetic) within the bound the reference form is held to,
  1e-12 of the coordinate scale, with fewer FP64 updates; where the state
  is ill-conditioned in the root or the reference retried a step in
  substeps, test_mixed_form_matches_oracle states the wider bound.
"""

import numpy as np
import pytest

import oracle
from tupan_gb300 import ics, learned
from tupan_gb300 import kepler as kp

pytestmark = pytest.mark.gpu
NAMES = ("m", "rx", "ry", "rz", "e2", "vx", "vy", "vz")


def pair_set(n, seed, soft=False):
    rng = np.random.default_rng(seed)
    m = rng.uniform(1e-4, 1e-2, n)
    e2 = rng.uniform(1e-9, 1e-8, n) if soft else np.zeros(n)
    r = rng.uniform(1e-3, 5e-2, n)
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = rng.standard_normal((n, 3))
    vc = np.sqrt(m / r)[:, None]
    # bound (0.2-1.2 x circular) and unbound (up to 2 x) pairs
    st = np.concatenate([u * r[:, None],
                         w * vc * rng.uniform(0.2, 2.0, (n, 1))], axis=1)
    return m, e2, st


def solve(torch, form, dt, m, e2, st, use_mlp=False):
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    n = len(m)
    out = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    iters = torch.zeros(n, dtype=torch.int32, device="cuda")
    old = kp.set_form(form)
    try:
        kp.kepler_pairs(n, dt, T(m), T(e2), T(st), out, iters=iters,
                        use_mlp=use_mlp)
    finally:
        kp.set_form(old)
    return out.cpu().numpy(), iters.cpu().numpy()


# Unsoftened pairs: with softening the reference's energy check compares a
# Keplerian solution against the softened energy and keeps subdividing
# eccentric orbits until the solve budget runs out (status 3 in every form);
# softened pairs are covered at the Sakura level, where the reference's
# leapfrog branch takes them.
CASES = [(1.0 / 512, False), (1.0 / 32, False), (1.0 / 4, False)]


@pytest.mark.parametrize("dt,soft", CASES)
def test_shared_form_bit_identical(dt, soft):
    torch = pytest.importorskip("torch")
    m, e2, st = pair_set(3000, 7, soft)
    a, ia = solve(torch, "reference", dt, m, e2, st)
    b, ib = solve(torch, "shared", dt, m, e2, st)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ia, ib)


def lagrange_f(dt0, m, e2, st, root):
    """The Lagrange coefficient f = 1 - m S2(root) / r0 of each pair's final
    state: the reference's step setup and set_new_pos_vel
    (universal_kepler_solver.h:312-357, 360-425) restated in numpy.  The new
    velocity divides by f (g' = (1 + g f') / f), so where f is a
    cancellation (|f| << 1) the state carries about 2^-53 / |f| of rounding
    relative to its scale, whatever root the solve found."""
    r0 = np.sqrt((st[:, :3] ** 2).sum(1) + e2)
    v2 = (st[:, 3:] ** 2).sum(1)
    al = v2 - (2 - e2 / r0 ** 2) * m / r0
    z = al * root * root
    w = np.sqrt(np.abs(z))
    with np.errstate(all="ignore"):
        c0 = np.where(z < 0, np.cos(w), np.where(z > 0, np.cosh(w), 1.0))
        c2 = np.where(z != 0, (c0 - 1) / z, 0.5)
    return 1 - m * root * root * c2 / r0


@pytest.mark.parametrize("dt,soft", CASES)
def test_mixed_form_matches_oracle(dt, soft):
    torch = pytest.importorskip("torch")
    m, e2, st = pair_set(3000, 8, soft)
    want, it_w, solves = oracle.kepler_pairs(dt, m, e2, st)
    got, it_g = solve(torch, "mixed", dt, m, e2, st)
    ref, _ = solve(torch, "reference", dt, m, e2, st)
    scale = np.abs(st).max(axis=1, keepdims=True)
    dev = (np.abs(got - want) / scale).max(axis=1)
    dev_ref = (np.abs(ref - want) / scale).max(axis=1)
    dev_mr = (np.abs(got - ref) / scale).max(axis=1)
    _, _, root, _ = oracle.kepler_root(dt, m, e2, st)
    noise = 2.0 ** -53 / np.abs(lagrange_f(dt, m, e2, st, root))
    retried = solves > 1
    bad = np.flatnonzero(dev > 1e-12)
    print("dt=%g mixed max %.3g; above 1e-12: %s; reference form there %s; "
          "mixed - reference form %s; 2^-53/|f| %s; oracle solves %s; "
          "FP64 updates mixed %s oracle %s" % (
              dt, dev.max(), bad, dev_ref[bad], dev_mr[bad], noise[bad],
              solves[bad], it_g[bad], it_w[bad]))
    # per pair: within 1e-12 of the coordinate scale of the oracle (the
    # reference's arithmetic on libm) or of the reference form on the GPU
    # (CUDA's cos/sin against libm's), plus eight times the rounding that
    # the division by f carries (the mixed form's root is within a quarter
    # of 2^-42 of the reference's, so its S2 and f differ in the last bits);
    # within 1e-10 where the reference retried the step in substeps (a step
    # it could not solve whole): the mixed form's FP32 start may solve it in
    # fewer substeps, another rounding path
    tol = 1e-12 + 8 * noise
    ok = (dev <= tol) | (dev_mr <= tol) | (retried & (dev <= 1e-10))
    assert np.all(ok), np.flatnonzero(~ok)
    # FP64 updates: the reference form needs at least two per solve (one to
    # move, one to see the update fall below the tolerance)
    assert it_g.mean() < it_w.mean()


def test_mixed_form_on_sakura_pairs_with_learned_start():
    torch = pytest.importorskip("torch")
    dt = 1.0 / 512
    st, m, e2 = learned.kepler_pair_states(2048, 11, dt, flag=-1)
    want, _ = solve(torch, "reference", dt, m, e2, st)
    got, it = solve(torch, "mixed", dt, m, e2, st)
    scale = np.abs(st).max(axis=1, keepdims=True)
    assert np.all(np.abs(got - want) <= 1e-12 * scale)
    assert it.mean() <= 1.05
    try:
        net = learned.LearnedStart.load()
    except (OSError, KeyError):
        pytest.skip("no trained start network shipped")
    net.install()
    try:
        got2, _ = solve(torch, "mixed", dt, m, e2, st, use_mlp=True)
    finally:
        kp.clear_mlp()
    assert np.all(np.abs(got2 - want) <= 1e-12 * scale)


@pytest.mark.parametrize("flag", [-1, 1])
def test_sakura_queue_mixed_form_matches_oracle(flag):
    torch = pytest.importorskip("torch")
    ps = ics.plummer(1024, eps=0.0, seed=5, masses="salpeter")
    d = {k: torch.from_numpy(np.ascontiguousarray(ps[k])).cuda()
         for k in NAMES}
    out = [torch.zeros(1024, dtype=torch.float64, device="cuda")
           for _ in range(6)]
    dt = 1.0 / 512
    old = kp.set_form("mixed")
    try:
        nk, _ = kp.sakura_queue(1024, [d[k].data_ptr() for k in NAMES], 1024,
                                [d[k].data_ptr() for k in NAMES],
                                [o.data_ptr() for o in out], dt, flag)
    finally:
        kp.set_form(old)
    assert nk > 0
    want = oracle.run("sakura_kernel", ps, ps, {"dt": dt, "flag": flag})
    rs = max(np.abs(ps[k]).max() for k in ("rx", "ry", "rz"))
    vs = max(np.abs(ps[k]).max() for k in ("vx", "vy", "vz"))
    for c in range(6):
        g = out[c].cpu().numpy()
        atol = 1e-12 * (rs if c < 3 else vs)
        assert np.max(np.abs(g - want[c])) <= atol, c


def test_set_form_rejects_unknown():
    pytest.importorskip("torch")
    with pytest.raises(KeyError):
        kp.set_form("quad")
    L = kp._lib()
    assert L.tupan_gb300_kepler_set_form(7) == -1
