"""Host restatement of the mixed-precision universal-Kepler root solve
(csrc/tg_kepler.cuh: stumpff_all_f32, kep_laguerre_f32, kep_laguerre_mixed)
in numpy: Laguerre updates of order 5 in FP32 (Stumpff c2, c3 from their
power series for |z| < 1) until |d| <= 2^-20 |s|, then FP64 updates
accepted when |d| <= 2^-42 or when Newton's bound on the next update,
|f'' / (2 f')| d^2, is below 2^-44.  Checks, on the Kepler-branch pairs of
a Sakura step, that the accepted root agrees with the oracle's root (the
reference's solve from the plain guess) to the reference's tolerance and
that one FP64 update suffices for nearly every pair.  numpy's FP32 cos/sin
stand in for the device's; the method, not the device arithmetic, is
checked here."""

import math

import numpy as np
import pytest

import oracle

f32 = np.float32
TOL = 2.0 ** -42


def setup(dt0, m, e2, p):
    r2 = float(p[0] ** 2 + p[1] ** 2 + p[2] ** 2)
    r2 += e2
    r = math.sqrt(r2)
    v2 = float(p[3] ** 2 + p[4] ** 2 + p[5] ** 2)
    rv = float(p[0] * p[3] + p[1] * p[4] + p[2] * p[5])
    beta = 2.0 - e2 / r2
    al = v2 - beta * m / r
    dt = dt0
    if al < 0:
        a = m / abs(al)
        T = 2 * 3.141592653589793 * a * math.sqrt(a / m)
        ratio = dt0 / T
        dt = (ratio - float(int(ratio))) * T
    g = dt / r
    if al > 0:
        sal = math.sqrt(al)
        ss = abs(2 * al * dt / (rv + (m + al * r) / sal))
        if ss > 1:
            g = math.copysign(1.0, dt) * math.log(ss) / sal
    return dt, r, rv, m, al, g


def stumpff(z, dtype):
    one = dtype(1)
    if abs(z) < 1 and dtype is f32:
        c2 = f32(1.0 / 20922789888000.0)
        c3 = f32(1.0 / 355687428096000.0)
        for k2, k3 in ((87178291200.0, 1307674368000.0),
                       (479001600.0, 6227020800.0), (3628800.0, 39916800.0),
                       (40320.0, 362880.0), (720.0, 5040.0),
                       (24.0, 120.0), (2.0, 6.0)):
            c2 = f32(c2 * z + f32(1.0 / k2))
            c3 = f32(c3 * z + f32(1.0 / k3))
        return f32(z * c2 + one), f32(z * c3 + one), c2, c3
    if z < 0:
        w = np.sqrt(dtype(-z))
        cw, sw = np.cos(w), np.sin(w)
    elif z > 0:
        w = np.sqrt(dtype(z))
        cw, sw = np.cosh(w), np.sinh(w)
    else:
        return one, one, dtype(0.5), dtype(1.0 / 6.0)
    s1 = dtype(sw / w)
    return (dtype(cw), s1, dtype((cw - one) / dtype(z)),
            dtype((s1 - one) / dtype(z)))


def fdd(s, k, dtype):
    dt, r0, rv0, m, al = (dtype(v) for v in k)
    s = dtype(s)
    c0, c1, c2, c3 = stumpff(dtype(al * s * s), dtype)
    S0, S1, S2, S3 = c0, s * c1, s * s * c2, s * s * s * c3
    b = m + al * r0
    f = dtype(r0 * s + rv0 * S2 + b * S3 - dt)
    df = dtype(r0 + rv0 * S1 + b * S2)
    ddf = dtype(rv0 * S0 + b * S1)
    return f, df, ddf


def lag_delta(f, df, ddf, dtype):
    a = df
    b = a * a - f * ddf
    h = a + math.copysign(1.0, float(a)) * np.sqrt(
        abs(dtype(4) * (dtype(5) * b - a * a)))
    return None if h == 0 else dtype(-dtype(5) * f / h)


def mixed_root(k, s0):
    s = f32(s0)
    kf = tuple(f32(v) for v in k)
    ok32 = False
    for it in range(16):
        d = lag_delta(*fdd(s, kf, f32), f32)
        if d is None or not np.isfinite(d):
            break
        s = f32(s + d)
        if abs(d) <= f32(9.5367431640625e-7) * abs(s):
            ok32 = True
            break
    x = float(s) if ok32 and math.copysign(1, float(s)) == math.copysign(
        1, s0) else s0
    n64 = 0
    for _ in range(64):
        f, df, ddf = fdd(x, k, np.float64)
        d = lag_delta(f, df, ddf, np.float64)
        x += d
        n64 += 1
        if abs(d) <= TOL or abs(ddf / (2 * df)) * d * d <= 0.25 * TOL:
            break
    return x, n64


def test_mixed_root_matches_the_reference_root():
    from tupan_gb300 import learned
    dt = 1.0 / 512
    st, m, e2 = learned.kepler_pair_states(1024, 7, dt, flag=-1)
    if len(m) == 0:
        pytest.skip("no Kepler-branch pairs")
    idx = np.random.default_rng(3).permutation(len(m))[:400]
    st, m, e2 = st[idx], m[idx], e2[idx]
    status, _, root, _ = oracle.kepler_root(dt, m, e2, st)
    ups = []
    for q in range(len(m)):
        if status[q] != 0:
            continue
        dtr, r0, rv0, mm, al, g = setup(dt, m[q], e2[q], st[q])
        x, n64 = mixed_root((dtr, r0, rv0, mm, al), g)
        ups.append(n64)
        assert abs(x - root[q]) <= 4 * TOL * max(1.0, abs(root[q])), (
            q, x, root[q])
    ups = np.array(ups)
    assert len(ups) > 100
    assert ups.mean() <= 1.05, ups.mean()
