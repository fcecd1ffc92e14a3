"""Host restatement of the centred sweep's (warp, tile) classes
(csrc/csweep.cu): Morton order over the common bounding box, 256-particle
tiles with centre c on the common grid and radius R, warps of 32 sorted i,
near / mid / far from D' = (xh_i - c) + xl_i.  Checks the invariant the far
and mid forms rely on: no pair of a far or mid tile can coincide (every i is
beyond 1.25 R of c, every j within R), so those tiles need no r2 > 0 mask
and their differences are at least a quarter of the tile radius, including
for particles present twice and for a warp that holds a tile's own
particles (the self pairs fall in near tiles)."""

import numpy as np

from tests.test_centred_grid import grid_exp, round_grid, ds_sub, split2
from tupan_gb300 import ics

f32 = np.float32
CT, WARP, NEAR, MID = 256, 32, 1.25, 3.0


def spread3(v):
    r = np.zeros_like(v)
    for b in range(16):
        r |= ((v >> b) & 1) << (3 * b)
    return r


def morton_order(x):
    """ct_bbox + ct_keys + a stable sort (the radix sort is stable)."""
    lo = x.astype(np.float32).min(0).astype(np.float64)
    hi = x.astype(np.float32).max(0).astype(np.float64)
    ext = (hi - lo).max()
    scale = 65535.0 / ext if ext > 0 else 0.0
    q = np.clip((x - lo) * scale, 0, 65535).astype(np.int64)
    key = spread3(q[:, 0]) | (spread3(q[:, 1]) << 1) | (spread3(q[:, 2]) << 2)
    return np.argsort(key, kind="stable"), lo.astype(np.float32), \
        hi.astype(np.float32)


def classes(x):
    order, lo, hi = morton_order(x)
    e = grid_exp(lo, hi)
    xs = x[order]
    n = len(xs)
    ntiles = (n + CT - 1) // CT
    out = []
    for t in range(ntiles):
        js = xs[t * CT:(t + 1) * CT]
        tl = js.min(0)
        th = js.max(0)
        c = np.array([round_grid(0.5 * tl[a] + 0.5 * th[a], e)
                      for a in range(3)], np.float32)
        dh = np.stack([ds_sub(*split2(js[q, a]), c[a])[0]
                       for q in range(len(js)) for a in range(3)]).reshape(
                           len(js), 3).astype(np.float64)
        R = f32(np.sqrt((dh ** 2).sum(1).max()) * 1.0001)
        for w0 in range(0, n, WARP):
            wi = xs[w0:w0 + WARP]
            dp = np.empty((len(wi), 3))
            for q in range(len(wi)):
                for a in range(3):
                    xh, xl = split2(wi[q, a])
                    dp[q, a] = f32(f32(xh - c[a]) + xl)
            d2 = (dp ** 2).sum(1)
            if np.any(d2 <= (NEAR * R) ** 2):
                cls = "near"
            elif np.any(d2 <= (MID * R) ** 2):
                cls = "mid"
            else:
                cls = "far"
            if cls != "near":
                sep = np.sqrt(((wi[:, None, :] - js[None, :, :]) ** 2).sum(2))
                out.append((cls, float(sep.min()), float(R)))
    return out


def check(x):
    res = classes(x)
    assert res, "no far or mid tiles"
    for cls, sep, R in res:
        assert sep > 0.0
        assert sep >= 0.2 * R, (cls, sep, R)


def test_far_and_mid_tiles_never_hold_a_coinciding_pair():
    ps = ics.plummer(2048, eps=1e-4, seed=19)
    x = np.stack([ps["rx"], ps["ry"], ps["rz"]], 1)
    check(x)


def test_duplicated_positions_stay_in_near_tiles():
    rng = np.random.default_rng(20)
    base = rng.random((1024, 3)) * 10.0
    x = np.concatenate([base, base])[rng.permutation(2048)]
    check(x)
