"""Host restatement of the centred sweeps' grid for tile and warp centres
(csrc/csweep.cu: ct_grid_exp, ct_round_grid) and of the double-single
difference near tiles use (ds_sub), checking the two properties the sweep
relies on:

* every centre rounded to the grid is an exact float, and the difference of
  any two of them (a tile's and a warp's) is exact in FP32, so mid tiles
  shift a tile's positions to a warp's centre with one rounding per record;
* ds_sub of a position against a centre gives the same (hi, lo) pair
  whether it is formed for the tile (j side) or for the particle (i side),
  so a particle seen from itself differs by exactly zero.
"""

import numpy as np

f32 = np.float32


def grid_exp(lo, hi):
    """ct_grid_exp on the box's float bounds (3 axes)."""
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    ext = np.max(hi - lo)
    amax = np.max(np.maximum(np.abs(lo), np.abs(hi)))
    if not (np.isfinite(ext) and np.isfinite(amax)):
        return 0
    _, e1 = np.frexp(ext)
    _, e2 = np.frexp(amax)
    return max(int(e1) - 20, int(e2) - 24, -100)


def round_grid(v, e):
    """ct_round_grid: v (double) to the nearest multiple of 2^e, as float."""
    return np.float32(np.ldexp(np.rint(np.ldexp(np.float64(v), -e)), e))


def ds_sub(ah, al, b):
    """ds_sub of csweep.cu in FP32: (ah + al) - b as a normalised pair."""
    s = f32(ah - b)
    bb = f32(s - ah)
    e = f32(f32(ah - f32(s - bb)) + f32(f32(-b) - bb))
    e = f32(e + al)
    h = f32(s + e)
    low = f32(e - f32(h - s))
    return h, low


def split2(x):
    xh = np.float32(x)
    return xh, np.float32(np.float64(x) - np.float64(xh))


def test_grid_centres_and_their_differences_are_exact():
    rng = np.random.default_rng(11)
    for trial in range(400):
        scale = 10.0 ** rng.uniform(-4, 6)
        offset = rng.uniform(-1, 1, 3) * 10.0 ** rng.uniform(-6, 6)
        pts = offset + scale * rng.standard_normal((64, 3))
        lo = pts.astype(np.float32).min(0)
        hi = pts.astype(np.float32).max(0)
        e = grid_exp(lo, hi)
        # centres of tiles and warps: midpoints of random sub-boxes
        a = pts[rng.integers(0, 64, (40, 2))]
        mids = 0.5 * a[:, 0] + 0.5 * a[:, 1]
        cs = np.array([[round_grid(m, e) for m in row] for row in mids])
        assert np.all(np.float64(cs) == np.float64(cs.astype(np.float32)))
        for i in range(0, 40, 2):
            d32 = (cs[i] - cs[i + 1]).astype(np.float32)
            d64 = np.float64(cs[i]) - np.float64(cs[i + 1])
            assert np.all(np.float64(d32) == d64), (trial, e)


def test_double_single_self_difference_is_zero():
    rng = np.random.default_rng(12)
    x = rng.standard_normal(2000) * 10.0 ** rng.uniform(-3, 3, 2000)
    c = np.float32(rng.standard_normal() * 0.1)
    for xv in x:
        xh, xl = split2(xv)
        # tile side and particle side take the same operations
        dh_j, dl_j = ds_sub(xh, xl, c)
        dh_i, dl_i = ds_sub(xh, xl, c)
        d = f32(f32(dh_j - dh_i) + f32(dl_j - dl_i))
        assert d == 0.0
        # and the pair represents x - c to about 2^-48 relative
        rep = np.float64(dh_j) + np.float64(dl_j)
        assert abs(rep - (xv - np.float64(c))) <= 2.0 ** -44 * max(
            abs(xv), abs(np.float64(c)))
