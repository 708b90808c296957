"""The rasterizers' per-Gaussian culling box must be conservative: no pixel
centre outside it may pass the reference's test alpha >= 1/255 (evaluated
in fp32 the way the kernels evaluate it).  This restates the box of
write_record (jaxsplat_gb300/csrc/splat_math.cuh) in numpy and checks it by brute
force around random Gaussians, anisotropic and nearly degenerate ones
included (CPU only)."""

import numpy as np

MARGIN, SIGMA_FACTOR, MAX_COND, FAR = 0.01, 0.98, 1e4, 1e5


def box(x, y, a, b, c, o):
    """pack_kernel's box, in fp32 (Kahan determinant)."""
    f = np.float32
    x, y, a, b, c, o = map(f, (x, y, a, b, c, o))
    w = f(b * b)
    e = f(np.float64(b) * np.float64(b) - np.float64(w))  # exact rounding error of b*b
    det = f(f(np.float64(a) * np.float64(c) - np.float64(w)) - e)  # fmaf(a, c, -w) - e
    tr = f(a + c)
    vals = np.array([x, y, o, a, b, c, det], np.float64)
    if not (np.isfinite(vals).all() and abs(x) < FAR and abs(y) < FAR):
        return np.inf, np.inf
    if not (a > 0 and c > 0 and det > 0 and f(tr * tr) <= f(MAX_COND) * det and o > 0):
        return np.inf, np.inf
    q = f(f(2.0) * f(np.log(f(255.0) * o).astype(f) + f(MARGIN)) / f(SIGMA_FACTOR))
    if q <= 0:
        return -np.inf, -np.inf
    ex = f(np.sqrt(f(q * c / det)).astype(f) * f(1.001) + f(0.01))
    ey = f(np.sqrt(f(q * a / det)).astype(f) * f(1.001) + f(0.01))
    if ex >= FAR or ey >= FAR:
        return np.inf, np.inf
    return ex, ey


def fma32(x, y, z):
    """fp32 fused multiply-add (the product of two fp32 values is exact in
    fp64)."""
    return (np.asarray(x, np.float64) * np.asarray(y, np.float64) + np.asarray(z, np.float64)).astype(np.float32)


def passes(x, y, a, b, c, o, px, py):
    """fp32 alpha test of the forward kernel (the falloff's roundings as
    splat_math.cuh spells them out, exp in fp32)."""
    f = np.float32
    dx = f(x) - px
    dy = f(y) - py
    inner = fma32(f(a) * dx, dx, (f(c) * dy) * dy)
    sigma = fma32(f(b) * dx, dy, f(0.5) * inner)
    alpha = np.minimum(f(0.999), f(o) * np.exp(-sigma).astype(f))
    return (sigma >= 0) & (alpha >= f(1.0) / f(255.0))


def test_box_is_conservative():
    rng = np.random.default_rng(0)
    checked = 0
    for k in range(3000):
        # random covariance: rotation, axis std devs from 0.3 to 40 px
        s1, s2 = np.exp(rng.uniform(np.log(0.3), np.log(40.0), 2))
        th = rng.uniform(0, np.pi)
        R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
        cov = R @ np.diag([s1 * s1, s2 * s2]) @ R.T + 0.3 * np.eye(2)
        con = np.linalg.inv(cov)
        a, b, c = np.float32(con[0, 0]), np.float32(con[0, 1]), np.float32(con[1, 1])
        o = np.float32(rng.choice([rng.uniform(0.001, 0.02), rng.uniform(0.02, 1.0), 0.99999]))
        x, y = np.float32(rng.uniform(-50, 50)), np.float32(rng.uniform(-50, 50))
        hx, hy = box(x, y, a, b, c, o)
        if not np.isfinite(hx) and hx > 0:
            continue  # no bound: never culled
        # all pixel centres within 5 px beyond the box (or the whole window
        # for boxes that cull everything)
        lim_x = (hx if np.isfinite(hx) else 0) + 5
        lim_y = (hy if np.isfinite(hy) else 0) + 5
        xs = np.arange(np.floor(x - lim_x), np.ceil(x + lim_x) + 1, dtype=np.float32) + np.float32(0.5)
        ys = np.arange(np.floor(y - lim_y), np.ceil(y + lim_y) + 1, dtype=np.float32) + np.float32(0.5)
        PX, PY = np.meshgrid(xs, ys)
        ok = passes(x, y, a, b, c, o, PX, PY)
        outside = (x + hx < PX) | (x - hx > PX) | (y + hy < PY) | (y - hy > PY)
        assert not (ok & outside).any(), (k, x, y, a, b, c, o, hx, hy)
        checked += int(ok.sum())
    assert checked > 100_000


def test_degenerate_inputs_are_never_culled():
    for args in [(0, 0, 1.0, 2.0, 1.0, 0.5),         # indefinite
                 (0, 0, 1.0, 0.999999, 1.0, 0.5),    # nearly singular: condition too large
                 (0, 0, np.nan, 0.0, 1.0, 0.5), (0, 0, 1.0, 0.0, 1.0, np.nan),
                 (2e5, 0, 1.0, 0.0, 1.0, 0.5), (0, 0, -1.0, 0.0, -1.0, 0.5)]:
        hx, hy = box(*args)
        assert hx == np.inf and hy == np.inf, args
    # too faint to pass anywhere: culled everywhere
    hx, hy = box(0, 0, 1.0, 0.0, 1.0, 1.0 / 300.0)
    assert hx == -np.inf and hy == -np.inf
