"""splat_count_pairs (the work counts behind the compute roofline) against a
NumPy recount over the same sorted list, packed records and final_idx.

The backward-evaluated count follows from final_idx and the tile bins alone and
must match exactly.  The others depend on fp32 exponentials at the 1/255 and
1e-4 thresholds, which NumPy's exp reproduces only to the last bits, so they
are compared within 0.5 %."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _falloff(a, b, c, dx, dy):
    """The rasterizers' falloff with its roundings (splat_math.cuh): products
    rounded to fp32, fused multiply-adds formed in fp64 and rounded once."""
    f32 = np.float32
    adx = (a * dx).astype(f32)
    cdy2 = ((c * dy).astype(f32) * dy).astype(f32)
    inner = (adx.astype(np.float64) * dx + cdy2).astype(f32)
    bdx = (b * dx).astype(f32)
    half = (f32(0.5) * inner).astype(f32)
    return (bdx.astype(np.float64) * dy + half).astype(f32)


def _recount(ids, bins, rec, final_idx, h, w, bw):
    tiles_x = (w + bw - 1) // bw
    e_fwd = e_bwd = e_valid = e_tile = 0
    for t, (lo, hi) in enumerate(bins):
        if hi <= lo:
            continue
        ty, tx = divmod(t, tiles_x)
        ys, xs = np.meshgrid(np.arange(ty * bw, min(ty * bw + bw, h)),
                             np.arange(tx * bw, min(tx * bw + bw, w)), indexing="ij")
        ys, xs = ys.ravel(), xs.ravel()
        px = xs.astype(np.float32) + np.float32(0.5)
        py = ys.astype(np.float32) + np.float32(0.5)
        fidx = final_idx[ys, xs]
        r = rec[ids[lo:hi]]  # (L, 12)
        dx = (r[:, 0:1] - px[None, :]).astype(np.float32)
        dy = (r[:, 1:2] - py[None, :]).astype(np.float32)
        sigma = _falloff(r[:, 2:3], r[:, 3:4], r[:, 4:5], dx, dy)
        vis = np.exp(-sigma.astype(np.float64)).astype(np.float32)
        opac = r[:, 5:6]
        a_f = np.minimum(np.float32(0.999), opac * vis)
        a_b = np.minimum(np.float32(0.99), opac * vis)
        # forward: per pixel, entries up to and including the saturating one
        T = np.ones(len(px), np.float32)
        done = np.zeros(len(px), bool)
        for k in range(hi - lo):
            e_fwd += int((~done).sum())
            ok = ~done & (sigma[k] >= 0) & (a_f[k] >= np.float32(1 / 255))
            nT = (T * (np.float32(1) - a_f[k])).astype(np.float32)
            sat = ok & (nT <= np.float32(1e-4))
            T = np.where(ok & ~sat, nT, T)
            done |= sat
        idx = lo + np.arange(hi - lo)[:, None]
        inb = idx <= fidx[None, :]
        e_bwd += int(inb.sum())
        valid = inb & (sigma >= 0) & (a_b >= np.float32(1 / 255))
        e_valid += int(valid.sum())
        e_tile += int(valid.any(axis=1).sum())
    return e_fwd, e_bwd, e_valid, e_tile


def test_count_pairs_matches_numpy_recount():
    from jaxsplat_gb300.scenes import make_scene
    from jaxsplat_gb300.session import RenderSession

    sc = make_scene("small", seed=5, num_points=4000, img_shape=(72, 104))
    kw = sc.kwargs
    s = RenderSession(sc.spec.num_points, img_shape=kw["img_shape"], f=kw["f"], c=kw["c"],
                      glob_scale=kw["glob_scale"], clip_thresh=kw["clip_thresh"], block_size=16)
    s.set_inputs(sc.means3d, sc.scales, sc.quats, sc.colors, sc.opacities, sc.viewmat,
                 sc.background, sc.target)
    count = s.measure_capacity()
    s.step()
    got = s.count_pairs()
    h, w = kw["img_shape"]
    ids = s.ids_sorted[:count].cpu().numpy()
    bins = s.tile_bins.cpu().numpy().reshape(-1, 2)
    rec = s.packed.cpu().numpy().reshape(-1, 12)
    fidx = s.final_idx.cpu().numpy().reshape(h, w)
    e_fwd, e_bwd, e_valid, e_tile = _recount(ids, bins, rec, fidx, h, w, 16)
    assert got["bwd_evaluated"] == e_bwd
    for name, ref in (("fwd_evaluated", e_fwd), ("bwd_contributing", e_valid),
                      ("tile_gaussian_contributing", e_tile)):
        assert ref > 0, name
        assert abs(got[name] - ref) <= 0.005 * ref, (name, got[name], ref)
    assert got["bwd_contributing"] <= got["bwd_evaluated"]
    assert got["tile_gaussian_contributing"] <= count
