"""CPU replay of how the 16x16 rasterizers walk a tile's list, on the oracle's
projection, sorted lists and final_idx (test infrastructure).

Warp layout (jaxsplat_gb300/csrc/raster.cu, fwd16_tile and bwd16_tile), the
same in both passes: 4 warps of 8x8 pixels, warp w at ((w & 1) * 8, (w >> 1) * 8);
lane l holds pixels (l & 7, l >> 3) and (l & 7, (l >> 3) + 4).
  forward:  a warp walks the batch entries whose culling box meets its
            rectangle until every one of its pixels has saturated;
  backward: a warp walks the entries up to its largest final_idx whose box
            meets its rectangle.
An iteration "does work" when at least one lane passes the pixel test
(sigma >= 0, alpha >= 1/255; in the backward also idx <= the pixel's
final_idx, backward.cu:240-265).

The replay checks three facts on realistic lists:
  * the replayed forward gives the oracle's final_idx at every pixel;
  * no pair that contributes lies outside the culling box of write_record
    (splat_math.cuh), so the box never changes a result;
  * per warp, the entries with a valid pixel in the backward are exactly the
    entries the same warp blended at some pixel in the forward: the blend
    bytes the forward records (one bit per warp and entry) are an exact skip
    list for the backward.
and counts the iterations each warp executes and how many of them do work.

``walk_stats(scene, tiles=k)`` returns the counts for a seeded sample of k
tiles of a scene (the figures quoted for the 1M-Gaussian 1920x1080 scene use
400 tiles of ``make_scene("hd", seed=0)``)."""


import numpy as np

f32, f64 = np.float32, np.float64

# write_record's culling-box constants (splat_math.cuh)
MARGIN, SIGMA_FACTOR, MAX_COND, FAR = 0.01, 0.98, 1e4, 1e5


def cull_boxes(x, y, a, b, c, o):
    """Half-extents (ex, ey) of write_record's box for arrays of Gaussians, in
    fp32: +inf where the record keeps every pixel, -inf where it keeps none."""
    w = (b * b).astype(f32)
    e = (b.astype(f64) * b - w).astype(f32)  # rounding error of b*b
    det = ((a.astype(f64) * c - w).astype(f32) - e).astype(f32)
    tr = (a + c).astype(f32)
    with np.errstate(all="ignore"):
        ok = (np.isfinite(x) & np.isfinite(y) & np.isfinite(a) & np.isfinite(b)
              & np.isfinite(c) & np.isfinite(o) & (abs(x) < FAR) & (abs(y) < FAR) & (a > 0)
              & (c > 0) & (det > 0) & ((tr * tr).astype(f32) <= f32(MAX_COND) * det) & (o > 0))
        q = (f32(2) * (np.log(f32(255) * o).astype(f32) + f32(MARGIN))
             / f32(SIGMA_FACTOR)).astype(f32)
        ex = (np.sqrt((q * c / det).astype(f32)) * f32(1.001) + f32(0.01)).astype(f32)
        ey = (np.sqrt((q * a / det).astype(f32)) * f32(1.001) + f32(0.01)).astype(f32)
    ex = np.where(q <= 0, -np.inf, ex)
    ey = np.where(q <= 0, -np.inf, ey)
    keep = ok & ~((ex >= FAR) | (ey >= FAR))
    return np.where(keep, ex, np.inf).astype(f32), np.where(keep, ey, np.inf).astype(f32)


def falloff(a, b, c, dx, dy):
    """The rasterizers' falloff with its roundings (splat_math.cuh)."""
    adx = (a * dx).astype(f32)
    cdy2 = ((c * dy).astype(f32) * dy).astype(f32)
    inner = (adx.astype(f64) * dx + cdy2).astype(f32)
    bdx = (b * dx).astype(f32)
    half = (f32(0.5) * inner).astype(f32)
    return (bdx.astype(f64) * dy + half).astype(f32)


def _meets(x, y, hx, hy, x0, x1, y0, y1):
    return ~((x + hx < x0) | (x - hx > x1) | (y + hy < y0) | (y - hy > y1))


COUNT_KEYS = ("entries", "tile_contributing", "past_saturation", "fwd_walk", "fwd_work",
              "fwd_active_pixels", "bwd_staged", "bwd_walk", "bwd_work", "bwd_valid_pixels", "bwd_atomics",
              "final_idx_mismatch", "box_culled_contributing", "identity_mismatch")


def _replay_tile(tot, lanes_hist, lo, hi, ox, oy, h, w, ids, xys, con, opac, ex_all, ey_all,
                 fidx_img, few_lanes):
    L = hi - lo
    g = ids[lo:hi]
    gx, gy = xys[g, 0], xys[g, 1]
    a, b, c = con[g, 0], con[g, 1], con[g, 2]
    op = opac[g]
    ex, ey = ex_all[g], ey_all[g]
    ky, kx = np.divmod(np.arange(256), 16)
    pxi, pyi = ox + kx, oy + ky
    inside = (pxi < w) & (pyi < h)
    px = pxi.astype(f32) + f32(0.5)
    py = pyi.astype(f32) + f32(0.5)
    dx = (gx[:, None] - px[None, :]).astype(f32)
    dy = (gy[:, None] - py[None, :]).astype(f32)
    sig = falloff(a[:, None], b[:, None], c[:, None], dx, dy)
    vis = np.exp(-sig.astype(f64)).astype(f32)
    al = np.minimum(f32(0.999), op[:, None] * vis)
    passes = (sig >= 0) & (al >= f32(1 / 255)) & inside[None, :]

    # forward, per pixel, in list order (forward.cu:399-440)
    T = np.ones(256, f32)
    done_at = np.full(256, L, np.int64)
    active = inside.copy()
    blended = np.zeros((L, 256), bool)
    for k in range(L):
        m = active & passes[k]
        nT = (T * (f32(1) - al[k])).astype(f32)
        sat = m & (nT <= f32(1e-4))
        done_at[sat] = k
        blended[k] = m & ~sat
        T = np.where(blended[k], nT, T)
        active &= ~sat
        if not active.any():
            break
    tot["entries"] += L
    tot["tile_contributing"] += int(blended.any(axis=1).sum())
    # entries after the last one any pixel of the tile evaluates
    tot["past_saturation"] += max(0, L - 1 - int(done_at[inside].max(initial=-1)))
    last = np.where(blended.any(axis=0), L - 1 - np.argmax(blended[::-1], axis=0), -1)
    replay_fidx = np.where(last >= 0, lo + last, 0)
    fid = np.where(inside, fidx_img[np.minimum(pyi, h - 1), np.minimum(pxi, w - 1)], 0)
    tot["final_idx_mismatch"] += int((replay_fidx != fid)[inside].sum())
    rows = np.arange(L)
    # the backward stages (gathers the records of) every entry up to the
    # block's largest final_idx
    tot["bwd_staged"] += min(L, max(0, int(fid[inside].max(initial=0)) - lo + 1))

    for wv in range(4):
        x0, y0 = (wv & 1) * 8, (wv >> 1) * 8
        sel = (kx >= x0) & (kx < x0 + 8) & (ky >= y0) & (ky < y0 + 8)
        mb = _meets(gx, gy, ex, ey, f32(ox + x0 + 0.5), f32(ox + x0 + 7.5), f32(oy + y0 + 0.5),
                    f32(oy + y0 + 7.5))
        pix_done = np.where(inside[sel], done_at[sel], -1)
        walk = mb & (rows <= pix_done.max())
        still = rows[:, None] <= pix_done[None, :]
        tot["fwd_walk"] += int(walk.sum())
        tot["fwd_work"] += int((walk & (passes[:, sel] & still).any(axis=1)).sum())
        # pixels not yet saturated (inside the image) in each walked iteration
        tot["fwd_active_pixels"] += int((still & inside[sel][None, :])[walk].sum())

    for W in range(4):
        x0, y0 = (W & 1) * 8, (W >> 1) * 8
        sel = (kx >= x0) & (kx < x0 + 8) & (ky >= y0) & (ky < y0 + 8)
        mb = _meets(gx, gy, ex, ey, f32(ox + x0 + 0.5), f32(ox + x0 + 7.5), f32(oy + y0 + 0.5),
                    f32(oy + y0 + 7.5))
        walk = mb & (rows <= fid[sel].max() - lo)
        valid = (rows[:, None] <= (fid[sel] - lo)[None, :]) & passes[:, sel]
        any_valid = valid.any(axis=1)
        work = walk & any_valid
        tot["bwd_walk"] += int(walk.sum())
        tot["bwd_work"] += int(work.sum())
        tot["box_culled_contributing"] += int((any_valid & ~mb).sum())
        tot["identity_mismatch"] += int((any_valid != blended[:, sel].any(axis=1)).sum())
        vv = valid[work]
        lane = (kx[sel] - x0) + 8 * ((ky[sel] - y0) % 4)
        lanes = np.zeros((vv.shape[0], 32), bool)
        for k in range(64):
            lanes[:, lane[k]] |= vv[:, k]
        nl = lanes.sum(axis=1)
        np.add.at(lanes_hist, nl, 1)
        tot["bwd_valid_pixels"] += int(vv.sum())
        # nine fields per (warp, Gaussian): per lane up to few_lanes lanes,
        # else once after the warp reduction (raster.cu, bwd16_tile)
        tot["bwd_atomics"] += int(np.where(nl <= few_lanes, 9 * nl, 9).sum())


def walk_stats(scene, tiles=None, seed=0, few_lanes=16, threads=None):
    """Replay the warp walks of the 16x16 rasterizers on ``scene`` (a
    jaxsplat_gb300.scenes.Scene with block width 16) over all non-empty tiles,
    or over ``tiles`` of them drawn with ``seed``.  Returns the totals of
    COUNT_KEYS, "tiles" and "lanes_hist" (backward iterations that do work,
    by number of lanes with a valid pixel)."""
    from oracle.oracle import Oracle

    kw = scene.kwargs
    h, w = kw["img_shape"]
    bw = scene.spec.block_width
    if bw != 16:
        raise ValueError("the replay follows the 16x16 warp layouts")
    o = Oracle("f32")
    o.set_threads(threads or o.max_threads())
    p = o.project_fwd(scene.means3d, scene.scales, scene.quats, scene.viewmat, block_width=bw,
                      **kw)
    s = o.sort_and_bin(p["xys"], p["depths"], p["radii"], p["cum_tiles_hit"], img_shape=(h, w),
                       block_width=bw)
    r = o.rasterize_fwd(s["gaussian_ids_sorted"], s["tile_bins"], p["xys"], p["conics"],
                        scene.colors, scene.opacities, scene.background, img_shape=(h, w),
                        block_width=bw)
    bins = s["tile_bins"]
    xys = p["xys"].astype(f32)
    con = p["conics"].astype(f32)
    opac = np.asarray(scene.opacities, f32).reshape(-1)
    ex, ey = cull_boxes(xys[:, 0], xys[:, 1], con[:, 0], con[:, 1], con[:, 2], opac)
    tiles_x = (w + bw - 1) // bw
    pick = np.nonzero(bins[:, 1] > bins[:, 0])[0]
    if tiles is not None and tiles < pick.size:
        pick = np.random.default_rng(seed).choice(pick, size=tiles, replace=False)
    tot = dict.fromkeys(COUNT_KEYS, 0)
    hist = np.zeros(33, np.int64)
    fidx_img = r["final_idx"].reshape(h, w)
    for t in pick:
        ty, tx = divmod(int(t), tiles_x)
        _replay_tile(tot, hist, int(bins[t, 0]), int(bins[t, 1]), tx * bw, ty * bw, h, w,
                     s["gaussian_ids_sorted"], xys, con, opac, ex, ey, fidx_img, few_lanes)
    tot["tiles"] = int(pick.size)
    tot["lanes_hist"] = hist
    return tot
