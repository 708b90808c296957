"""splat_batch_layout on the host (no GPU): entry blocks aligned to 256 per
view, tiles and pixels numbered view after view, scene bases, totals, and
the argument checks."""

import ctypes as C

import numpy as np
import pytest


def _layout(points, views, bw=16):
    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    arr = (_lib.SplatView * len(views))()
    for k, (scene, h, w) in enumerate(views):
        arr[k].scene, arr[k].img_height, arr[k].img_width = scene, h, w
        arr[k].fx = arr[k].fy = 100.0
    b = _lib.SplatBatch()
    b.num_scenes, b.num_views, b.block_width = len(points), len(views), bw
    pts = (C.c_uint32 * len(points))(*points)
    rc = lib.splat_batch_layout(C.byref(b), arr, pts)
    return rc, b, arr, lib


def test_layout_bases_and_totals():
    points = [300, 1000, 256]
    views = [(0, 50, 70), (1, 32, 32), (0, 17, 33), (2, 1, 1), (1, 100, 20)]
    rc, b, arr, _ = _layout(points, views, bw=16)
    assert rc == 0
    entry = tile = pix = 0
    gbase = [0, 300, 1300]
    for k, (s, h, w) in enumerate(views):
        v = arr[k]
        assert v.entry_base == entry and v.entry_base % 256 == 0
        assert v.tile_base == tile and v.pixel_base == pix
        assert v.gauss_base == gbase[s] and v.num_points == points[s]
        assert v.tiles_x == (w + 15) // 16 and v.tiles_y == (h + 15) // 16
        entry += (points[s] + 255) // 256 * 256
        tile += v.tiles_x * v.tiles_y
        pix += h * w
    assert (b.num_entries, b.num_tiles, b.num_pixels, b.num_points) == (entry, tile, pix, 1556)


@pytest.mark.parametrize("points,views,bw,msg", [
    ([10], [(1, 8, 8)], 16, b"scene 1 of 1"),
    ([10], [(0, 0, 8)], 16, b"empty image"),
    ([10], [(0, 8, 8)], 17, b"block_width"),
])
def test_layout_rejects_bad_views(points, views, bw, msg):
    rc, _, _, lib = _layout(points, views, bw)
    assert rc == 1
    assert msg in lib.splat_last_error()


def _expected(points, views, bw):
    """Bases and totals recomputed in Python: entries in blocks of 256 per view,
    tiles and pixels view after view, scene bases from the point counts."""
    gbase = np.concatenate([[0], np.cumsum(points)[:-1]]).astype(np.int64)
    entry = tile = pix = 0
    rows = []
    for s, h, w in views:
        tx, ty = (w + bw - 1) // bw, (h + bw - 1) // bw
        rows.append((int(gbase[s]), points[s], tx, ty, entry, tile, pix))
        entry += (points[s] + 255) // 256 * 256
        tile += tx * ty
        pix += h * w
    return rows, (entry, tile, pix, int(sum(points)))


def test_layout_random_batches():
    """200 seeded batches: scene sizes around the 256-entry block (empty scenes
    included), 1-10 views of random scenes and image sizes, every block
    width."""
    rng = np.random.default_rng(11)
    for _ in range(200):
        ns = int(rng.integers(1, 6))
        points = [int(rng.choice([0, 1, 255, 256, 257, int(rng.integers(0, 5000))]))
                  for _ in range(ns)]
        views = [(int(rng.integers(0, ns)), int(rng.integers(1, 300)), int(rng.integers(1, 300)))
                 for _ in range(int(rng.integers(1, 11)))]
        bw = int(rng.integers(2, 17))
        rc, b, arr, lib = _layout(points, views, bw)
        assert rc == 0, lib.splat_last_error()
        rows, totals = _expected(points, views, bw)
        for k, row in enumerate(rows):
            v = arr[k]
            assert (v.gauss_base, v.num_points, v.tiles_x, v.tiles_y, v.entry_base, v.tile_base,
                    v.pixel_base) == row
        assert (b.num_entries, b.num_tiles, b.num_pixels, b.num_points) == totals


@pytest.mark.parametrize("points,views,msg", [
    ([2**31 - 1, 1], [(1, 8, 8)], b"Gaussians in total"),
    ([2**31 - 300, 100], [(0, 8, 8), (0, 8, 8)], b"entries or tiles"),
])
def test_layout_overflow(points, views, msg):
    rc, _, _, lib = _layout(points, views)
    assert rc == 4
    assert msg in lib.splat_last_error()
