"""Size-independent properties of the sort/bin/scan stages, on the oracle
(CPU).  The same properties are checked on the CUDA path at full size in
test_gpu_parity.py."""

import numpy as np
import pytest

from oracle.oracle import Oracle


@pytest.fixture(scope="module")
def o32():
    return Oracle("f32")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_sort_is_stable_permutation(o32, seed):
    rng = np.random.default_rng(seed)
    n = 5000
    tiles = rng.integers(0, 37, n, dtype=np.int64)
    depth_bits = rng.choice(np.array([0x40000000, 0x40400000, 0x40800000], np.int64), n)
    keys = (tiles << 32) | depth_bits
    vals = np.arange(n, dtype=np.int32)
    end_bit = o32.sort_end_bit(37)
    ks, vs = o32.sort_pairs(keys, vals, end_bit)
    mask = (1 << end_bit) - 1
    order = np.argsort(keys & mask, kind="stable")
    np.testing.assert_array_equal(vs, vals[order])
    np.testing.assert_array_equal(ks, keys[order])
    assert np.all(np.diff(ks & mask) >= 0)


def test_sort_end_bit_matches_reference_rule(o32):
    # lib/ops.cu:723-724: 32 + (32 - clz(T)) + 1
    for t, want in [(1, 34), (256, 42), (8160, 46), (32400, 48), (64, 40)]:
        assert o32.sort_end_bit(t) == want


def test_bins_partition_the_sorted_list(o32):
    rng = np.random.default_rng(7)
    n_tiles = 50
    tiles = np.sort(rng.choice(np.arange(n_tiles), 3000))
    tiles = tiles[tiles != 13]  # one empty tile in the middle
    keys = (tiles.astype(np.int64) << 32) | 0x3f800000
    bins = o32.tile_bin_edges(keys, n_tiles)
    nonempty = bins[:, 1] > bins[:, 0]
    assert (bins[~nonempty] == 0).all()  # empty tiles stay (0, 0)
    assert int((bins[:, 1] - bins[:, 0]).sum()) == keys.size
    for t in np.nonzero(nonempty)[0]:
        assert (tiles[bins[t, 0]:bins[t, 1]] == t).all()


def test_scan_and_emission_consistent(o32):
    from jaxsplat_gb300.scenes import make_scene

    sc = make_scene("small", seed=5, num_points=3000, img_shape=(96, 160))
    kw = sc.kwargs
    p = o32.project_fwd(sc.means3d, sc.scales, sc.quats, sc.viewmat, block_width=16, **kw)
    cum = p["cum_tiles_hit"].ravel()
    assert np.all(np.diff(cum) >= 0)
    assert cum[-1] == p["num_tiles_hit"].sum()
    assert ((p["radii"] > 0) == (p["num_tiles_hit"] > 0)).all()
    keys, ids = o32.map_intersects(p["xys"], p["depths"], p["radii"], p["cum_tiles_hit"],
                                   img_shape=kw["img_shape"], block_width=16)
    assert keys.size == cum[-1]
    np.testing.assert_array_equal(np.bincount(ids, minlength=3000), p["num_tiles_hit"].ravel())
