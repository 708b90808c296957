"""The 16x16 rasterizers' warp walks, replayed on the CPU over every tile of
small scenes (tests/warp_walks.py): the replayed forward reproduces the
oracle's final_idx, the culling box never drops a contributing pair, and each
backward warp's entries with a valid pixel are exactly the entries the same
warp blended in the forward."""

import numpy as np
import pytest

from warp_walks import walk_stats


@pytest.mark.parametrize("num_points,img_shape,seed", [(20_000, (96, 128), 3),
                                                       (100_000, (64, 80), 4)])
def test_warp_walk_replay(num_points, img_shape, seed):
    from jaxsplat_gb300.scenes import make_scene

    sc = make_scene("small", seed=seed, num_points=num_points, img_shape=img_shape,
                    block_width=16)
    st = walk_stats(sc, threads=2)
    assert st["tiles"] > 0 and st["entries"] > 0
    assert st["final_idx_mismatch"] == 0
    assert st["box_culled_contributing"] == 0
    assert st["identity_mismatch"] == 0
    assert 0 < st["bwd_work"] <= st["bwd_walk"]
    assert 0 < st["fwd_work"] <= st["fwd_walk"]
    assert st["fwd_work"] <= st["fwd_active_pixels"] <= 64 * st["fwd_walk"]
    assert st["tile_contributing"] + st["past_saturation"] <= st["entries"]
    assert st["tile_contributing"] <= st["bwd_staged"] <= st["entries"]
    hist = st["lanes_hist"]
    assert hist[0] == 0 and hist.sum() == st["bwd_work"]
    assert st["bwd_valid_pixels"] >= st["bwd_work"]
    assert np.all(hist >= 0)
