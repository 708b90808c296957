"""The fused entry points against their unfused pairs, on the same inputs:
splat_project_fwd_packed = splat_project_fwd + splat_pack_splats (every output
bit-identical), splat_rasterize_fwd_l2 = splat_rasterize_fwd + splat_l2_loss
(image, final_Ts, final_idx and v_img bit-identical; the loss, summed in a
different order, within 1e-6 relative).  Block widths 16, 12 (a partial last
warp) and 5 (a block smaller than a warp)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(bw):
    from jaxsplat_gb300.scenes import make_scene

    return make_scene("small", seed=11, num_points=20_000, img_shape=(90, 130), block_width=bw)


@pytest.mark.parametrize("bw", [16, 12, 5])
def test_fused_projection_and_forward_loss(bw):
    import torch

    from jaxsplat_gb300 import _ops

    sc = _scene(bw)
    kw = sc.kwargs
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(sc, k), np.float32)).cuda()
         for k in ("means3d", "scales", "quats", "colors", "opacities", "viewmat", "background",
                   "target")}
    proj_kw = dict(img_shape=kw["img_shape"], f=kw["f"], c=kw["c"], glob_scale=kw["glob_scale"],
                   clip_thresh=kw["clip_thresh"], block_width=bw)
    a = _ops.project_fwd(t["means3d"], t["scales"], t["quats"], t["viewmat"], **proj_kw)
    b = _ops.project_fwd(t["means3d"], t["scales"], t["quats"], t["viewmat"], **proj_kw,
                         colors=t["colors"], opacities=t["opacities"])
    packed = _ops.pack_splats(a["xys"], a["conics"], t["colors"], t["opacities"],
                              img_shape=kw["img_shape"], block_width=bw)
    for k in a:
        assert torch.equal(a[k], b[k]), k
    assert torch.equal(packed.view(torch.int32), b["packed"].view(torch.int32))
    # without cum_tiles_hit: the same outputs and the same total
    c = _ops.project_fwd(t["means3d"], t["scales"], t["quats"], t["viewmat"], **proj_kw,
                         colors=t["colors"], opacities=t["opacities"], with_cum=False)
    assert "cum_tiles_hit" not in c
    for k in c:
        assert torch.equal(b[k], c[k]), k

    n = sc.spec.num_points
    count = _ops.read_counts(n, a["cum_tiles_hit"], a["total"], device=t["means3d"].device)
    assert count > 0
    s = _ops.sort_and_bin(count, a["xys"], a["depths"], a["radii"], a["cum_tiles_hit"],
                          img_shape=kw["img_shape"], block_width=bw)
    r = _ops.rasterize_fwd(count, s["gaussian_ids_sorted"], s["tile_bins"], packed,
                           t["background"], img_shape=kw["img_shape"], block_width=bw)
    loss, v_img = _ops.l2_loss(r["img"], t["target"])
    f = _ops.rasterize_fwd_l2(count, s["gaussian_ids_sorted"], s["tile_bins"], packed,
                              t["background"], t["target"], img_shape=kw["img_shape"],
                              block_width=bw)
    for k in ("img", "final_Ts", "final_idx"):
        assert torch.equal(r[k], f[k]), k
    assert torch.equal(v_img, f["v_img"])
    ref = float(((r["img"].double() - t["target"].double()) ** 2).mean())
    assert abs(float(f["loss"]) - ref) <= 1e-6 * ref
    assert abs(float(f["loss"]) - float(loss)) <= 1e-6 * ref


def test_fused_forward_loss_without_intersections():
    """No Gaussian in view: the image is the background and the loss is
    taken against it (lib/ops.cu:119-127)."""
    import torch

    from jaxsplat_gb300 import _ops

    h, w = 40, 56
    n = 8
    packed = torch.zeros(n, 12, device="cuda")
    bins = torch.zeros((w + 15) // 16 * ((h + 15) // 16), 2, dtype=torch.int32, device="cuda")
    ids = torch.zeros(1, dtype=torch.int32, device="cuda")
    bg = torch.tensor([0.2, 0.4, 0.6], device="cuda")
    target = torch.rand(h, w, 3, device="cuda", generator=torch.Generator("cuda").manual_seed(3))
    f = _ops.rasterize_fwd_l2(0, ids, bins, packed, bg, target, img_shape=(h, w), block_width=16)
    assert torch.equal(f["img"], bg.expand(h, w, 3))
    loss, v_img = _ops.l2_loss(f["img"], target)
    assert torch.equal(v_img, f["v_img"])
    assert abs(float(f["loss"]) - float(loss)) <= 1e-6 * float(loss)


def test_fused_batch_projection_matches_projection_and_pack():
    """splat_batch_project_fwd_packed = splat_batch_project_fwd +
    splat_batch_pack, padding entries included, bit for bit."""
    import torch

    from jaxsplat_gb300.batch import BatchSession
    from jaxsplat_gb300.scenes import make_batch

    scenes, views, targets = make_batch(4, scene_points=(1500, 2600), views_per_scene=2,
                                        sizes=((40, 56), (72, 48)))
    bs = BatchSession(scenes, views, targets, block_size=16)
    bs._project(pack=False)
    import ctypes

    rc = bs.lib.splat_batch_pack(ctypes.byref(bs.batch),
                                 *(bs._p(t) for t in (bs.xys, bs.conics, bs.colors,
                                                      bs.opacities, bs.packed)), bs._stream())
    assert rc == 0
    ref = {k: getattr(bs, k).clone() for k in ("packed", "xys", "conics", "cov3d", "depths",
                                                "radii", "comp", "total")}
    for k in ("packed", "xys", "conics"):
        getattr(bs, k).fill_(-7.0)
    bs._project(pack=True)
    for k, v in ref.items():
        assert torch.equal(v.view(torch.int32) if v.is_floating_point() else v,
                           getattr(bs, k).view(torch.int32) if v.is_floating_point()
                           else getattr(bs, k)), k
