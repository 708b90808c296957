"""Batched multi-view, multi-scene render (BatchSession): every view's image,
final_Ts and final_idx match the reference's kernels rendering that view
alone (one call per view, jaxsplat/__init__.py:6-70), and each scene's
gradients match the sum of the reference's per-view gradients; every view
also equals this library's single-view render of that view bit for bit;
per-entry screen-space gradients equal the view's own; scene gradients equal
the sum over the scene's views of the single-view gradients; graph replay
equals eager; capacity overflow is reported."""

import numpy as np
import pytest

from conftest import GRAD_RTOL, IMG_ATOL, assert_elementwise, normwise_rel

pytestmark = pytest.mark.gpu

SIZES = ((48, 64), (80, 96), (70, 50), (33, 17))


def _batch(bw, points=(3000, 5000), views_per_scene=3, seed=3):
    from jaxsplat_gb300.batch import BatchSession
    from jaxsplat_gb300.scenes import make_batch

    scenes, views, targets = make_batch(seed, scene_points=points, views_per_scene=views_per_scene,
                                        sizes=SIZES)
    views[1]["background"] = np.array([0.2, 0.5, 0.9], np.float32)
    bs = BatchSession(scenes, views, targets, block_size=bw)
    return bs, scenes, views, targets


def _single(scene, view, target, bw):
    from jaxsplat_gb300.session import RenderSession

    h, w = view["img_shape"]
    n = scene["means3d"].shape[0]
    s = RenderSession(n, img_shape=(h, w), f=view["f"], c=view["c"], glob_scale=1.0,
                      clip_thresh=0.01, block_size=bw)
    s.set_inputs(scene["means3d"], scene["scales"], scene["quats"], scene["colors"],
                 scene["opacities"], view["viewmat"], view.get("background", np.zeros(3)), target)
    s.measure_capacity()
    s.step()
    s.check()
    return s


@pytest.mark.parametrize("bw", [16, 8, 12])
def test_batch_views_match_single_view_renders(bw):
    import torch

    bs, scenes, views, targets = _batch(bw)
    bs.measure_capacity()
    bs.step()
    bs.check()
    sums = [None] * len(scenes)
    loss = 0.0
    lengths = (bs.tile_bins[:, 1] - bs.tile_bins[:, 0]).long()
    for k, v in enumerate(views):
        s = _single(scenes[v["scene"]], v, targets[k], bw)
        Ts, idx = bs.view_final(k)
        torch.testing.assert_close(bs.view_image(k), s.img, rtol=0, atol=0)
        torch.testing.assert_close(Ts, s.final_Ts, rtol=0, atol=0)
        # the loss cotangent from the fused epilogue, per view
        b0, h, w = bs._pix(k)
        torch.testing.assert_close(bs.v_img[b0:b0 + h * w].reshape(h, w, 3), s.v_img, rtol=0,
                                   atol=0)
        # final_idx indexes the batch's list: the view's own index plus the
        # intersections of the views before it, for pixels with a contributor
        off = int(lengths[:bs.views_host[k].tile_base].sum())
        expect = torch.where(s.final_Ts < 1.0, s.final_idx + off, torch.zeros_like(s.final_idx))
        torch.testing.assert_close(idx, expect, rtol=0, atol=0)
        e = bs.view_entries(k)
        for name, a, b in (("v_xy", bs.v_xy[e], s.v_xy), ("v_conic", bs.v_conic[e], s.v_conic)):
            assert normwise_rel(a.cpu().numpy(), b.cpu().numpy()) <= 1e-5, (k, name)
        g = {kk: vv.detach().cpu().numpy().astype(np.float64) for kk, vv in s.grads.items()}
        sc = v["scene"]
        sums[sc] = g if sums[sc] is None else {kk: sums[sc][kk] + g[kk] for kk in g}
        loss += float(s.loss.item())
    for sc in range(len(scenes)):
        got = bs.scene_grads(sc)
        for name in ("means3d", "scales", "quats", "colors", "opacities"):
            assert normwise_rel(got[name].cpu().numpy(), sums[sc][name]) <= 1e-5, (sc, name)
    assert abs(float(bs.loss.item()) - loss) <= 1e-5 * max(1.0, loss)


REF_SIZES = ((128, 128), (90, 160), (108, 192))  # 512^2, 1280x720, 1920x1080 scaled down


@pytest.mark.parametrize("bw,sizes", [(16, REF_SIZES), (8, REF_SIZES), (12, REF_SIZES),
                                      (8, ((720, 1280),))])
def test_batch_views_match_reference(bw, sizes):
    """Four scenes of a few thousand Gaussians, two views each, mixed image
    sizes: the batch against the reference's kernels, one call per view.
    The last case has eight 1280x720 views at 8x8 tiles, 115,200 tiles in
    all: 17-bit tile ids, sorted in three passes (8 + 8 + 1 bits), one view's
    tiles on both sides of 2^16."""
    import torch

    from oracle import ref
    from jaxsplat_gb300.batch import BatchSession
    from jaxsplat_gb300.scenes import make_batch

    if not ref.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    rk = ref.RefKernels()
    scenes, views, targets = make_batch(11, scene_points=(2000, 3000, 4000, 6000),
                                        views_per_scene=2, sizes=sizes)
    views[3]["background"] = np.array([0.2, 0.5, 0.9], np.float32)
    bs = BatchSession(scenes, views, targets, block_size=bw)
    bs.measure_capacity()
    bs.step()
    bs.check()
    if len(sizes) == 1:  # 17-bit tile ids
        assert 1 << 16 < int(bs.batch.num_tiles) <= 1 << 17
    lengths = (bs.tile_bins[:, 1] - bs.tile_bins[:, 0]).long()
    sums = [None] * len(scenes)
    loss = 0.0
    bit_identical = True
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()  # noqa: E731
    for k, v in enumerate(views):
        sc = scenes[v["scene"]]
        h, w = v["img_shape"]
        kw = dict(img_shape=(h, w), f=v["f"], c=v["c"], glob_scale=1.0, clip_thresh=0.01)
        args = [dev(sc[n]) for n in ("means3d", "scales", "quats", "colors", "opacities")]
        vm, bg, tgt = dev(v["viewmat"]), dev(v["background"]), dev(targets[k])
        fwd = rk.render(*args, viewmat=vm, background=bg, block_size=bw, **kw)
        v_img = (2.0 * (fwd["img"] - tgt) / fwd["img"].numel()).contiguous()
        r = rk.render(*args, viewmat=vm, background=bg, block_size=bw, v_img=v_img, **kw)
        loss += float(torch.mean((fwd["img"] - tgt) ** 2))
        assert int(r["cum_tiles_hit"][-1]) > 0, k
        img = bs.view_image(k)
        Ts, idx = bs.view_final(k)
        for name, a, b in (("img", img, r["img"]), ("final_Ts", Ts, r["final_Ts"])):
            err = float((a.double() - b.double()).abs().max())
            assert err <= IMG_ATOL, (k, name, err)
            bit_identical &= bool(torch.equal(a, b))
        off = int(lengths[:bs.views_host[k].tile_base].sum())
        expect = torch.where(r["final_Ts"] < 1.0, r["final_idx"] + off,
                             torch.zeros_like(r["final_idx"]))
        assert torch.equal(idx, expect), k
        e = bs.view_entries(k)
        for name in ("v_xy", "v_conic"):
            err = normwise_rel(getattr(bs, name)[e].cpu().numpy(), r[name].cpu().numpy())
            assert err <= GRAD_RTOL, (k, name, err)
        g = dict(means3d=r["v_mean3d"], scales=r["v_scale"], quats=r["v_quat"],
                 colors=r["v_colors"], opacities=r["v_opacity"])
        g = {n: t.double().cpu().numpy() for n, t in g.items()}
        sums[v["scene"]] = g if sums[v["scene"]] is None else \
            {n: sums[v["scene"]][n] + g[n] for n in g}
    for s in range(len(scenes)):
        got = bs.scene_grads(s)
        for name in ("means3d", "scales", "quats", "colors", "opacities"):
            a = got[name].detach().cpu().numpy()
            assert normwise_rel(a, sums[s][name]) <= GRAD_RTOL, (s, name)
            assert_elementwise(a, sums[s][name], f"bw{bw} scene {s} {name}")
    # the batch's loss is an fp32 sum of per-tile atomics over every pixel of
    # every view: its rounding grows with the pixel count (7.4M in the
    # 1280x720 case, ~0.1M in the others)
    npix = sum(int(h) * int(w) for h, w in (v["img_shape"] for v in views))
    assert abs(float(bs.loss.item()) - loss) <= 1e-5 * max(1.0, loss) * max(1.0, npix / 1e6)
    print(f"bw {bw}: every view's image and final_Ts bit-identical to the reference's: "
          f"{bit_identical}")


def test_batch_graph_replay_matches_eager():
    import torch

    bs, *_ = _batch(16, (4000, 2500, 1000), 2)
    bs.chunk = 3
    bs.measure_capacity()
    bs.step()
    eager = bs.img.clone()
    grads = {k: v.clone() for k, v in bs.scene_grads(0).items()}
    count = bs.check()
    bs.capture()
    bs.replay()
    bs.replay()
    assert bs.check() == count
    torch.testing.assert_close(bs.img, eager, rtol=0, atol=0)
    for k, v in bs.scene_grads(0).items():
        assert normwise_rel(v.cpu().numpy(), grads[k].cpu().numpy()) <= 1e-5, k


def test_batch_capacity_overflow_is_reported():
    from jaxsplat_gb300._lib import SplatError

    bs, *_ = _batch(16)
    bs._size(500)
    bs.step()
    with pytest.raises(SplatError, match="capacity-exceeded"):
        bs.check()


def test_batch_autotune_picks_a_measured_config():
    bs, *_ = _batch(16, (2000, 3000), 2)
    res = bs.autotune(block_sizes=(8, 16), chunks=(1, 4), steps=1)
    assert set(res) == {(8, 1), (8, 4), (16, 1), (16, 4)}
    assert bs.best == min(res, key=res.get)
    assert bs.bw == bs.best[0] and bs.chunk == bs.best[1]
    bs.replay()
    bs.check()


def test_batch_step_io_matches_device_step():
    import torch

    bs, *_ = _batch(16, (3000, 2000), 2)
    bs.measure_capacity()
    host_in = bs.inputs.cpu().pin_memory()
    host_out = torch.empty(bs.outputs.numel(), dtype=torch.float32, pin_memory=True)
    bs.capture_io(host_in, host_out)
    host_out.fill_(float("nan"))
    bs.replay_io()
    torch.cuda.synchronize()
    got = host_out.clone()
    bs.step()
    torch.cuda.synchronize()
    ref = bs.outputs.cpu()
    assert abs(float(got[0]) - float(ref[0])) <= 1e-6 * max(1.0, abs(float(ref[0])))
    assert normwise_rel(got.numpy(), ref.numpy()) <= 1e-5


def test_batch_stream_step_matches_step_io_for_each_input():
    """BatchSession.stream_step: consecutive steps alternating two input
    blocks return what step_io returns for each."""
    import torch

    bs, *_ = _batch(16, (3000, 2000), 2)
    bs.measure_capacity()
    host_a = bs.inputs.cpu().pin_memory()
    host_b = host_a.clone().pin_memory()
    tgt = bs.target.data_ptr() - bs.inputs.data_ptr()
    host_b[tgt // 4:] *= 0.5  # the targets
    n_out = bs.outputs.numel()
    refs = []
    for h in (host_a, host_b):
        out = torch.empty(n_out, dtype=torch.float32, pin_memory=True)
        bs.step_io(h, out)
        torch.cuda.synchronize()
        refs.append(out.clone())
    assert float(refs[0][0]) != float(refs[1][0])
    outs = [torch.full((n_out,), float("nan"), pin_memory=True) for _ in range(4)]
    for i in range(4):
        bs.stream_step((host_a, host_b)[i % 2], outs[i])
    bs.stream_sync()
    torch.cuda.synchronize()
    for i in range(4):
        ref = refs[i % 2]
        assert abs(float(outs[i][0]) - float(ref[0])) <= 1e-6 * max(1.0, abs(float(ref[0]))), i
        assert normwise_rel(outs[i].numpy(), ref.numpy()) <= 1e-5, i
