"""Parity of the CUDA path with the reference (GPU).

* against the golden fixtures made by the reference's own kernels: integer
  and index outputs bit-exact, image within 1e-5 absolute, gradients within
  1e-4 relative (normwise);
* against the reference kernels run live on the same inputs (when the
  reference cubins built by oracle/build.py are present), up to the
  1M-Gaussian 1920x1080 scene;
* against the CPU oracle on seeded inputs, including edge cases;
* size-independent properties at full size.
"""

import hashlib

import numpy as np
import pytest

from conftest import (GOLDEN_CASES, GRAD_KEYS, GRAD_RTOL, IMG_ATOL, INT_KEYS, assert_elementwise,
                      golden_kwargs, load_golden, load_small_digests, normwise_rel)

pytestmark = pytest.mark.gpu


def _kw(g):
    return golden_kwargs(g)


def _inputs(g):
    return {k[3:]: g[k] for k in g if k.startswith("in_")}


def assert_parity(out, ref, grads=True, label=""):
    for k in INT_KEYS:
        np.testing.assert_array_equal(out[k], ref[k], err_msg=f"{label} {k}")
    np.testing.assert_array_equal(out["xys"], ref["xys"], err_msg=f"{label} xys")
    np.testing.assert_array_equal(out["depths"], ref["depths"], err_msg=f"{label} depths")
    for k in ("cov3d", "conics", "compensation"):
        assert normwise_rel(out[k], ref[k]) <= 1e-6, f"{label} {k}"
    for k in ("img", "final_Ts"):
        err = float(np.abs(out[k].astype(np.float64) - ref[k]).max())
        assert err <= IMG_ATOL, f"{label} {k}: {err}"
    if grads:
        for k in GRAD_KEYS + ["v_xy_abs", "v_cov2d", "v_cov3d"]:
            if k in out and k in ref:
                err = normwise_rel(out[k], ref[k])
                assert err <= GRAD_RTOL, f"{label} {k}: {err}"
        for k in GRAD_KEYS:
            assert_elementwise(out[k], ref[k], f"{label} {k}")


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_cuda_matches_reference_fixture(case):
    from gpu_pipeline import run_cuda

    g = load_golden(case)
    ref = {k[4:]: g[k] for k in g if k.startswith("out_")}
    out = run_cuda(_inputs(g), _kw(g), int(g["block_width"]), v_img=g["out_v_img"])
    assert_parity(out, ref, label=case)
    # the projection floats come out of the same expressions: report exactness
    exact = {k: bool(np.array_equal(out[k], ref[k])) for k in ("cov3d", "conics", "compensation",
                                                              "img", "final_Ts")}
    print(case, "bit-identical floats:", exact)


def test_cuda_matches_reference_digests_100k():
    from gpu_pipeline import run_cuda
    from make_golden import INPUT_KEYS, spec_inputs

    d = load_small_digests()
    inp = spec_inputs("small", 0)
    for k in INPUT_KEYS:
        if hashlib.sha256(np.ascontiguousarray(inp[k]).tobytes()).hexdigest() != d["inputs_sha256"][k]:
            pytest.skip("seeded inputs differ from the fixture's")
    kw = dict(img_shape=tuple(int(x) for x in inp["img_shape"]), f=tuple(inp["f"]),
              c=tuple(inp["c"]), glob_scale=float(inp["glob_scale"]),
              clip_thresh=float(inp["clip_thresh"]))
    out = run_cuda(inp, kw, 16)
    for k in INT_KEYS + ["xys", "depths"]:
        got = hashlib.sha256(np.ascontiguousarray(out[k]).tobytes()).hexdigest()
        assert got == d["sha256"][k], k
    for k in ("img", "final_Ts"):
        st = d["stats"][k]
        assert abs(float(out[k].astype(np.float64).sum()) - st["sum"]) <= IMG_ATOL * out[k].size


def _ref_or_skip():
    from oracle import ref

    if not ref.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    return ref.RefKernels()


@pytest.mark.parametrize("scene", ["small", "hd"])
def test_cuda_matches_live_reference(scene):
    """Same seeded inputs through the reference's kernels and ours."""
    import torch

    from gpu_pipeline import run_cuda, to_dev
    from jaxsplat_gb300.scenes import make_scene

    rk = _ref_or_skip()
    sc = make_scene(scene, seed=0)
    inp = dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
               opacities=sc.opacities, viewmat=sc.viewmat, background=sc.background)
    kw = sc.kwargs
    t = to_dev(inp)
    fwd = rk.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                    viewmat=t["viewmat"], background=t["background"], block_size=16, **kw)
    target = torch.from_numpy(sc.target).cuda()
    v_img = (2.0 * (fwd["img"] - target) / fwd["img"].numel()).contiguous()
    full = rk.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                     viewmat=t["viewmat"], background=t["background"], block_size=16,
                     v_img=v_img, **kw)
    s = rk.sort_and_bin(full["xys"], full["depths"], full["radii"], full["cum_tiles_hit"],
                        img_shape=kw["img_shape"], block_width=16)
    full.update(s)
    ref = {k: v.cpu().numpy() for k, v in full.items()}
    out = run_cuda(inp, kw, 16, v_img=v_img.cpu().numpy())
    assert_parity(out, ref, label=scene)
    # the per-pixel arithmetic is the reference's: image and transmittance
    # come out bit for bit
    np.testing.assert_array_equal(out["img"], ref["img"])
    np.testing.assert_array_equal(out["final_Ts"], ref["final_Ts"])


def test_cuda_matches_live_reference_uhd():
    """6M Gaussians at 3840x2160 (146M intersections): the reference's
    kernels and ours on the same inputs, compared on the device.  Keys,
    sorted ids, tile bins, radii, tile counts and final_idx bit-exact; image
    and final_Ts within 1e-5; gradients within 1e-4 normwise and the
    element-wise bar.  The backward recomputes each pixel's blend state from
    final_Ts and final_idx in both implementations (backward.cu:153-343)."""
    import time

    import torch

    from gpu_pipeline import run_cuda, to_dev
    from jaxsplat_gb300.scenes import make_scene

    rk = _ref_or_skip()
    t0 = time.perf_counter()
    sc = make_scene("uhd", seed=0)
    inp = dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
               opacities=sc.opacities, viewmat=sc.viewmat, background=sc.background)
    kw = sc.kwargs
    t = to_dev(inp)
    fwd = rk.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                    viewmat=t["viewmat"], background=t["background"], block_size=16, **kw)
    target = torch.from_numpy(sc.target).cuda()
    v_img = (2.0 * (fwd["img"] - target) / fwd["img"].numel()).contiguous()
    del fwd
    ref = rk.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                    viewmat=t["viewmat"], background=t["background"], block_size=16,
                    v_img=v_img, **kw)
    ref.update(rk.sort_and_bin(ref["xys"], ref["depths"], ref["radii"], ref["cum_tiles_hit"],
                               img_shape=kw["img_shape"], block_width=16))
    out = run_cuda(inp, kw, 16, v_img=v_img, device=True)
    torch.cuda.synchronize()
    count = int(out["count"])
    assert count == int(ref["cum_tiles_hit"][-1]) > 100_000_000
    for k in INT_KEYS:
        assert torch.equal(out[k].reshape(ref[k].shape), ref[k]), k
    for k in ("xys", "depths"):
        assert torch.equal(out[k], ref[k]), k
    for k in ("cov3d", "conics", "compensation"):
        err = float((out[k] - ref[k]).abs().max() / ref[k].abs().max())
        assert err <= 1e-6, (k, err)
    for k in ("img", "final_Ts"):
        err = float((out[k].double() - ref[k].double()).abs().max())
        print(f"uhd {k}: max abs err {err:.3g}, bit-identical {bool(torch.equal(out[k], ref[k]))}")
        assert err <= IMG_ATOL, (k, err)
    for k in GRAD_KEYS:
        a, b = out[k].double(), ref[k].double()
        err = float((a - b).abs().max() / b.abs().max())
        print(f"uhd {k}: normwise rel err {err:.3g}")
        assert err <= GRAD_RTOL, (k, err)
        assert_elementwise(out[k], ref[k], f"uhd {k}")
    print(f"uhd: {count} intersections, test {time.perf_counter() - t0:.1f} s")


@pytest.mark.parametrize("scene", ["small", "hd"])
def test_blend_bytes_backward_matches_box_walk(scene):
    """The forward's per-slot warp bytes (bit w: some pixel of 8x8 warp w
    passed the entry) let the backward skip every entry no pixel of a warp
    needs; its gradients equal those of the box-culled walk (a missing bit
    would drop that warp's contributions to the entry)."""
    import torch

    from gpu_pipeline import run_cuda
    from jaxsplat_gb300.scenes import make_scene

    sc = make_scene(scene, seed=2)
    inp = dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
               opacities=sc.opacities, viewmat=sc.viewmat, background=sc.background)
    h, w = sc.kwargs["img_shape"]
    v_img = torch.randn(h, w, 3, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    a = run_cuda(inp, sc.kwargs, 16, v_img=v_img, device=True, blend=True)
    b = run_cuda(inp, sc.kwargs, 16, v_img=v_img, device=True, blend=False)
    assert torch.equal(a["img"], b["img"]) and torch.equal(a["final_idx"], b["final_idx"])
    # the rasterizer's own sums: the same terms, in another atomic order
    for k in ("v_colors", "v_opacity", "v_xy", "v_conic"):
        err = normwise_rel(a[k].cpu().numpy(), b[k].cpu().numpy())
        assert err <= 1e-6, (k, err)
    # the projection backward amplifies that order noise where terms cancel
    for k in ("v_mean3d", "v_scale", "v_quat"):
        assert normwise_rel(a[k].cpu().numpy(), b[k].cpu().numpy()) <= GRAD_RTOL, k
        assert_elementwise(a[k].cpu().numpy(), b[k].cpu().numpy(), f"{scene} blend {k}")


def _oracle_case(o, inp, kw, bw, v_img=None):
    return o.render(inp["means3d"], inp["scales"], inp["quats"], inp["colors"],
                    inp["opacities"], viewmat=inp["viewmat"], background=inp["background"],
                    block_size=bw, v_img=v_img, **kw)


@pytest.mark.parametrize("bw", [2, 5, 8, 12, 16])
@pytest.mark.parametrize("shape", [(1, 1), (17, 33), (45, 70)])
def test_cuda_matches_oracle_edge_shapes(bw, shape):
    from gpu_pipeline import run_cuda
    from jaxsplat_gb300.scenes import make_scene
    from oracle.oracle import Oracle

    sc = make_scene("small", seed=bw * 100 + shape[0], num_points=400, img_shape=shape)
    inp = dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
               opacities=sc.opacities, viewmat=sc.viewmat,
               background=np.asarray([0.3, 0.1, 0.7], np.float32))
    kw = sc.kwargs
    o = Oracle("f32")
    ref = _oracle_case(o, inp, kw, bw)
    v_img = np.random.default_rng(1).normal(size=ref["img"].shape).astype(np.float32)
    ref = _oracle_case(o, inp, kw, bw, v_img=v_img)
    out = run_cuda(inp, kw, bw, v_img=v_img)
    for k in ("radii", "num_tiles_hit", "cum_tiles_hit", "isect_ids", "gaussian_ids_sorted",
              "tile_bins", "final_idx"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    assert np.abs(out["img"] - ref["img"]).max() <= IMG_ATOL
    for k in ("v_colors", "v_opacity", "v_xy", "v_conic", "v_mean3d", "v_scale", "v_quat"):
        assert normwise_rel(out[k], ref[k]) <= GRAD_RTOL, k


@pytest.mark.parametrize("bw,shape", [(16, (320, 400)), (2, (600, 800))])
def test_cuda_matches_oracle_tile_ids_one_bit_past_a_byte(bw, shape):
    """Tile ids of 9 bits (500 tiles) and of 17 bits (120,000 tiles): a last
    radix pass over a single bit sorts like the reference."""
    from gpu_pipeline import run_cuda
    from jaxsplat_gb300.scenes import make_scene
    from oracle.oracle import Oracle

    h, w = shape
    tiles = ((w + bw - 1) // bw) * ((h + bw - 1) // bw)
    bits = (tiles - 1).bit_length()
    assert bits % 8 == 1
    sc = make_scene("small", seed=17 + bw, num_points=3000, img_shape=shape)
    inp = dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
               opacities=sc.opacities, viewmat=sc.viewmat,
               background=np.asarray([0.3, 0.1, 0.7], np.float32))
    kw = sc.kwargs
    ref = _oracle_case(Oracle("f32"), inp, kw, bw)
    out = run_cuda(inp, kw, bw)
    assert int(out["count"]) > 2 * 4096  # several sort partitions
    for k in ("isect_ids", "gaussian_ids_sorted", "tile_bins", "final_idx"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    assert np.abs(out["img"] - ref["img"]).max() <= IMG_ATOL


def test_all_culled_renders_background():
    """No intersections (lib/ops.cu:119-127): image = background, final_Ts =
    final_idx = 0, zero gradients."""
    from gpu_pipeline import run_cuda

    n = 64
    rng = np.random.default_rng(3)
    inp = dict(means3d=np.c_[rng.uniform(-1, 1, (n, 2)), -np.ones(n)].astype(np.float32),
               scales=np.full((n, 3), 0.1, np.float32),
               quats=np.tile(np.asarray([1, 0, 0, 0], np.float32), (n, 1)),
               colors=rng.uniform(size=(n, 3)).astype(np.float32),
               opacities=np.full((n, 1), 0.9, np.float32), viewmat=np.eye(4, dtype=np.float32),
               background=np.asarray([0.25, 0.5, 0.75], np.float32))
    kw = dict(img_shape=(20, 30), f=(30.0, 30.0), c=(15.0, 10.0), glob_scale=1.0,
              clip_thresh=0.01)
    out = run_cuda(inp, kw, 16, v_img=np.ones((20, 30, 3), np.float32))
    assert int(out["count"]) == 0
    np.testing.assert_array_equal(out["img"], np.broadcast_to(inp["background"], (20, 30, 3)))
    assert (out["final_Ts"] == 0).all() and (out["final_idx"] == 0).all()
    for k in ("v_colors", "v_opacity", "v_xy", "v_conic", "v_mean3d"):
        assert (out[k] == 0).all(), k


def test_no_gaussians_renders_background():
    """N = 0 through the public render API: the background image, and a
    backward pass that completes with empty gradients."""
    import torch

    import jaxsplat_gb300 as js

    dev = "cuda"
    params = [torch.zeros(0, k, device=dev, requires_grad=True) for k in (3, 3, 4, 3, 1)]
    bg = torch.tensor([0.25, 0.5, 0.75], device=dev)
    img = js.render(*params, viewmat=torch.eye(4, device=dev), background=bg, img_shape=(20, 30),
                    f=(30.0, 30.0), c=(15.0, 10.0), glob_scale=1.0, clip_thresh=0.01)
    assert tuple(img.shape) == (20, 30, 3)
    assert torch.equal(img, bg.expand(20, 30, 3))
    img.sum().backward()
    torch.cuda.synchronize()
    for t in params:
        assert t.grad is None or t.grad.numel() == 0


def test_single_gaussian():
    from gpu_pipeline import run_cuda
    from oracle.oracle import Oracle

    inp = dict(means3d=np.asarray([[0.1, -0.05, 3.0]], np.float32),
               scales=np.asarray([[0.2, 0.1, 0.05]], np.float32),
               quats=np.asarray([[0.9, 0.1, 0.3, -0.2]], np.float32) / np.float32(0.9695),
               colors=np.asarray([[0.9, 0.5, 0.1]], np.float32),
               opacities=np.asarray([[0.8]], np.float32), viewmat=np.eye(4, dtype=np.float32),
               background=np.zeros(3, np.float32))
    kw = dict(img_shape=(40, 50), f=(40.0, 40.0), c=(25.0, 20.0), glob_scale=1.0,
              clip_thresh=0.01)
    v_img = np.ones((40, 50, 3), np.float32)
    ref = _oracle_case(Oracle("f32"), inp, kw, 16, v_img=v_img)
    out = run_cuda(inp, kw, 16, v_img=v_img)
    np.testing.assert_array_equal(out["gaussian_ids_sorted"], ref["gaussian_ids_sorted"])
    np.testing.assert_array_equal(out["final_idx"], ref["final_idx"])
    assert np.abs(out["img"] - ref["img"]).max() <= IMG_ATOL
    assert normwise_rel(out["v_mean3d"], ref["v_mean3d"]) <= GRAD_RTOL


@pytest.mark.parametrize("scene", ["hd", "uhd"])
def test_full_size_properties(scene):
    """1M Gaussians at 1920x1080 and 6M at 3840x2160: sortedness, stability,
    bin coverage, index ranges (checked on the device)."""
    import torch

    from gpu_pipeline import to_dev
    from jaxsplat_gb300 import _ops
    from jaxsplat_gb300.scenes import make_scene

    sc = make_scene(scene, seed=1)
    kw = sc.kwargs
    t = to_dev(dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
                    opacities=sc.opacities, viewmat=sc.viewmat, background=sc.background))
    n = sc.spec.num_points
    p = _ops.project_fwd(t["means3d"], t["scales"], t["quats"], t["viewmat"], block_width=16, **kw)
    count = _ops.read_counts(n, p["cum_tiles_hit"], p["total"], device=t["means3d"].device)
    assert count == int(p["num_tiles_hit"].sum().item()) == int(p["cum_tiles_hit"][-1].item())
    s = _ops.sort_and_bin(count, p["xys"], p["depths"], p["radii"], p["cum_tiles_hit"],
                          img_shape=kw["img_shape"], block_width=16, intermediates=True)
    keys = s["isect_ids_sorted"]
    ids = s["gaussian_ids_sorted"].long()
    assert bool((keys[1:] >= keys[:-1]).all())
    ties = keys[1:] == keys[:-1]
    assert bool((ids[1:][ties] > ids[:-1][ties]).all())  # stable: emission order on ties
    # a permutation of the emission
    emitted = torch.sort(s["gaussian_ids"].long() * (1 << 33) + (s["isect_ids"] >> 32))[0]
    resorted = torch.sort(ids * (1 << 33) + (keys >> 32))[0]
    assert bool((emitted == resorted).all())
    bins = s["tile_bins"].long()
    lens = (bins[:, 1] - bins[:, 0]).clamp(min=0)
    assert int(lens.sum().item()) == count
    tile_of = (keys >> 32)
    starts = bins[:, 0][lens > 0]
    assert bool((tile_of[starts] == torch.nonzero(lens > 0).ravel()).all())
    packed = _ops.pack_splats(p["xys"], p["conics"], t["colors"], t["opacities"],
                              img_shape=kw["img_shape"], block_width=16)
    r = _ops.rasterize_fwd(count, s["gaussian_ids_sorted"], s["tile_bins"], packed,
                           t["background"], img_shape=kw["img_shape"], block_width=16)
    assert bool(torch.isfinite(r["img"]).all())
    assert int(r["final_idx"].min().item()) >= 0 and int(r["final_idx"].max().item()) < count
    assert float(r["final_Ts"].min().item()) >= 0.0 and float(r["final_Ts"].max().item()) <= 1.0
