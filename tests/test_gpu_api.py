"""The public torch API (render / project / rasterize with autograd), the
legacy XLA custom-call entry points, and the error behaviour (GPU)."""

import ctypes as C

import numpy as np
import pytest

from conftest import GRAD_RTOL, IMG_ATOL, golden_kwargs, load_golden, normwise_rel

pytestmark = pytest.mark.gpu


def _params_t(g, requires_grad=True):
    import torch

    t = {k: torch.from_numpy(np.ascontiguousarray(g["in_" + k])).cuda()
         for k in ("means3d", "scales", "quats", "colors", "opacities", "viewmat", "background",
                   "target")}
    for k in ("means3d", "scales", "quats", "colors", "opacities"):
        t[k].requires_grad_(requires_grad)
    return t


@pytest.mark.parametrize("case", ["tiny_bw16", "tiny_bw12", "gradcheck"])
def test_render_autograd_matches_reference(case):
    import torch

    import jaxsplat_gb300 as js

    g = load_golden(case)
    t = _params_t(g)
    kw = golden_kwargs(g)
    img = js.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                    viewmat=t["viewmat"], background=t["background"],
                    block_size=int(g["block_width"]), **kw)
    assert np.abs(img.detach().cpu().numpy() - g["out_img"]).max() <= IMG_ATOL
    loss = torch.mean((img - t["target"]) ** 2)
    loss.backward()
    for k, gk in (("means3d", "v_mean3d"), ("scales", "v_scale"), ("quats", "v_quat"),
                  ("colors", "v_colors"), ("opacities", "v_opacity")):
        err = normwise_rel(t[k].grad.cpu().numpy(), g["out_" + gk])
        assert err <= GRAD_RTOL, (k, err)


def test_project_and_rasterize_compose_like_render():
    import jaxsplat_gb300 as js

    g = load_golden("tiny_bw16")
    t = _params_t(g, requires_grad=False)
    kw = golden_kwargs(g)
    xys, depths, radii, conics, nt, cum = js.project(t["means3d"], t["scales"], t["quats"],
                                                     t["viewmat"], block_width=16, **kw)
    np.testing.assert_array_equal(cum.cpu().numpy(), g["out_cum_tiles_hit"])
    img = js.rasterize(t["colors"], t["opacities"], t["background"], xys, depths, radii, conics,
                       cum, img_shape=kw["img_shape"], block_width=16)
    assert np.abs(img.cpu().numpy() - g["out_img"]).max() <= IMG_ATOL


def test_shape_mismatch_raises_assertion():
    import torch

    import jaxsplat_gb300 as js

    m = torch.zeros(10, 3, device="cuda")
    with pytest.raises(AssertionError):
        js.project(m, torch.zeros(10, 3, device="cuda"), torch.zeros(10, 3, device="cuda"),
                   torch.eye(4, device="cuda"), img_shape=(8, 8), f=(8.0, 8.0), c=(4.0, 4.0),
                   glob_scale=1.0, clip_thresh=0.01, block_width=16)


def test_legacy_custom_calls_match_reference():
    """splat_xla_* with the reference's buffer order and 80-byte descriptor."""
    import torch

    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    g = load_golden("tiny_bw16")
    kw = golden_kwargs(g)
    n = g["in_means3d"].shape[0]
    h, w = kw["img_shape"]
    dev = "cuda"
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    E = lambda *s, dt=torch.float32: torch.empty(*s, dtype=dt, device=dev)  # noqa: E731

    def call(fn, bufs, desc):
        arr = (C.c_void_p * len(bufs))(*[b.data_ptr() for b in bufs])
        fn(C.c_void_p(torch.cuda.current_stream().cuda_stream), arr, desc, len(desc))
        torch.cuda.synchronize()

    desc = C.create_string_buffer(80)
    assert lib.splat_xla_make_descriptor(n, h, w, *kw["f"], *kw["c"], kw["glob_scale"],
                                         kw["clip_thresh"], 16, desc, 80) == 0
    desc = desc.raw
    ins = [T(g["in_" + k]) for k in ("means3d", "scales", "quats", "viewmat")]
    pout = [E(n, 6), E(n, 2), E(n, 1), E(n, 1, dt=torch.int32), E(n, 3), E(n, 1),
            E(n, 1, dt=torch.int32), E(n, 1, dt=torch.int32)]
    call(lib.splat_xla_project_fwd, ins + pout, desc)
    np.testing.assert_array_equal(pout[7].cpu().numpy(), g["out_cum_tiles_hit"])
    np.testing.assert_array_equal(pout[7 - 4].cpu().numpy(), g["out_radii"])
    cov3d, xys, depths, radii, conics, comp, nt, cum = pout
    rdesc = C.create_string_buffer(80)
    lib.splat_xla_make_descriptor(n, h, w, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 16, rdesc, 80)
    colors, opac, bg = T(g["in_colors"]), T(g["in_opacities"]), T(g["in_background"])
    rout = [E(h, w, 1), E(h, w, 1, dt=torch.int32), E(h, w, 3)]
    call(lib.splat_xla_rasterize_fwd, [colors, opac, bg, xys, depths, radii, conics, cum] + rout,
         rdesc.raw)
    np.testing.assert_array_equal(rout[1].cpu().numpy(), g["out_final_idx"])
    assert np.abs(rout[2].cpu().numpy() - g["out_img"]).max() <= IMG_ATOL
    v_img = T(g["out_v_img"])
    bout = [E(n, 3), E(n, 1), E(n, 2), E(n, 2), E(n, 3)]
    call(lib.splat_xla_rasterize_bwd, [colors, opac, bg, xys, depths, radii, conics, cum,
                                       rout[0], rout[1], v_img, torch.zeros(h, w, 1, device=dev)]
         + bout, rdesc.raw)
    for t_, k in zip(bout, ("v_colors", "v_opacity", "v_xy", "v_xy_abs", "v_conic")):
        assert normwise_rel(t_.cpu().numpy(), g["out_" + k]) <= GRAD_RTOL, k
    z = torch.zeros(n, 1, device=dev)
    jout = [E(n, 3), E(n, 3), E(n, 4), E(n, 3), E(n, 6)]
    call(lib.splat_xla_project_bwd, ins + [cov3d, xys, radii, conics, comp, z, bout[2], z,
                                           bout[4]] + jout, desc)
    for t_, k in zip(jout, ("v_mean3d", "v_scale", "v_quat", "v_cov2d", "v_cov3d")):
        assert normwise_rel(t_.cpu().numpy(), g["out_" + k]) <= GRAD_RTOL, k


def test_workspace_too_small_is_reported():
    import torch

    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    n = 1000
    p = _lib.make_params(n, (64, 64), (64.0, 64.0), (32.0, 32.0), 1.0, 0.01, 16)
    bufs = [torch.zeros(n * 8, device="cuda") for _ in range(13)]
    ws = torch.empty(8, dtype=torch.uint8, device="cuda")
    rc = lib.splat_project_fwd(C.byref(p), *[C.c_void_p(b.data_ptr()) for b in bufs],
                               C.c_void_p(ws.data_ptr()), 8,
                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 3 and b"workspace" in lib.splat_last_error()


def test_bounded_wait_times_out_and_context_survives():
    """A wait on a flag that nothing sets gives up after its poll limit,
    records the timeout bit and returns; the context keeps working."""
    import torch

    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.splat_selftest_wait_timeout(1000, C.c_void_p(status.data_ptr()),
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(status.item()) & 1
    assert float((torch.ones(4, device="cuda") * 2).sum().item()) == 8.0


def test_l2_loss_kernel():
    import torch

    from jaxsplat_gb300 import _ops

    rng = np.random.default_rng(0)
    a = torch.from_numpy(rng.uniform(size=(37, 29, 3)).astype(np.float32)).cuda()
    b = torch.from_numpy(rng.uniform(size=(37, 29, 3)).astype(np.float32)).cuda()
    loss, v = _ops.l2_loss(a, b)
    ref = torch.mean((a - b) ** 2)
    assert abs(float(loss.item()) - float(ref.item())) <= 1e-6
    assert torch.allclose(v, 2 * (a - b) / a.numel(), atol=1e-9)
