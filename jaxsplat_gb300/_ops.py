"""Torch operators over libsplat: the forward/backward pairs behind
``render``, ``project`` and ``rasterize``.

Shapes and dtypes follow the reference's abstract evaluation rules
(jaxsplat/_project/abstract.py:7-77, jaxsplat/_rasterize/abstract.py:7-85);
a mismatch raises AssertionError as the reference's ``Type.assert_`` does
(jaxsplat/_types.py:30-33).  The one dtype difference: num_tiles_hit and
cum_tiles_hit are int32 tensors (the reference declares uint32 but its
kernels write int32; torch has no general uint32 arithmetic).
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib

_status_words: dict[int, torch.Tensor] = {}


def _status_word(device: torch.device) -> torch.Tensor:
    """Per-device uint32 word that kernels OR failure bits into."""
    idx = device.index if device.index is not None else torch.cuda.current_device()
    t = _status_words.get(idx)
    if t is None:
        t = torch.zeros(1, dtype=torch.int32, device=torch.device("cuda", idx))
        _status_words[idx] = t
    return t


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_type(t: torch.Tensor, shape, dtype, name):
    assert tuple(t.shape) == tuple(shape) and t.dtype == dtype, (
        f"{name}: expected {tuple(shape)} {dtype}, got {tuple(t.shape)} {t.dtype}")
    assert t.is_cuda, f"{name}: expected a CUDA tensor"


def _contig(t: torch.Tensor) -> torch.Tensor:
    return t if t.is_contiguous() else t.contiguous()


def _params(num_points, img_shape, f=(0.0, 0.0), c=(0.0, 0.0), glob_scale=0.0,
            clip_thresh=0.0, block_width=16, device=None):
    status = _status_word(device) if device is not None else None
    return _lib.make_params(num_points, img_shape, f, c, glob_scale, clip_thresh, block_width,
                            status.data_ptr() if status is not None else None)


def _workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


# ---------------------------------------------------------------------------
# project

def project_fwd(means3d, scales, quats, viewmat, *, img_shape, f, c, glob_scale, clip_thresh,
                block_width, colors=None, opacities=None, with_cum=True):
    """lib/ops.cu:12-61 -> dict(cov3d, xys, depths, radii, conics, compensation,
    num_tiles_hit, cum_tiles_hit, total); with colors and opacities also the
    packed rasterizer records ("packed", splat_project_fwd_packed), and then
    with_cum=False skips cum_tiles_hit (only the total is formed)."""
    lib = _lib.load()
    n = means3d.shape[0]
    dev = means3d.device
    _check_type(means3d, (n, 3), torch.float32, "means3d")
    _check_type(scales, (n, 3), torch.float32, "scales")
    _check_type(quats, (n, 4), torch.float32, "quats")
    _check_type(viewmat, (4, 4), torch.float32, "viewmat")
    means3d, scales, quats, viewmat = map(_contig, (means3d, scales, quats, viewmat))
    p = _params(n, img_shape, f, c, glob_scale, clip_thresh, block_width, dev)
    f32 = dict(dtype=torch.float32, device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    out = dict(cov3d=torch.empty(n, 6, **f32), xys=torch.empty(n, 2, **f32),
               depths=torch.empty(n, 1, **f32), radii=torch.empty(n, 1, **i32),
               conics=torch.empty(n, 3, **f32), compensation=torch.empty(n, 1, **f32),
               num_tiles_hit=torch.empty(n, 1, **i32), cum_tiles_hit=torch.empty(n, 1, **i32),
               total=torch.empty(1, dtype=torch.int64, device=dev))
    ws = _workspace(lib.splat_project_fwd_workspace_size(C.byref(p)), dev)
    if colors is None:
        rc = lib.splat_project_fwd(
            C.byref(p), _ptr(means3d), _ptr(scales), _ptr(quats), _ptr(viewmat),
            _ptr(out["cov3d"]), _ptr(out["xys"]), _ptr(out["depths"]), _ptr(out["radii"]),
            _ptr(out["conics"]), _ptr(out["compensation"]), _ptr(out["num_tiles_hit"]),
            _ptr(out["cum_tiles_hit"]), _ptr(out["total"]), _ptr(ws), ws.numel(), _stream())
        _lib.check(rc, "project_fwd")
        return out
    _check_type(colors, (n, 3), torch.float32, "colors")
    _check_type(opacities, (n, 1), torch.float32, "opacities")
    colors, opacities = _contig(colors), _contig(opacities)
    out["packed"] = torch.empty(n, 12, **f32)
    rc = lib.splat_project_fwd_packed(
        C.byref(p), _ptr(means3d), _ptr(scales), _ptr(quats), _ptr(viewmat), _ptr(colors),
        _ptr(opacities), _ptr(out["cov3d"]), _ptr(out["xys"]), _ptr(out["depths"]),
        _ptr(out["radii"]), _ptr(out["conics"]), _ptr(out["compensation"]),
        _ptr(out["num_tiles_hit"]), _ptr(out["cum_tiles_hit"]) if with_cum else None,
        _ptr(out["total"]), _ptr(out["packed"]), _ptr(ws), ws.numel(), _stream())
    _lib.check(rc, "project_fwd_packed")
    if not with_cum:
        del out["cum_tiles_hit"]
    return out


def project_bwd(means3d, scales, quats, viewmat, cov3d, radii, conics, compensation, v_xy,
                v_depth, v_conic, v_compensation, *, img_shape, f, c, glob_scale, clip_thresh,
                block_width):
    """lib/ops.cu:63-105 -> dict(v_mean3d, v_scale, v_quat, v_cov2d, v_cov3d)."""
    lib = _lib.load()
    n = means3d.shape[0]
    dev = means3d.device
    p = _params(n, img_shape, f, c, glob_scale, clip_thresh, block_width, dev)
    f32 = dict(dtype=torch.float32, device=dev)
    out = dict(v_mean3d=torch.empty(n, 3, **f32), v_scale=torch.empty(n, 3, **f32),
               v_quat=torch.empty(n, 4, **f32), v_cov2d=torch.empty(n, 3, **f32),
               v_cov3d=torch.empty(n, 6, **f32))
    args = [_contig(t) for t in (means3d, scales, quats, viewmat, cov3d, radii, conics,
                                  compensation, v_xy, v_depth, v_conic, v_compensation)]
    rc = lib.splat_project_bwd(C.byref(p), *[_ptr(t) for t in args], _ptr(out["v_mean3d"]),
                               _ptr(out["v_scale"]), _ptr(out["v_quat"]), _ptr(out["v_cov2d"]),
                               _ptr(out["v_cov3d"]), _stream())
    _lib.check(rc, "project_bwd")
    return out


# ---------------------------------------------------------------------------
# rasterize

def read_counts(num_points, cum_tiles_hit, total=None, device=None):
    """Blocking read of the intersection count (and the device status word)."""
    lib = _lib.load()
    dev = device if device is not None else cum_tiles_hit.device
    p = _params(num_points, (1, 1), device=dev)
    count = C.c_int64(0)
    bits = C.c_uint32(0)
    rc = lib.splat_read_counts(C.byref(p), _ptr(cum_tiles_hit), _ptr(total),
                               _ptr(_status_word(dev)), C.byref(count), C.byref(bits), _stream())
    _lib.check(rc, "read_counts")
    return int(count.value)


def sort_and_bin(num_intersects, xys, depths, radii, cum_tiles_hit, *, img_shape, block_width,
                 intermediates=False, count_dev=None):
    """lib/ops.cu:645-793 -> dict(gaussian_ids_sorted, tile_bins[, isect_ids,
    gaussian_ids, isect_ids_sorted])."""
    lib = _lib.load()
    n = xys.shape[0]
    dev = xys.device
    p = _params(n, img_shape, block_width=block_width, device=dev)
    h, w = img_shape
    ntiles = ((w + block_width - 1) // block_width) * ((h + block_width - 1) // block_width)
    i32 = dict(dtype=torch.int32, device=dev)
    out = dict(gaussian_ids_sorted=torch.empty(num_intersects, **i32),
               tile_bins=torch.empty(ntiles, 2, **i32))
    if intermediates:
        out["isect_ids"] = torch.empty(num_intersects, dtype=torch.int64, device=dev)
        out["gaussian_ids"] = torch.empty(num_intersects, **i32)
        out["isect_ids_sorted"] = torch.empty(num_intersects, dtype=torch.int64, device=dev)
    ws = _workspace(lib.splat_sort_workspace_size(C.byref(p), num_intersects), dev)
    args = [_contig(t) for t in (xys, depths, radii, cum_tiles_hit)]
    rc = lib.splat_sort_and_bin(C.byref(p), num_intersects, _ptr(count_dev),
                                *[_ptr(t) for t in args],
                                _ptr(out["gaussian_ids_sorted"]), _ptr(out["tile_bins"]),
                                _ptr(out.get("isect_ids")), _ptr(out.get("gaussian_ids")),
                                _ptr(out.get("isect_ids_sorted")), _ptr(ws), ws.numel(),
                                _stream())
    _lib.check(rc, "sort_and_bin")
    return out


def pack_splats(xys, conics, colors, opacities, *, img_shape, block_width):
    """(N, 12) packed rasterizer records (include/splat.h splat_pack_splats)."""
    lib = _lib.load()
    n = colors.shape[0]
    dev = colors.device
    p = _params(n, img_shape, block_width=block_width, device=dev)
    packed = torch.empty(n, 12, dtype=torch.float32, device=dev)
    args = [_contig(t) for t in (xys, conics, colors, opacities)]
    rc = lib.splat_pack_splats(C.byref(p), *[_ptr(t) for t in args], _ptr(packed), _stream())
    _lib.check(rc, "pack_splats")
    return packed


def rasterize_fwd(num_intersects, ids_sorted, tile_bins, packed, background, *, img_shape,
                  block_width, count_dev=None, blend=False):
    """lib/ops.cu:144-160 over a sorted list -> dict(final_Ts, final_idx, img)
    [+ blend: the per-slot warp bytes for rasterize_bwd, block width 16]."""
    lib = _lib.load()
    n = packed.shape[0]
    dev = packed.device
    p = _params(n, img_shape, block_width=block_width, device=dev)
    h, w = img_shape
    out = dict(final_Ts=torch.empty(h, w, 1, dtype=torch.float32, device=dev),
               final_idx=torch.empty(h, w, 1, dtype=torch.int32, device=dev),
               img=torch.empty(h, w, 3, dtype=torch.float32, device=dev))
    if blend and block_width == 16:
        out["blend"] = torch.empty(max(1, ids_sorted.numel()), dtype=torch.uint8, device=dev)
    args = [_contig(t) for t in (ids_sorted, tile_bins, packed, background)]
    rc = lib.splat_rasterize_fwd(C.byref(p), num_intersects, _ptr(count_dev),
                                 *[_ptr(t) for t in args],
                                 _ptr(out["final_Ts"]), _ptr(out["final_idx"]), _ptr(out["img"]),
                                 _ptr(out.get("blend")), _stream())
    _lib.check(rc, "rasterize_fwd")
    return out


def rasterize_fwd_l2(num_intersects, ids_sorted, tile_bins, packed, background, target, *,
                     img_shape, block_width, count_dev=None):
    """rasterize_fwd with the L2 loss against `target` fused in (include/splat.h
    splat_rasterize_fwd_l2) -> dict(final_Ts, final_idx, img, v_img, loss)."""
    lib = _lib.load()
    n = packed.shape[0]
    dev = packed.device
    p = _params(n, img_shape, block_width=block_width, device=dev)
    h, w = img_shape
    f32 = dict(dtype=torch.float32, device=dev)
    out = dict(final_Ts=torch.empty(h, w, 1, **f32),
               final_idx=torch.empty(h, w, 1, dtype=torch.int32, device=dev),
               img=torch.empty(h, w, 3, **f32), v_img=torch.empty(h, w, 3, **f32),
               loss=torch.empty(1, **f32))
    _check_type(target, (h, w, 3), torch.float32, "target")
    args = [_contig(t) for t in (ids_sorted, tile_bins, packed, background, target)]
    rc = lib.splat_rasterize_fwd_l2(C.byref(p), num_intersects, _ptr(count_dev),
                                    *[_ptr(t) for t in args], _ptr(out["final_Ts"]),
                                    _ptr(out["final_idx"]), _ptr(out["img"]), _ptr(out["v_img"]),
                                    _ptr(out["loss"]), None, _stream())
    _lib.check(rc, "rasterize_fwd_l2")
    return out


def rasterize_bwd(num_intersects, ids_sorted, tile_bins, packed, background, final_Ts,
                  final_idx, v_img, v_img_alpha, *, img_shape, block_width, with_abs=False,
                  count_dev=None, blend=None):
    """lib/ops.cu:203-225 over the stored sorted list -> dict(v_colors,
    v_opacity, v_xy, v_conic[, v_xy_abs]); `blend`: the forward's per-slot
    warp bytes (rasterize_fwd(..., blend=True)), or None."""
    lib = _lib.load()
    n = packed.shape[0]
    dev = packed.device
    p = _params(n, img_shape, block_width=block_width, device=dev)
    f32 = dict(dtype=torch.float32, device=dev)
    out = dict(v_colors=torch.empty(n, 3, **f32), v_opacity=torch.empty(n, 1, **f32),
               v_xy=torch.empty(n, 2, **f32), v_conic=torch.empty(n, 3, **f32))
    if with_abs:
        out["v_xy_abs"] = torch.empty(n, 2, **f32)
    args = [_contig(t) for t in (ids_sorted, tile_bins, packed, background, final_Ts, final_idx,
                                  v_img, v_img_alpha)]
    rc = lib.splat_rasterize_bwd(C.byref(p), num_intersects, _ptr(count_dev),
                                 *[_ptr(t) for t in args],
                                 _ptr(out["v_colors"]), _ptr(out["v_opacity"]), _ptr(out["v_xy"]),
                                 _ptr(out.get("v_xy_abs")), _ptr(out["v_conic"]), _ptr(blend),
                                 _stream())
    _lib.check(rc, "rasterize_bwd")
    return out


def l2_loss(img, target):
    """mean((img - target)^2) and its cotangent, on the device."""
    lib = _lib.load()
    img, target = _contig(img), _contig(target)
    loss = torch.empty(1, dtype=torch.float32, device=img.device)
    v_img = torch.empty_like(img)
    rc = lib.splat_l2_loss(_ptr(img), _ptr(target), img.numel(), _ptr(loss), _ptr(v_img),
                           _stream())
    _lib.check(rc, "l2_loss")
    return loss, v_img


# ---------------------------------------------------------------------------
# autograd

class ProjectFn(torch.autograd.Function):
    """custom_vjp of jaxsplat/_project/__init__.py:90-205."""

    @staticmethod
    def forward(ctx, means3d, scales, quats, viewmat, kw):
        out = project_fwd(means3d, scales, quats, viewmat, **kw)
        ctx.kw = kw
        ctx.save_for_backward(means3d, scales, quats, viewmat, out["cov3d"], out["radii"],
                              out["conics"], out["compensation"])
        ctx.mark_non_differentiable(out["radii"], out["num_tiles_hit"], out["cum_tiles_hit"],
                                    out["total"])
        return (out["xys"], out["depths"], out["radii"], out["conics"], out["num_tiles_hit"],
                out["cum_tiles_hit"], out["total"])

    @staticmethod
    def backward(ctx, v_xy, v_depth, _r, v_conic, _n, _c, _t):
        means3d, scales, quats, viewmat, cov3d, radii, conics, comp = ctx.saved_tensors
        n = means3d.shape[0]
        z = lambda *s: torch.zeros(*s, dtype=torch.float32, device=means3d.device)  # noqa: E731
        v_xy = v_xy if v_xy is not None else z(n, 2)
        v_depth = v_depth if v_depth is not None else z(n, 1)
        v_conic = v_conic if v_conic is not None else z(n, 3)
        g = project_bwd(means3d, scales, quats, viewmat, cov3d, radii, conics, comp, v_xy,
                        v_depth, v_conic, z(n, 1), **ctx.kw)
        # jaxsplat/_project/__init__.py:200-205: no gradient for viewmat
        return g["v_mean3d"], g["v_scale"], g["v_quat"], None, None


class RasterizeFn(torch.autograd.Function):
    """custom_vjp of jaxsplat/_rasterize/__init__.py:71-190.  The sorted
    intersection list, the packed records and (block width 16) the forward's
    per-slot warp bytes are kept as residuals, so the backward does not
    re-emit and re-sort (lib/ops.cu:188-198 does)."""

    @staticmethod
    def forward(ctx, colors, opacities, background, xys, depths, radii, conics, cum_tiles_hit,
                total, kw):
        n = colors.shape[0]
        count = read_counts(n, cum_tiles_hit, total, device=colors.device)
        s = sort_and_bin(count, xys, depths, radii, cum_tiles_hit, **kw)
        packed = pack_splats(xys, conics, colors, opacities, **kw)
        r = rasterize_fwd(count, s["gaussian_ids_sorted"], s["tile_bins"], packed, background,
                          blend=True, **kw)
        ctx.kw = kw
        ctx.count = count
        blend = r.get("blend", torch.empty(0, dtype=torch.uint8, device=colors.device))
        ctx.save_for_backward(packed, background, r["final_Ts"], r["final_idx"],
                              s["gaussian_ids_sorted"], s["tile_bins"], blend)
        ctx.mark_non_differentiable(r["final_idx"])
        img_alpha = 1.0 - r["final_Ts"]  # jaxsplat/_rasterize/__init__.py:136
        return r["img"], img_alpha, r["final_idx"]

    @staticmethod
    def backward(ctx, v_img, v_img_alpha, _fi):
        packed, background, final_Ts, final_idx, ids, bins, blend = ctx.saved_tensors
        h, w = ctx.kw["img_shape"]
        if v_img is None:
            v_img = torch.zeros(h, w, 3, dtype=torch.float32, device=packed.device)
        if v_img_alpha is None:  # render() drops the alpha image: zero cotangent
            v_img_alpha = torch.zeros(h, w, 1, dtype=torch.float32, device=packed.device)
        g = rasterize_bwd(ctx.count, ids, bins, packed, background, final_Ts, final_idx, v_img,
                          v_img_alpha, blend=blend if blend.numel() else None, **ctx.kw)
        # jaxsplat/_rasterize/__init__.py:187
        return (g["v_colors"], g["v_opacity"], None, g["v_xy"], None, None, g["v_conic"], None,
                None, None)
