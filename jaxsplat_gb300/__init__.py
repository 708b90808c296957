"""jaxsplat_gb300: the jaxsplat Gaussian-splatting render path on GB300.

``render``, ``project`` and ``rasterize`` keep the signatures, keyword
arguments, shapes and differentiable inputs of ``jaxsplat.render``,
``jaxsplat.project`` and ``jaxsplat.rasterize`` (jaxsplat/__init__.py:6-70,
jaxsplat/_project/__init__.py:56-87, jaxsplat/_rasterize/__init__.py:40-68),
on torch CUDA tensors, with torch autograd standing in for jax.custom_vjp.
All compute runs in libsplat.so (hand-written sm_103a CUDA behind the C ABI
of include/splat.h); there is no CPU path.
"""

from __future__ import annotations

import torch

from . import _lib
from ._ops import ProjectFn, RasterizeFn

__all__ = ["render", "project", "rasterize"]


def _kw(img_shape, f, c, glob_scale, clip_thresh, block_width):
    return dict(img_shape=(int(img_shape[0]), int(img_shape[1])), f=(float(f[0]), float(f[1])),
                c=(float(c[0]), float(c[1])), glob_scale=float(glob_scale),
                clip_thresh=float(clip_thresh), block_width=int(block_width))


def project(mean3ds: torch.Tensor, scales: torch.Tensor, quats: torch.Tensor,
            viewmat: torch.Tensor, *, img_shape: tuple[int, int], f: tuple[float, float],
            c: tuple[float, float], glob_scale: float, clip_thresh: float, block_width: int):
    """Project 3D Gaussians to 2D.

    Returns (xys (N,2), depths (N,1), radii (N,1) int32, conics (N,3),
    num_tiles_hit (N,1) int32, cum_tiles_hit (N,1) int32), differentiable with
    respect to mean3ds, scales and quats (jaxsplat/_project/__init__.py:56-87).
    """
    kw = _kw(img_shape, f, c, glob_scale, clip_thresh, block_width)
    xys, depths, radii, conics, nt, cum, _total = ProjectFn.apply(mean3ds, scales, quats,
                                                                   viewmat, kw)
    return xys, depths, radii, conics, nt, cum


def rasterize(colors: torch.Tensor, opacities: torch.Tensor, background: torch.Tensor,
              xys: torch.Tensor, depths: torch.Tensor, radii: torch.Tensor,
              conics: torch.Tensor, cum_tiles_hit: torch.Tensor, *, img_shape: tuple[int, int],
              block_width: int) -> torch.Tensor:
    """Sort and rasterize projected Gaussians into an (H, W, 3) image,
    differentiable with respect to colors, opacities, xys and conics
    (jaxsplat/_rasterize/__init__.py:40-68)."""
    _check_raster(colors, opacities, background, xys, depths, radii, conics, cum_tiles_hit)
    kw = dict(img_shape=(int(img_shape[0]), int(img_shape[1])), block_width=int(block_width))
    img, _alpha, _idx = RasterizeFn.apply(colors, opacities, background, xys, depths, radii,
                                          conics, cum_tiles_hit, None, kw)
    return img


def render(means3d: torch.Tensor, scales: torch.Tensor, quats: torch.Tensor,
           colors: torch.Tensor, opacities: torch.Tensor, *, viewmat: torch.Tensor,
           background: torch.Tensor, img_shape: tuple[int, int], f: tuple[float, float],
           c: tuple[int, int], glob_scale: float, clip_thresh: float,
           block_size: int = 16) -> torch.Tensor:
    """Render 3D Gaussians to an (H, W, 3) image, differentiably with respect
    to means3d, scales, quats, colors and opacities (jaxsplat/__init__.py:6-70).

    quats must be normalised (w, x, y, z); block_size is the tile side,
    1 < block_size <= 16.
    """
    kw = _kw(img_shape, f, c, glob_scale, clip_thresh, block_size)
    xys, depths, radii, conics, _nt, cum, total = ProjectFn.apply(means3d, scales, quats,
                                                                  viewmat, kw)
    _check_raster(colors, opacities, background, xys, depths, radii, conics, cum)
    rkw = dict(img_shape=kw["img_shape"], block_width=kw["block_width"])
    img, _alpha, _idx = RasterizeFn.apply(colors, opacities, background, xys, depths, radii,
                                          conics, cum, total, rkw)
    return img


def _check_raster(colors, opacities, background, xys, depths, radii, conics, cum):
    # jaxsplat/_rasterize/abstract.py:7-24
    n = colors.shape[0]
    for t, shape, dt, name in (
        (colors, (n, 3), torch.float32, "colors"), (opacities, (n, 1), torch.float32, "opacities"),
        (background, (3,), torch.float32, "background"), (xys, (n, 2), torch.float32, "xys"),
        (depths, (n, 1), torch.float32, "depths"), (radii, (n, 1), torch.int32, "radii"),
        (conics, (n, 3), torch.float32, "conics"), (cum, (n, 1), torch.int32, "cum_tiles_hit"),
    ):
        assert tuple(t.shape) == shape and t.dtype == dt, (
            f"{name}: expected {shape} {dt}, got {tuple(t.shape)} {t.dtype}")
        assert t.is_cuda, f"{name}: expected a CUDA tensor"


def library_path() -> str:
    return _lib.LIB_PATH
