"""Python driver for the reference's own kernels (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/libref_harness.so, which loads the reference kernels
built from its sources into oracle/_ref/*.cubin, and exposes the reference's
four custom calls (lib/ops.h:45-92, buffers in the operand-then-result order
of jaxsplat/_{project,rasterize}/lowering.py) on torch CUDA tensors, plus the
sort/bin intermediates.  ``render_step`` chains them the way jax.grad of an L2
loss over jaxsplat.render dispatches them (jaxsplat/__init__.py:44-68, the
custom_vjp backward of jaxsplat/_rasterize/__init__.py:155-187 and
jaxsplat/_project/__init__.py:155-205).
"""

from __future__ import annotations

import ctypes as C
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_build", "libref_harness.so")
CUBINS = os.path.join(HERE, "_ref")


def available() -> bool:
    return os.path.exists(HARNESS) and all(
        os.path.exists(os.path.join(CUBINS, f"{n}.cubin")) for n in ("forward", "backward", "other"))


class RefKernels:
    def __init__(self):
        if not available():
            raise RuntimeError("reference kernels not built (oracle/_ref cubins or harness missing)")
        self.lib = C.CDLL(HARNESS)
        self.lib.ref_last_error.restype = C.c_char_p
        for fn in ("ref_xla_project_fwd", "ref_xla_project_bwd", "ref_xla_rasterize_fwd",
                   "ref_xla_rasterize_bwd"):
            getattr(self.lib, fn).argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_char_p,
                                              C.c_size_t]
        self.lib.ref_stage_sort_and_bin.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t,
                                                    C.c_uint] + [C.c_void_p] * 9
        self.lib.ref_make_descriptor.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_float,
                                                 C.c_float, C.c_float, C.c_float, C.c_float,
                                                 C.c_float, C.c_uint, C.c_void_p]
        torch.cuda.init()
        self._check(self.lib.ref_load(CUBINS.encode()))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference harness: " + self.lib.ref_last_error().decode())

    def descriptor(self, num_points, img_shape, f=(0.0, 0.0), c=(0.0, 0.0), glob_scale=0.0,
                   clip_thresh=0.0, block_width=16) -> bytes:
        """lib/ffi.cu:15-52 (the rasterize lowering passes zeros for f, c,
        glob_scale and clip_thresh, jaxsplat/_rasterize/lowering.py:28-36)."""
        buf = C.create_string_buffer(80)
        h, w = img_shape
        self.lib.ref_make_descriptor(num_points, h, w, f[0], f[1], c[0], c[1], glob_scale,
                                     clip_thresh, block_width, buf)
        return buf.raw

    def _call(self, fn, tensors, desc):
        arr = (C.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])
        stream = torch.cuda.current_stream().cuda_stream
        self._check(fn(C.c_void_p(stream), arr, desc, len(desc)))

    def project_fwd(self, means3d, scales, quats, viewmat, *, img_shape, f, c, glob_scale,
                    clip_thresh, block_width):
        n = means3d.shape[0]
        dev = means3d.device
        fz = lambda *s: torch.empty(*s, dtype=torch.float32, device=dev)  # noqa: E731
        iz = lambda *s: torch.empty(*s, dtype=torch.int32, device=dev)  # noqa: E731
        out = dict(cov3d=fz(n, 6), xys=fz(n, 2), depths=fz(n, 1), radii=iz(n, 1),
                   conics=fz(n, 3), compensation=fz(n, 1), num_tiles_hit=iz(n, 1),
                   cum_tiles_hit=iz(n, 1))
        desc = self.descriptor(n, img_shape, f, c, glob_scale, clip_thresh, block_width)
        self._call(self.lib.ref_xla_project_fwd, [means3d, scales, quats, viewmat, *out.values()],
                   desc)
        return out

    def rasterize_fwd(self, colors, opacities, background, xys, depths, radii, conics,
                      cum_tiles_hit, *, img_shape, block_width):
        h, w = img_shape
        dev = colors.device
        out = dict(final_Ts=torch.empty(h, w, 1, device=dev),
                   final_idx=torch.empty(h, w, 1, dtype=torch.int32, device=dev),
                   img=torch.empty(h, w, 3, device=dev))
        desc = self.descriptor(colors.shape[0], img_shape, block_width=block_width)
        self._call(self.lib.ref_xla_rasterize_fwd,
                   [colors, opacities, background, xys, depths, radii, conics, cum_tiles_hit,
                    out["final_Ts"], out["final_idx"], out["img"]], desc)
        return out

    def rasterize_bwd(self, colors, opacities, background, xys, depths, radii, conics,
                      cum_tiles_hit, final_Ts, final_idx, v_img, v_img_alpha, *, img_shape,
                      block_width):
        n = colors.shape[0]
        dev = colors.device
        out = dict(v_colors=torch.empty(n, 3, device=dev), v_opacity=torch.empty(n, 1, device=dev),
                   v_xy=torch.empty(n, 2, device=dev), v_xy_abs=torch.empty(n, 2, device=dev),
                   v_conic=torch.empty(n, 3, device=dev))
        desc = self.descriptor(n, img_shape, block_width=block_width)
        self._call(self.lib.ref_xla_rasterize_bwd,
                   [colors, opacities, background, xys, depths, radii, conics, cum_tiles_hit,
                    final_Ts, final_idx, v_img, v_img_alpha, *out.values()], desc)
        return out

    def project_bwd(self, means3d, scales, quats, viewmat, cov3d, xys, radii, conics,
                    compensation, v_compensation, v_xy, v_depth, v_conic, *, img_shape, f, c,
                    glob_scale, clip_thresh, block_width):
        n = means3d.shape[0]
        dev = means3d.device
        out = dict(v_mean3d=torch.empty(n, 3, device=dev), v_scale=torch.empty(n, 3, device=dev),
                   v_quat=torch.empty(n, 4, device=dev), v_cov2d=torch.empty(n, 3, device=dev),
                   v_cov3d=torch.empty(n, 6, device=dev))
        desc = self.descriptor(n, img_shape, f, c, glob_scale, clip_thresh, block_width)
        self._call(self.lib.ref_xla_project_bwd,
                   [means3d, scales, quats, viewmat, cov3d, xys, radii, conics, compensation,
                    v_compensation, v_xy, v_depth, v_conic, *out.values()], desc)
        return out

    def sort_and_bin(self, xys, depths, radii, cum_tiles_hit, *, img_shape, block_width):
        n = xys.shape[0]
        count = int(cum_tiles_hit[-1].item()) if n else 0
        h, w = img_shape
        ntiles = ((w + block_width - 1) // block_width) * ((h + block_width - 1) // block_width)
        dev = xys.device
        out = dict(isect_ids=torch.zeros(count, dtype=torch.int64, device=dev),
                   gaussian_ids=torch.zeros(count, dtype=torch.int32, device=dev),
                   isect_ids_sorted=torch.zeros(count, dtype=torch.int64, device=dev),
                   gaussian_ids_sorted=torch.zeros(count, dtype=torch.int32, device=dev),
                   tile_bins=torch.zeros(ntiles, 2, dtype=torch.int32, device=dev))
        desc = self.descriptor(n, img_shape, block_width=block_width)
        stream = torch.cuda.current_stream().cuda_stream
        self._check(self.lib.ref_stage_sort_and_bin(
            C.c_void_p(stream), desc, len(desc), count, xys.data_ptr(), depths.data_ptr(),
            radii.data_ptr(), cum_tiles_hit.data_ptr(), out["isect_ids"].data_ptr(),
            out["gaussian_ids"].data_ptr(), out["isect_ids_sorted"].data_ptr(),
            out["gaussian_ids_sorted"].data_ptr(), out["tile_bins"].data_ptr()))
        return out

    def render(self, means3d, scales, quats, colors, opacities, *, viewmat, background,
               img_shape, f, c, glob_scale, clip_thresh, block_size=16, v_img=None):
        """Forward (and with ``v_img`` the backward) of jaxsplat.render."""
        kw = dict(img_shape=img_shape, f=f, c=c, glob_scale=glob_scale, clip_thresh=clip_thresh,
                  block_width=block_size)
        p = self.project_fwd(means3d, scales, quats, viewmat, **kw)
        r = self.rasterize_fwd(colors, opacities, background, p["xys"], p["depths"], p["radii"],
                               p["conics"], p["cum_tiles_hit"], img_shape=img_shape,
                               block_width=block_size)
        out = {**p, **r}
        if v_img is None:
            return out
        h, w = img_shape
        n = means3d.shape[0]
        rb = self.rasterize_bwd(colors, opacities, background, p["xys"], p["depths"], p["radii"],
                                p["conics"], p["cum_tiles_hit"], r["final_Ts"], r["final_idx"],
                                v_img, torch.zeros(h, w, 1, device=v_img.device),
                                img_shape=img_shape, block_width=block_size)
        z = torch.zeros(n, 1, device=means3d.device)
        pb = self.project_bwd(means3d, scales, quats, viewmat, p["cov3d"], p["xys"], p["radii"],
                              p["conics"], p["compensation"], z, rb["v_xy"], z, rb["v_conic"],
                              **kw)
        out.update(rb)
        out.update(pb)
        return out
