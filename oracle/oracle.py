"""ctypes wrapper around the CPU restatement in splat_oracle.c.

TEST INFRASTRUCTURE ONLY: this is the checker.  tests/, ``smoke()`` and the
cpu_baseline leg of bench.py use it; the jaxsplat_gb300 package never does.

``Oracle("f32")`` evaluates the reference's fp32 arithmetic (with nvcc's
multiply-add contraction written out); ``Oracle("f64")`` evaluates the same
algorithm in double precision (the FP64 transcription).  Every method takes
and returns numpy arrays with the reference's shapes (jaxsplat/_project/
abstract.py:7-21, jaxsplat/_rasterize/abstract.py:7-24).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


def build(force: bool = False) -> None:
    """Compile both precisions of the oracle into oracle/_build/."""
    from .build import build_oracle

    build_oracle(force)


_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


class Oracle:
    def __init__(self, precision: str = "f32"):
        assert precision in ("f32", "f64")
        build()
        bits = "32" if precision == "f32" else "64"
        self.lib = C.CDLL(os.path.join(BUILD, f"liboracle{bits}.so"))
        self.dtype = np.float32 if precision == "f32" else np.float64
        self.real = C.c_float if precision == "f32" else C.c_double
        self.prefix = f"oracle{bits}_"
        rp = np.ctypeslib.ndpointer(self.dtype, flags="C_CONTIGUOUS")
        R, U, I = self.real, C.c_uint, C.c_int
        sig = {
            "project_fwd": [I, rp, rp, R, rp, rp, R, R, R, R, U, U, U, R, rp, rp, rp, _i32p, rp,
                            rp, _i32p, _i32p],
            "map_intersects": [I, rp, rp, _i32p, _i32p, U, U, U, _i64p, _i32p],
            "sort_end_bit": [U],
            "sort_pairs": [C.c_int64, _i64p, _i32p, I, _i64p, _i32p],
            "tile_bin_edges": [C.c_int64, _i64p, I, _i32p],
            "rasterize_fwd": [U, U, U, C.c_int64, _i32p, _i32p, rp, rp, rp, rp, rp, rp, _i32p, rp],
            "rasterize_bwd": [U, U, U, I, C.c_int64, _i32p, _i32p, rp, rp, rp, rp, rp, rp, _i32p,
                              rp, rp, rp, rp, rp, rp, rp],
            "project_bwd": [I, rp, rp, R, rp, rp, R, R, rp, _i32p, rp, rp, rp, rp, rp, rp, rp, rp,
                            rp, rp, rp],
            "set_threads": [I],
            "max_threads": [],
        }
        for name, args in sig.items():
            fn = getattr(self.lib, self.prefix + name)
            fn.argtypes = args
            fn.restype = I if name in ("sort_end_bit", "max_threads") else None
            setattr(self, "_" + name, fn)

    def set_threads(self, n: int) -> None:
        self._set_threads(int(n))

    def max_threads(self) -> int:
        return int(self._max_threads())

    def _r(self, a) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(a, dtype=self.dtype))

    @staticmethod
    def tiles(img_shape, block_width):
        h, w = img_shape
        return (w + block_width - 1) // block_width, (h + block_width - 1) // block_width

    # jaxsplat/_project/__init__.py:56-87 + lib/ops.cu:12-61
    def project_fwd(self, means3d, scales, quats, viewmat, *, img_shape, f, c, glob_scale,
                    clip_thresh, block_width):
        n = int(np.shape(means3d)[0])
        h, w = img_shape
        out = dict(
            cov3d=np.zeros((n, 6), self.dtype), xys=np.zeros((n, 2), self.dtype),
            depths=np.zeros((n, 1), self.dtype), radii=np.zeros((n, 1), np.int32),
            conics=np.zeros((n, 3), self.dtype), compensation=np.zeros((n, 1), self.dtype),
            num_tiles_hit=np.zeros((n, 1), np.int32), cum_tiles_hit=np.zeros((n, 1), np.int32),
        )
        self._project_fwd(
            n, self._r(means3d), self._r(scales), glob_scale, self._r(quats), self._r(viewmat),
            f[0], f[1], c[0], c[1], w, h, block_width, clip_thresh, out["cov3d"], out["xys"],
            out["depths"], out["radii"], out["conics"], out["compensation"],
            out["num_tiles_hit"], out["cum_tiles_hit"])
        return out

    # lib/kernels/forward.cu:135-179
    def map_intersects(self, xys, depths, radii, cum_tiles_hit, *, img_shape, block_width):
        n = int(np.shape(xys)[0])
        total = int(np.asarray(cum_tiles_hit).reshape(-1)[-1]) if n else 0
        keys = np.zeros(total, np.int64)
        ids = np.zeros(total, np.int32)
        h, w = img_shape
        self._map_intersects(n, self._r(xys), self._r(depths),
                             np.ascontiguousarray(radii, np.int32),
                             np.ascontiguousarray(cum_tiles_hit, np.int32), w, h, block_width,
                             keys, ids)
        return keys, ids

    def sort_end_bit(self, n_tiles: int) -> int:
        return int(self._sort_end_bit(n_tiles))

    # lib/ops.cu:723-757
    def sort_pairs(self, keys, vals, end_bit):
        keys = np.ascontiguousarray(keys, np.int64)
        vals = np.ascontiguousarray(vals, np.int32)
        ko = np.empty_like(keys)
        vo = np.empty_like(vals)
        self._sort_pairs(keys.size, keys, vals, int(end_bit), ko, vo)
        return ko, vo

    # lib/kernels/forward.cu:184-208
    def tile_bin_edges(self, sorted_keys, n_tiles):
        sorted_keys = np.ascontiguousarray(sorted_keys, np.int64)
        bins = np.zeros((n_tiles, 2), np.int32)
        self._tile_bin_edges(sorted_keys.size, sorted_keys, n_tiles, bins)
        return bins

    def sort_and_bin(self, xys, depths, radii, cum_tiles_hit, *, img_shape, block_width):
        """lib/ops.cu:645-793: emission, stable sort, bin edges."""
        tx, ty = self.tiles(img_shape, block_width)
        keys, ids = self.map_intersects(xys, depths, radii, cum_tiles_hit, img_shape=img_shape,
                                        block_width=block_width)
        ks, vs = self.sort_pairs(keys, ids, self.sort_end_bit(tx * ty))
        bins = self.tile_bin_edges(ks, tx * ty)
        return dict(isect_ids=keys, gaussian_ids=ids, isect_ids_sorted=ks,
                    gaussian_ids_sorted=vs, tile_bins=bins)

    # lib/kernels/forward.cu:339-462 + lib/ops.cu:107-170
    def rasterize_fwd(self, ids_sorted, tile_bins, xys, conics, colors, opacities, background,
                      *, img_shape, block_width):
        h, w = img_shape
        ids_sorted = np.ascontiguousarray(ids_sorted, np.int32)
        final_Ts = np.zeros((h, w, 1), self.dtype)
        final_idx = np.zeros((h, w, 1), np.int32)
        img = np.zeros((h, w, 3), self.dtype)
        self._rasterize_fwd(w, h, block_width, ids_sorted.size, ids_sorted,
                            np.ascontiguousarray(tile_bins, np.int32), self._r(xys),
                            self._r(conics), self._r(colors), self._r(opacities),
                            self._r(background), final_Ts, final_idx, img)
        return dict(final_Ts=final_Ts, final_idx=final_idx, img=img)

    # lib/kernels/backward.cu:153-343 + lib/ops.cu:172-235
    def rasterize_bwd(self, ids_sorted, tile_bins, xys, conics, colors, opacities, background,
                      final_Ts, final_idx, v_img, v_img_alpha, *, img_shape, block_width):
        h, w = img_shape
        n = int(np.shape(xys)[0])
        ids_sorted = np.ascontiguousarray(ids_sorted, np.int32)
        out = dict(v_xy=np.zeros((n, 2), self.dtype), v_xy_abs=np.zeros((n, 2), self.dtype),
                   v_conic=np.zeros((n, 3), self.dtype), v_colors=np.zeros((n, 3), self.dtype),
                   v_opacity=np.zeros((n, 1), self.dtype))
        self._rasterize_bwd(w, h, block_width, n, ids_sorted.size, ids_sorted,
                            np.ascontiguousarray(tile_bins, np.int32), self._r(xys),
                            self._r(conics), self._r(colors), self._r(opacities),
                            self._r(background), self._r(final_Ts),
                            np.ascontiguousarray(final_idx, np.int32), self._r(v_img),
                            self._r(v_img_alpha), out["v_xy"], out["v_xy_abs"], out["v_conic"],
                            out["v_colors"], out["v_opacity"])
        return out

    # lib/kernels/backward.cu:345-418 + lib/ops.cu:63-105
    def project_bwd(self, means3d, scales, quats, viewmat, cov3d, radii, conics, compensation,
                    v_xy, v_depth, v_conic, v_compensation, *, f, glob_scale):
        n = int(np.shape(means3d)[0])
        out = dict(v_cov2d=np.zeros((n, 3), self.dtype), v_cov3d=np.zeros((n, 6), self.dtype),
                   v_mean3d=np.zeros((n, 3), self.dtype), v_scale=np.zeros((n, 3), self.dtype),
                   v_quat=np.zeros((n, 4), self.dtype))
        self._project_bwd(n, self._r(means3d), self._r(scales), glob_scale, self._r(quats),
                          self._r(viewmat), f[0], f[1], self._r(cov3d),
                          np.ascontiguousarray(radii, np.int32), self._r(conics),
                          self._r(compensation), self._r(v_xy), self._r(v_depth),
                          self._r(v_conic), self._r(v_compensation), out["v_cov2d"],
                          out["v_cov3d"], out["v_mean3d"], out["v_scale"], out["v_quat"])
        return out

    def render(self, means3d, scales, quats, colors, opacities, *, viewmat, background,
               img_shape, f, c, glob_scale, clip_thresh, block_size=16, v_img=None):
        """jaxsplat/__init__.py:6-70 forward, and with ``v_img`` the custom_vjp
        backward chain (jaxsplat/_rasterize/__init__.py:155-187 then
        jaxsplat/_project/__init__.py:155-205) with zero cotangents for depth,
        compensation and the alpha image.  Returns every intermediate."""
        bw = block_size
        p = self.project_fwd(means3d, scales, quats, viewmat, img_shape=img_shape, f=f, c=c,
                             glob_scale=glob_scale, clip_thresh=clip_thresh, block_width=bw)
        s = self.sort_and_bin(p["xys"], p["depths"], p["radii"], p["cum_tiles_hit"],
                              img_shape=img_shape, block_width=bw)
        r = self.rasterize_fwd(s["gaussian_ids_sorted"], s["tile_bins"], p["xys"], p["conics"],
                               colors, opacities, background, img_shape=img_shape,
                               block_width=bw)
        out = {**p, **s, **r}
        if v_img is None:
            return out
        h, w = img_shape
        n = int(np.shape(means3d)[0])
        rb = self.rasterize_bwd(s["gaussian_ids_sorted"], s["tile_bins"], p["xys"], p["conics"],
                                colors, opacities, background, r["final_Ts"], r["final_idx"],
                                v_img, np.zeros((h, w, 1), self.dtype), img_shape=img_shape,
                                block_width=bw)
        pb = self.project_bwd(means3d, scales, quats, viewmat, p["cov3d"], p["radii"],
                              p["conics"], p["compensation"], rb["v_xy"],
                              np.zeros((n, 1), self.dtype), rb["v_conic"],
                              np.zeros((n, 1), self.dtype), f=f, glob_scale=glob_scale)
        out.update(rb)
        out.update(pb)
        return out
