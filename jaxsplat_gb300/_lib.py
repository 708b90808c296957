"""ctypes binding of libsplat.so (the C ABI in include/splat.h).

The library is built in-tree by ``jaxsplat_gb300.build`` (or
``__graft_entry__.build()``).  There is no fallback: if the shared library is
missing or fails to load, every operation raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsplat.so")


class SplatParams(C.Structure):
    """Mirror of ``splat_params`` (include/splat.h)."""

    _fields_ = [
        ("num_points", C.c_uint32),
        ("img_height", C.c_uint32),
        ("img_width", C.c_uint32),
        ("fx", C.c_float),
        ("fy", C.c_float),
        ("cx", C.c_float),
        ("cy", C.c_float),
        ("glob_scale", C.c_float),
        ("clip_thresh", C.c_float),
        ("block_width", C.c_uint32),
        ("device_status", C.c_void_p),
        ("spin_limit", C.c_uint32),
    ]


class SplatView(C.Structure):
    """Mirror of ``splat_view`` (include/splat.h)."""

    _fields_ = [
        ("viewmat", C.c_float * 16),
        ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("background", C.c_float * 3),
        ("scene", C.c_uint32),
        ("img_height", C.c_uint32), ("img_width", C.c_uint32),
        ("tiles_x", C.c_uint32), ("tiles_y", C.c_uint32),
        ("gauss_base", C.c_uint32), ("num_points", C.c_uint32),
        ("entry_base", C.c_uint32), ("tile_base", C.c_uint32),
        ("pixel_base", C.c_uint64),
    ]


class SplatBatch(C.Structure):
    """Mirror of ``splat_batch`` (include/splat.h)."""

    _fields_ = [
        ("num_scenes", C.c_uint32), ("num_views", C.c_uint32),
        ("glob_scale", C.c_float), ("clip_thresh", C.c_float),
        ("block_width", C.c_uint32),
        ("device_status", C.c_void_p),
        ("spin_limit", C.c_uint32),
        ("views", C.c_void_p),
        ("num_points", C.c_uint64),
        ("num_entries", C.c_uint64), ("num_tiles", C.c_uint64), ("num_pixels", C.c_uint64),
    ]


class SplatAdamSeg(C.Structure):
    """Mirror of ``splat_adam_seg`` (include/splat.h)."""

    _fields_ = [
        ("w", C.c_void_p), ("m", C.c_void_p), ("v", C.c_void_p), ("g", C.c_void_p),
        ("w16", C.c_void_p), ("n", C.c_int64),
    ]


STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "workspace too small",
          4: "intersection count out of range", 5: "device-side check failed"}

# (name, restype, argtypes)
_P = C.POINTER(SplatParams)
_v = C.c_void_p
_SIGS = [
    ("splat_last_error", C.c_char_p, []),
    ("splat_status_string", C.c_char_p, [C.c_int]),
    ("splat_device_status_string", C.c_char_p, [C.c_uint32]),
    ("splat_version", C.c_int, []),
    ("splat_project_fwd_workspace_size", C.c_size_t, [_P]),
    ("splat_project_fwd", C.c_int, [_P] + [_v] * 13 + [_v, C.c_size_t, _v]),
    ("splat_project_fwd_packed", C.c_int, [_P] + [_v] * 16 + [_v, C.c_size_t, _v]),
    ("splat_read_counts", C.c_int, [_P, _v, _v, _v, C.POINTER(C.c_int64),
                                    C.POINTER(C.c_uint32), _v]),
    ("splat_sort_workspace_size", C.c_size_t, [_P, C.c_int64]),
    ("splat_sort_and_bin", C.c_int, [_P, C.c_int64] + [_v] * 10 + [_v, C.c_size_t, _v]),
    ("splat_pack_splats", C.c_int, [_P] + [_v] * 5 + [_v]),
    ("splat_rasterize_fwd", C.c_int, [_P, C.c_int64] + [_v] * 9 + [_v]),
    ("splat_rasterize_fwd_l2", C.c_int, [_P, C.c_int64] + [_v] * 12 + [_v]),
    ("splat_rasterize_bwd", C.c_int, [_P, C.c_int64] + [_v] * 15 + [_v]),
    ("splat_project_bwd", C.c_int, [_P] + [_v] * 17 + [_v]),
    ("splat_l2_loss", C.c_int, [_v, _v, C.c_int64, _v, _v, _v]),
    ("splat_count_pairs", C.c_int, [_P, C.c_int64] + [_v] * 6 + [_v]),
    ("splat_xla_project_fwd", None, [_v, C.POINTER(_v), C.c_char_p, C.c_size_t]),
    ("splat_xla_project_bwd", None, [_v, C.POINTER(_v), C.c_char_p, C.c_size_t]),
    ("splat_xla_rasterize_fwd", None, [_v, C.POINTER(_v), C.c_char_p, C.c_size_t]),
    ("splat_xla_rasterize_bwd", None, [_v, C.POINTER(_v), C.c_char_p, C.c_size_t]),
    ("splat_xla_make_descriptor", C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_float,
                                            C.c_float, C.c_float, C.c_float, C.c_float,
                                            C.c_float, C.c_uint32, _v, C.c_size_t]),
    ("splat_selftest_wait_timeout", C.c_int, [C.c_uint32, _v, _v]),
    ("splat_project_fwd_noalloc", C.c_int, [_P] + [_v] * 13 + [_v]),
    ("splat_fit_transform", C.c_int, [C.c_int] + [_v] * 6 + [_v]),
    ("splat_fit_adam", C.c_int, [C.c_int, C.c_float] + [_v] * 16 + [_v]),
    ("splat_batch_layout", C.c_int, [C.POINTER(SplatBatch), C.POINTER(SplatView),
                                     C.POINTER(C.c_uint32)]),
    ("splat_batch_project_fwd", C.c_int, [C.POINTER(SplatBatch)] + [_v] * 10 + [_v]),
    ("splat_batch_project_fwd_packed", C.c_int, [C.POINTER(SplatBatch)] + [_v] * 13 + [_v]),
    ("splat_batch_sort_workspace_size", C.c_size_t, [C.POINTER(SplatBatch), C.c_int64]),
    ("splat_batch_sort_and_bin", C.c_int, [C.POINTER(SplatBatch), C.c_int64] + [_v] * 7
     + [_v, C.c_size_t, _v]),
    ("splat_batch_pack", C.c_int, [C.POINTER(SplatBatch)] + [_v] * 5 + [_v]),
    ("splat_batch_rasterize_fwd", C.c_int, [C.POINTER(SplatBatch), C.c_int64] + [_v] * 8
     + [C.c_uint32, _v, _v]),
    ("splat_batch_rasterize_fwd_l2", C.c_int, [C.POINTER(SplatBatch), C.c_int64] + [_v] * 11
     + [C.c_uint32, _v, _v]),
    ("splat_batch_rasterize_bwd", C.c_int, [C.POINTER(SplatBatch), C.c_int64] + [_v] * 13
     + [C.c_uint32, _v, _v]),
    ("splat_batch_l2_loss", C.c_int, [C.POINTER(SplatBatch)] + [_v] * 4 + [_v]),
    ("splat_batch_project_bwd", C.c_int, [C.POINTER(SplatBatch)] + [_v] * 12 + [_v]),
    ("splat_gemm_bf16", C.c_int, [_v, _v, _v] + [C.c_int] * 7 + [_v, _v]),
    ("splat_gemm_bf16_mn", C.c_int, [_v, C.c_int, _v, C.c_int, _v] + [C.c_int] * 7 + [_v, _v]),
    ("splat_gemm_bf16_bias_act", C.c_int, [_v] * 5 + [C.c_int] * 7 + [_v, _v]),
    ("splat_nn_im2col3x3", C.c_int, [_v, _v] + [C.c_int] * 6 + [_v]),
    ("splat_nn_col2im3x3", C.c_int, [_v, _v] + [C.c_int] * 6 + [_v]),
    ("splat_nn_col2im_act3x3", C.c_int, [_v, _v, _v, _v] + [C.c_int] * 6 + [_v]),
    ("splat_nn_bias_act", C.c_int, [_v, _v, _v, _v, C.c_int64, C.c_int, C.c_int, _v]),
    ("splat_nn_act_grad", C.c_int, [_v, _v, _v, _v, C.c_int64, C.c_int, C.c_int, _v]),
    ("splat_nn_adam", C.c_int, [_v, _v, _v, _v, _v, C.c_int64, C.c_float, C.c_int, _v]),
    ("splat_nn_adam_multi", C.c_int, [C.POINTER(SplatAdamSeg), C.c_int, C.c_float, C.c_int, _v]),
]

EXPORTED = [name for name, _, _ in _SIGS]

_lock = threading.Lock()
_lib = None


class SplatError(RuntimeError):
    pass


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libsplat.so once; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise SplatError(
                f"libsplat.so not found at {path}: build it with "
                "`python -m jaxsplat_gb300.build` (there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, res, args in _SIGS:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        lib = load()
        msg = lib.splat_last_error().decode(errors="replace")
        raise SplatError(f"{what}: {STATUS.get(rc, rc)}: {msg}")


def make_params(num_points, img_shape, f=(0.0, 0.0), c=(0.0, 0.0), glob_scale=1.0,
                clip_thresh=0.01, block_width=16, device_status=None, spin_limit=0):
    h, w = img_shape
    return SplatParams(int(num_points), int(h), int(w), float(f[0]), float(f[1]), float(c[0]),
                       float(c[1]), float(glob_scale), float(clip_thresh), int(block_width),
                       device_status, int(spin_limit))
