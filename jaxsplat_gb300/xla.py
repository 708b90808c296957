"""The reference's native-module interface for XLA: ``registrations()`` and
``make_descriptor(...)``, served by libsplat.so.

jaxsplat imports a pybind11 module ``_jaxsplat`` with these two functions
(``lib/ffi.cu:4-52``): ``registrations()`` maps the custom-call target names
``project_fwd``, ``project_bwd``, ``rasterize_fwd`` and ``rasterize_bwd`` to
PyCapsules named ``xla._CUSTOM_CALL_TARGET`` (registered with XLA in
``jaxsplat/_project/impl.py:11-13`` and ``jaxsplat/_rasterize/impl.py:11-13``),
and ``make_descriptor`` packs the 80-byte opaque descriptor that the
lowerings pass (``jaxsplat/_project/lowering.py:28-36``,
``jaxsplat/_rasterize/lowering.py:28-36``).  This module provides the same
two functions with the same names and keyword arguments, over the
``splat_xla_*`` entry points (same call signature, buffer order and
descriptor as the reference's targets), so that ``_jaxsplat`` can be
replaced by ``jaxsplat_gb300.xla`` without touching the lowerings.  jax itself
is not needed to build the capsules.
"""

from __future__ import annotations

import ctypes as C

from . import _lib

CAPSULE_NAME = b"xla._CUSTOM_CALL_TARGET"
TARGETS = {
    "project_fwd": "splat_xla_project_fwd",
    "project_bwd": "splat_xla_project_bwd",
    "rasterize_fwd": "splat_xla_rasterize_fwd",
    "rasterize_bwd": "splat_xla_rasterize_bwd",
}
DESCRIPTOR_BYTES = 80

_PyCapsule_New = C.pythonapi.PyCapsule_New
_PyCapsule_New.restype = C.py_object
_PyCapsule_New.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]


def _capsule(symbol: str):
    fn = C.cast(getattr(_lib.load(), symbol), C.c_void_p).value
    return _PyCapsule_New(fn, CAPSULE_NAME, None)


def registrations() -> dict:
    """Custom-call target name -> PyCapsule of its ``splat_xla_*`` function
    (``void(cudaStream_t, void **buffers, const char *opaque, size_t)``)."""
    return {name: _capsule(symbol) for name, symbol in TARGETS.items()}


def make_descriptor(num_points, img_shape, f, c, glob_scale, clip_thresh, block_width) -> bytes:
    """The 80-byte descriptor of ``lib/ops.h:9-22`` (img_shape is (H, W))."""
    lib = _lib.load()
    buf = C.create_string_buffer(DESCRIPTOR_BYTES)
    rc = lib.splat_xla_make_descriptor(
        int(num_points), int(img_shape[0]), int(img_shape[1]), float(f[0]), float(f[1]),
        float(c[0]), float(c[1]), float(glob_scale), float(clip_thresh), int(block_width), buf,
        DESCRIPTOR_BYTES)
    _lib.check(rc, "make_descriptor")
    return buf.raw
