"""The C ABI library loads, exports every symbol include/splat.h declares,
and its plain-data layouts match the header and the reference's descriptor.
No kernel is launched here (no GPU needed)."""

import ctypes as C
import os
import re
import struct
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "splat.h")


@pytest.fixture(scope="module")
def lib():
    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300.build import build

    build()
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(splat_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    from jaxsplat_gb300 import _lib

    assert sorted(_lib.EXPORTED) == names


_C_SCALARS = {"int": (4, "i"), "int32_t": (4, "i"), "uint32_t": (4, "u"), "int64_t": (8, "i"),
              "uint64_t": (8, "u"), "size_t": (8, "u"), "float": (4, "f"), "double": (8, "f")}


def _c_kind(decl: str):
    """'ptr' for pointers and the stream handle, else (bytes, i/u/f)."""
    decl = decl.strip()
    if "*" in decl or decl.split()[0] == "splat_stream_t":
        return "ptr"
    words = [w for w in decl.split() if w != "const"]
    return _C_SCALARS[words[0]]


def _ctypes_kind(t):
    if t in (C.c_void_p, C.c_char_p) or issubclass(t, C._Pointer):
        return "ptr"
    if t in (C.c_float, C.c_double):
        return (C.sizeof(t), "f")
    return (C.sizeof(t), "i" if t(-1).value < 0 else "u")


def declared_prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    protos = {}
    for ret, name, params in re.findall(r"SPLAT_API\s+([\w\s\*]+?)\s*\b(splat_\w+)\s*\(([^)]*)\)\s*;",
                                        text):
        ps = [p for p in (q.strip() for q in params.split(",")) if p and p != "void"]
        protos[name] = (ret.strip(), ps)
    return protos


def test_ctypes_signatures_match_header():
    """Every binding in _lib has the header's parameter count, and each
    parameter (and the result) the same class: pointer, or a scalar of the
    same width and signedness."""
    from jaxsplat_gb300 import _lib

    protos = declared_prototypes()
    assert sorted(protos) == declared_functions()
    for name, res, args in _lib._SIGS:
        ret, params = protos[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for k, (t, p) in enumerate(zip(args, params)):
            assert _ctypes_kind(t) == _c_kind(p + " x"), (name, k, p)
        if ret == "void":
            assert res is None, name
        else:
            assert _ctypes_kind(res) == _c_kind(ret + " x"), (name, ret)


@pytest.mark.parametrize("c_name,py_name", [("splat_params", "SplatParams"),
                                             ("splat_view", "SplatView"),
                                             ("splat_batch", "SplatBatch"),
                                             ("splat_adam_seg", "SplatAdamSeg")])
def test_struct_layout_matches_header(tmp_path, c_name, py_name):
    """Size, and offset and size of every field, of the ctypes mirror against
    the C compiler's layout of the header's struct."""
    from jaxsplat_gb300 import _lib

    mirror = getattr(_lib, py_name)
    fields = [f[0] for f in mirror._fields_]
    lines = [f'printf("%zu\\n", sizeof({c_name}));']
    for f in fields:
        lines.append(f'printf("%zu %zu\\n", offsetof({c_name}, {f}), '
                     f"sizeof((({c_name} *)0)->{f}));")
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "splat.h"\n'
                   "int main(void){" + "".join(lines) + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert C.sizeof(mirror) == out[0], c_name
    for k, f in enumerate(fields):
        desc = getattr(mirror, f)
        assert (desc.offset, desc.size) == (out[1 + 2 * k], out[2 + 2 * k]), (c_name, f)


def test_descriptor_matches_reference_layout(lib):
    """splat_xla_make_descriptor writes the 80 bytes that jaxsplat's
    make_descriptor packs (lib/ffi.cu:15-52, struct lib/ops.h:9-22)."""
    buf = C.create_string_buffer(80)
    rc = lib.splat_xla_make_descriptor(100_000, 1080, 1920, 1200.0, 1100.0, 960.0, 540.0, 1.0,
                                       0.01, 16, buf, 80)
    assert rc == 0
    want = struct.pack("<I3I4f", 100_000, 1920, 1080, 1, 1200.0, 1100.0, 960.0, 540.0)
    want += struct.pack("<ffII I3I3I", 1.0, 0.01, 16, 391, 256, 120, 68, 1, 16, 16, 1)
    want += b"\0" * (80 - len(want))
    assert buf.raw == want


def test_descriptor_size_is_checked(lib):
    buf = C.create_string_buffer(40)
    assert lib.splat_xla_make_descriptor(1, 1, 1, 1.0, 1.0, 0.0, 0.0, 1.0, 0.0, 16, buf, 40) == 1
    assert b"80" in lib.splat_last_error()


@pytest.mark.parametrize("bw", [0, 1, 17, 64])
def test_invalid_block_width_rejected_without_gpu(lib, bw):
    from jaxsplat_gb300 import _lib

    p = _lib.make_params(10, (32, 32), block_width=bw)
    rc = lib.splat_project_fwd(C.byref(p), *([None] * 13), None, 0, None)
    assert rc == 1  # SPLAT_ERR_INVALID_ARG, before any CUDA call
    assert b"block_width" in lib.splat_last_error()


@pytest.mark.parametrize("n,shape,bw,msg", [
    (10, (0, 32), 16, b"image size"),
    (10, (65535, 65535), 2, b"tiles"),          # 32768^2 tiles > 2^22
    (2**31, (32, 32), 16, b"exceeds int32"),
])
def test_invalid_sizes_rejected_without_gpu(lib, n, shape, bw, msg):
    """Every typed entry point validates the parameters before any CUDA call:
    empty images, tile grids past 2^22 tiles, point counts past int32."""
    from jaxsplat_gb300 import _lib

    p = _lib.make_params(n, shape, block_width=bw)
    for call in (lambda: lib.splat_project_fwd(C.byref(p), *([None] * 13), None, 0, None),
                 lambda: lib.splat_rasterize_fwd(C.byref(p), 0, *([None] * 9), None),
                 lambda: lib.splat_project_bwd(C.byref(p), *([None] * 17), None)):
        assert call() == 1
        assert msg in lib.splat_last_error()


def test_strings(lib):
    assert lib.splat_status_string(4) == b"intersection count out of range"
    assert b"lookback-timeout" in lib.splat_device_status_string(1)
    assert lib.splat_version() >= 1


def test_misaligned_workspace_rejected_without_gpu(lib):
    """Workspaces must be 256-byte aligned (they hold words updated by 64-bit
    atomics); a misaligned one is refused before any CUDA call.  The other
    pointers are placeholders that are never dereferenced."""
    from jaxsplat_gb300 import _lib

    p = _lib.make_params(10, (32, 32), (32.0, 32.0), (16.0, 16.0), 1.0, 0.01, 16)
    fake = [C.c_void_p(0x10000 + 256 * i) for i in range(13)]
    rc = lib.splat_project_fwd(C.byref(p), *fake, C.c_void_p(0x20008), 1 << 20, None)
    assert rc == 1 and b"256-byte aligned" in lib.splat_last_error()
    rc = lib.splat_sort_and_bin(C.byref(p), 100, None, *fake[:4], fake[4], fake[5], None, None,
                                None, C.c_void_p(0x20010), 1 << 20, None)
    assert rc == 1 and b"256-byte aligned" in lib.splat_last_error()


def test_project_fwd_needs_a_count_output_without_gpu(lib):
    """cum_tiles_hit is optional when total_out is given (count-only
    projection); with neither the call is refused before any CUDA call."""
    from jaxsplat_gb300 import _lib

    p = _lib.make_params(10, (32, 32), (32.0, 32.0), (16.0, 16.0), 1.0, 0.01, 16)
    fake = [C.c_void_p(0x10000 + 256 * i) for i in range(11)]
    rc = lib.splat_project_fwd(C.byref(p), *fake, None, None, C.c_void_p(0x20000), 1 << 20, None)
    assert rc == 1 and b"cum_tiles_hit or total_out" in lib.splat_last_error()


def test_misaligned_tile_bins_rejected_without_gpu(lib):
    """tile_bins is accessed as int2: a 4-byte offset is refused before any
    CUDA call."""
    from jaxsplat_gb300 import _lib

    p = _lib.make_params(10, (32, 32), (32.0, 32.0), (16.0, 16.0), 1.0, 0.01, 16)
    fake = [C.c_void_p(0x10000 + 256 * i) for i in range(8)]
    rc = lib.splat_rasterize_fwd(C.byref(p), 100, None, fake[0], C.c_void_p(0x30004), fake[1],
                                 fake[2], fake[3], fake[4], fake[5], None, None)
    assert rc == 1 and b"8-byte aligned" in lib.splat_last_error()


def test_xla_module_mirrors_the_reference_native_module(lib):
    """jaxsplat_gb300.xla: registrations() gives the four custom-call targets
    as PyCapsules named xla._CUSTOM_CALL_TARGET pointing at the splat_xla_*
    functions; make_descriptor(**kwargs) takes the reference lowering's
    keyword arguments and returns the 80-byte descriptor."""
    from jaxsplat_gb300 import xla

    regs = xla.registrations()
    assert set(regs) == {"project_fwd", "project_bwd", "rasterize_fwd", "rasterize_bwd"}
    get_name = C.pythonapi.PyCapsule_GetName
    get_name.restype, get_name.argtypes = C.c_char_p, [C.py_object]
    get_ptr = C.pythonapi.PyCapsule_GetPointer
    get_ptr.restype, get_ptr.argtypes = C.c_void_p, [C.py_object, C.c_char_p]
    for name, cap in regs.items():
        assert get_name(cap) == b"xla._CUSTOM_CALL_TARGET"
        want = C.cast(getattr(lib, "splat_xla_" + name), C.c_void_p).value
        assert get_ptr(cap, b"xla._CUSTOM_CALL_TARGET") == want
    d = xla.make_descriptor(num_points=100_000, img_shape=(1080, 1920), f=(1200.0, 1100.0),
                            c=(960.0, 540.0), glob_scale=1.0, clip_thresh=0.01, block_width=16)
    want = struct.pack("<I3I4f", 100_000, 1920, 1080, 1, 1200.0, 1100.0, 960.0, 540.0)
    want += struct.pack("<ffII I3I3I", 1.0, 0.01, 16, 391, 256, 120, 68, 1, 16, 16, 1)
    assert d == want + b"\0" * (80 - len(want))


def test_xla_make_descriptor_rejects_bad_block_width(lib):
    from jaxsplat_gb300 import _lib, xla

    with pytest.raises(_lib.SplatError):
        xla.make_descriptor(num_points=10, img_shape=(32, 32), f=(32.0, 32.0), c=(16.0, 16.0),
                            glob_scale=1.0, clip_thresh=0.01, block_width=0)


def test_network_entry_points_reject_bad_arguments_without_gpu(lib):
    """The warm-start network's entry points refuse bad shapes, strides,
    alignments and segment tables before any CUDA call; the pointers are
    placeholders that are never dereferenced."""
    from jaxsplat_gb300 import _lib

    a, b, c = C.c_void_p(0x10000), C.c_void_p(0x20000), C.c_void_p(0x30000)

    def refused(rc, what):
        assert rc == 1, what
        assert what.encode() in lib.splat_last_error(), lib.splat_last_error()

    # MN-major A stored [K, M]: its leading dimension must cover M
    refused(lib.splat_gemm_bf16_mn(a, 1, b, 1, c, 48, 64, 64, 32, 64, 64, 0, None, None),
            "covering the stored rows")
    # K-major operands: K a multiple of 8
    refused(lib.splat_gemm_bf16_mn(a, 0, b, 1, c, 64, 64, 60, 64, 64, 64, 0, None, None),
            "multiples of 8")
    # 16-byte aligned operands
    refused(lib.splat_gemm_bf16(C.c_void_p(0x10008), b, c, 64, 64, 64, 64, 64, 64, 0, None,
                                None), "16-byte aligned")
    # im2col: kpad a multiple of 8 and >= 9c; cols 16-byte aligned
    refused(lib.splat_nn_im2col3x3(a, b, 1, 8, 8, 3, 2, 28, None), "im2col3x3")
    refused(lib.splat_nn_im2col3x3(a, C.c_void_p(0x20008), 1, 8, 8, 3, 2, 32, None),
            "im2col3x3")
    # col2im through the ReLU: channels a multiple of 4
    refused(lib.splat_nn_col2im_act3x3(a, b, c, C.c_void_p(0x40000), 1, 8, 8, 6, 2, 56, None),
            "col2im_act3x3")
    # Adam over arrays: at most 16 segments, pointers of non-empty ones
    segs = (_lib.SplatAdamSeg * 17)()
    refused(lib.splat_nn_adam_multi(segs, 17, 1e-3, 1, None), "adam_multi")
    one = (_lib.SplatAdamSeg * 1)(_lib.SplatAdamSeg(None, None, None, None, None, 10))
    refused(lib.splat_nn_adam_multi(one, 1, 1e-3, 1, None), "adam_multi")
    refused(lib.splat_nn_adam_multi(one, 1, 1e-3, 0, None), "adam_multi")  # step >= 1
