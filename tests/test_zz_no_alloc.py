"""splat_project_fwd_noalloc: the projection forward for callers that cannot
allocate device memory (a plugin whose host pools all device memory, or a
handler inside another runtime where cudaMalloc is not allowed).

It is called through the C ABI and must give exactly what the workspace
entry point splat_project_fwd gives on the same inputs, on two calls in a
row: the second call is smaller than the first, so anything the shared
fixed scratch kept from the first call and failed to clear would show up.
This file is collected last so a failure here comes after every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OUT_KEYS = ("cov3d", "xys", "depths", "radii", "conics", "compensation", "num_tiles_hit",
            "cum_tiles_hit", "total")


def _alloc_outputs(torch, n):
    f32 = dict(dtype=torch.float32, device="cuda")
    i32 = dict(dtype=torch.int32, device="cuda")
    return dict(cov3d=torch.full((n, 6), -7.0, **f32), xys=torch.full((n, 2), -7.0, **f32),
                depths=torch.full((n, 1), -7.0, **f32), radii=torch.full((n, 1), -7, **i32),
                conics=torch.full((n, 3), -7.0, **f32),
                compensation=torch.full((n, 1), -7.0, **f32),
                num_tiles_hit=torch.full((n, 1), -7, **i32),
                cum_tiles_hit=torch.full((n, 1), -7, **i32),
                total=torch.full((1,), -7, dtype=torch.int64, device="cuda"))


def _run(lib, torch, p, inputs, use_noalloc, with_total=True):
    n = inputs[0].shape[0]
    out = _alloc_outputs(torch, n)
    ptrs = [C.c_void_p(t.data_ptr()) for t in inputs] + \
           [C.c_void_p(out[k].data_ptr()) for k in OUT_KEYS]
    if not with_total:
        # no total_out: the total goes to the scratch array's last word
        ptrs[-1] = None
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if use_noalloc:
        rc = lib.splat_project_fwd_noalloc(C.byref(p), *ptrs, stream)
    else:
        nbytes = lib.splat_project_fwd_workspace_size(C.byref(p))
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        rc = lib.splat_project_fwd(C.byref(p), *ptrs, C.c_void_p(ws.data_ptr()), nbytes, stream)
    assert rc == 0, lib.splat_last_error()
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_noalloc_matches_workspace_entry_point_twice():
    import torch

    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300.scenes import make_scene

    lib = _lib.load()
    for n, seed, shape in ((100_000, 3, (256, 256)), (20_000, 4, (128, 160))):
        sc = make_scene("small", seed=seed, num_points=n, img_shape=shape)
        kw = sc.kwargs
        p = _lib.make_params(n, kw["img_shape"], kw["f"], kw["c"], kw["glob_scale"],
                             kw["clip_thresh"], 16)
        inputs = [torch.from_numpy(getattr(sc, k)).cuda()
                  for k in ("means3d", "scales", "quats", "viewmat")]
        want = _run(lib, torch, p, inputs, use_noalloc=False)
        got = _run(lib, torch, p, inputs, use_noalloc=True)
        for k in OUT_KEYS:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"N={n} {k}")
        assert int(got["total"][0]) == int(want["cum_tiles_hit"][-1, 0]) > 0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    p = _lib.make_params((1 << 24) + 1, (64, 64), (64.0, 64.0), (32.0, 32.0), 1.0, 0.01, 16)
    rc = lib.splat_project_fwd_noalloc(C.byref(p), *([None] * 13), None)
    assert rc == 1
    assert b"at most 16777216" in lib.splat_last_error()


def test_noalloc_without_total_and_without_allocating():
    """total_out = NULL (the total lands in the library's own scratch), and
    a call after the first leaves the device's free memory and torch's
    allocator untouched."""
    import torch

    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300.scenes import make_scene

    lib = _lib.load()
    sc = make_scene("small", seed=5, num_points=50_000, img_shape=(200, 240))
    kw = sc.kwargs
    p = _lib.make_params(50_000, kw["img_shape"], kw["f"], kw["c"], kw["glob_scale"],
                         kw["clip_thresh"], 16)
    inputs = [torch.from_numpy(getattr(sc, k)).cuda()
              for k in ("means3d", "scales", "quats", "viewmat")]
    want = _run(lib, torch, p, inputs, use_noalloc=False)
    _run(lib, torch, p, inputs, use_noalloc=True, with_total=False)  # first call: set-up
    n = 50_000
    out = _alloc_outputs(torch, n)
    ptrs = [C.c_void_p(t.data_ptr()) for t in inputs] + \
           [C.c_void_p(out[k].data_ptr()) for k in OUT_KEYS[:-1]] + [None]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = (torch.cuda.memory_allocated(), torch.cuda.memory_reserved())
    rc = lib.splat_project_fwd_noalloc(C.byref(p), *ptrs, stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = (torch.cuda.memory_allocated(), torch.cuda.memory_reserved())
    assert rc == 0, lib.splat_last_error()
    assert free1 == free0, (free0, free1)
    assert stats1 == stats0
    got = {k: v.cpu().numpy() for k, v in out.items()}
    for k in OUT_KEYS[:-1]:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    assert int(got["total"][0]) == -7  # untouched: no total_out was given
