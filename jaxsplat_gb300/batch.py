"""Batched multi-view, multi-scene render: many views of several scenes, each
with its own Gaussian count and image size, in one pass of each kernel.

``BatchSession`` owns every buffer of one batch (fixed scenes, views and
image sizes) and enqueues the whole forward+backward -- projection of every
(view, Gaussian) entry, one sort over all views, rasterize forward with
persistent blocks over a longest-list-first tile order, the per-view L2
loss, rasterize backward, projection backward with the scene gradients
summed over each scene's views -- without host read-back, so the step is
captured once as a CUDA graph and replayed.  Each view's image and
gradients equal those of rendering that view alone with ``render``; the
reference renders one view per call (jaxsplat/__init__.py:6-70).

``autotune`` measures the block sizes {8, 12, 16} and several scheduler chunk
sizes on the batch itself and keeps the fastest.
"""

from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from ._buffers import block as _block
from ._ops import _status_word
from .streaming import StreamingSteps


class BatchSession(StreamingSteps):
    """scenes: list of dicts with means3d (N,3), scales (N,3), quats (N,4),
    colors (N,3), opacities (N,1).  views: list of dicts with scene (index),
    viewmat (4,4), img_shape (H, W), f (fx, fy), c (cx, cy) and optionally
    background (3,).  targets: one (H, W, 3) image per view (for the loss)."""

    def __init__(self, scenes, views, targets=None, *, glob_scale: float = 1.0,
                 clip_thresh: float = 0.01, block_size: int = 16, chunk: int = 1,
                 capacity: int | None = None, device="cuda"):
        self.lib = _lib.load()
        self.dev = torch.device(device)
        if self.dev.index is None:
            self.dev = torch.device("cuda", torch.cuda.current_device())
        self.scene_points = [int(np.shape(s["means3d"])[0]) for s in scenes]
        self.view_specs = [dict(v) for v in views]
        self.glob_scale, self.clip_thresh = float(glob_scale), float(clip_thresh)
        self.chunk = int(chunk)
        self.status = _status_word(self.dev)
        G = sum(self.scene_points)
        P = sum(int(v["img_shape"][0]) * int(v["img_shape"][1]) for v in self.view_specs)
        # inputs (scene arrays, targets) and outputs (loss, scene gradients) as
        # single blocks: one host transfer each way per step
        self._io_shapes = (self.input_shapes(G, P), self.output_shapes(G))
        self.inputs, views_in = _block(self._io_shapes[0], self.dev)
        self.outputs, views_out = _block(self._io_shapes[1], self.dev)
        for name, t in list(views_in.items()) + list(views_out.items()):
            setattr(self, name, t)
        for k, w in (("means3d", 3), ("scales", 3), ("quats", 4), ("colors", 3), ("opacities", 1)):
            getattr(self, k).copy_(torch.as_tensor(np.concatenate(
                [np.reshape(np.asarray(s[k], np.float32), (-1, w)) for s in scenes])))
        self.target.zero_()
        self._targets = targets
        self._layout(int(block_size))
        if capacity is not None:
            self._size(int(capacity))

    # -- layout and buffers ----------------------------------------------------
    def _stream_shapes(self):
        return self._io_shapes

    @staticmethod
    def input_shapes(G, P):
        return [("means3d", (G, 3)), ("scales", (G, 3)), ("quats", (G, 4)), ("colors", (G, 3)),
                ("opacities", (G, 1)), ("target", (P, 3))]

    @staticmethod
    def output_shapes(G):
        # final after the rasterizer's backward first, then the projection's
        return [("loss", (1,)), ("v_colors", (G, 3)), ("v_opacity", (G, 1)), ("v_mean3d", (G, 3)),
                ("v_scale", (G, 3)), ("v_quat", (G, 4))]

    def upload(self, host_block):
        """All inputs of a step from a pinned host copy of ``self.inputs``."""
        self.inputs.copy_(host_block, non_blocking=True)

    def download(self, host_block):
        """Loss and scene gradients into a pinned host block shaped like
        ``self.outputs``."""
        host_block.copy_(self.outputs, non_blocking=True)

    def _layout(self, block_size: int):
        n_views = len(self.view_specs)
        arr = (_lib.SplatView * n_views)()
        for k, v in enumerate(self.view_specs):
            sv = arr[k]
            vm = np.asarray(v["viewmat"], np.float32).reshape(16)
            for q in range(16):
                sv.viewmat[q] = float(vm[q])
            sv.fx, sv.fy = float(v["f"][0]), float(v["f"][1])
            sv.cx, sv.cy = float(v["c"][0]), float(v["c"][1])
            bg = np.asarray(v.get("background", (0.0, 0.0, 0.0)), np.float32)
            for q in range(3):
                sv.background[q] = float(bg[q])
            sv.scene = int(v["scene"])
            sv.img_height, sv.img_width = int(v["img_shape"][0]), int(v["img_shape"][1])
        b = _lib.SplatBatch()
        b.num_scenes, b.num_views = len(self.scene_points), n_views
        b.glob_scale, b.clip_thresh, b.block_width = self.glob_scale, self.clip_thresh, block_size
        b.device_status = self.status.data_ptr()
        pts = (C.c_uint32 * len(self.scene_points))(*self.scene_points)
        _lib.check(self.lib.splat_batch_layout(C.byref(b), arr, pts), "batch_layout")
        raw = bytes(C.string_at(C.addressof(arr), C.sizeof(arr)))
        self.view_table = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.dev)
        b.views = self.view_table.data_ptr()
        self.batch, self.views_host, self.bw = b, arr, block_size
        E, T, P, G = b.num_entries, b.num_tiles, b.num_pixels, b.num_points
        dev = self.dev
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        Em = torch.empty
        self.cov3d, self.xys, self.depths = Em(E, 6, **f32), Em(E, 2, **f32), Em(E, 1, **f32)
        self.radii, self.conics, self.comp = Em(E, 1, **i32), Em(E, 3, **f32), Em(E, 1, **f32)
        self.total = torch.zeros(1, dtype=torch.int64, device=dev)
        self.packed = Em(E, 12, **f32)
        self.tile_bins, self.tile_order = Em(T, 2, **i32), Em(T, **i32)
        self.counter = torch.zeros(1, **i32)
        self.final_Ts, self.final_idx = Em(P, 1, **f32), Em(P, 1, **i32)
        self.img, self.v_img = Em(P, 3, **f32), Em(P, 3, **f32)
        self.v_alpha = torch.zeros(P, 1, **f32)
        if self._targets is not None:
            self.set_targets(self._targets)
        self.v_xy, self.v_conic = Em(E, 2, **f32), Em(E, 3, **f32)
        self.capacity = None
        self.graph = None
        self.graph_io = None
        self._stream_graphs = None

    def _size(self, capacity: int):
        self.capacity = max(int(capacity), 1)
        self.ids_sorted = torch.empty(self.capacity, dtype=torch.int32, device=self.dev)
        nbytes = self.lib.splat_batch_sort_workspace_size(C.byref(self.batch), self.capacity)
        if nbytes == 0:
            raise _lib.SplatError("batch sort workspace size query failed: " +
                                  self.lib.splat_last_error().decode())
        self.sort_ws = torch.empty(nbytes, dtype=torch.uint8, device=self.dev)
        self.graph = None
        self.graph_io = None
        self._stream_graphs = None

    def set_targets(self, targets):
        for k, t in enumerate(targets):
            v = self.views_host[k]
            n = v.img_height * v.img_width
            self.target[v.pixel_base:v.pixel_base + n].copy_(
                torch.as_tensor(np.asarray(t, np.float32)).reshape(n, 3))

    def measure_capacity(self, headroom: float = 1.25) -> int:
        self._project()
        torch.cuda.synchronize(self.dev)
        count = int(self.total.item())
        self._size(int(math.ceil(count * headroom)) + 4096)
        return count

    # -- the step -------------------------------------------------------------
    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr())

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _project(self, pack=False):
        P = self._p
        if pack:  # the packed records too (no separate packing pass)
            _lib.check(self.lib.splat_batch_project_fwd_packed(
                C.byref(self.batch), P(self.means3d), P(self.scales), P(self.quats),
                P(self.colors), P(self.opacities), P(self.cov3d), P(self.xys), P(self.depths),
                P(self.radii), P(self.conics), P(self.comp), P(self.total), P(self.packed),
                self._stream()), "batch_project_fwd_packed")
            return
        _lib.check(self.lib.splat_batch_project_fwd(
            C.byref(self.batch), P(self.means3d), P(self.scales), P(self.quats), P(self.cov3d),
            P(self.xys), P(self.depths), P(self.radii), P(self.conics), P(self.comp),
            P(self.total), self._stream()), "batch_project_fwd")

    def step(self, mark=None, side=None):
        """Enqueue one forward+backward of every view (no host sync).  The
        projection writes the packed records too; with ``side`` (a stream on
        which colours, opacities and targets are still arriving, see step_io)
        the packing pass instead runs on it once they and the projection are
        done.  The forward rasterizer computes the per-view L2 loss in its
        epilogue."""
        if self.capacity is None:
            self.measure_capacity()
        P, b, cap, lib = self._p, C.byref(self.batch), self.capacity, self.lib
        cur = torch.cuda.current_stream(self.dev)
        s = C.c_void_p(cur.cuda_stream)
        mark = mark or (lambda name: None)
        chk = _lib.check
        mark("project_fwd")
        self._project(pack=side is None)
        if side is not None:
            projected = torch.cuda.Event()
            projected.record(cur)
            side.wait_event(projected)
            with torch.cuda.stream(side):
                chk(lib.splat_batch_pack(b, P(self.xys), P(self.conics), P(self.colors),
                                         P(self.opacities), P(self.packed),
                                         C.c_void_p(side.cuda_stream)), "batch_pack")
        mark("sort")
        chk(lib.splat_batch_sort_and_bin(b, cap, P(self.total), P(self.xys), P(self.depths),
                                         P(self.radii), P(self.ids_sorted), P(self.tile_bins),
                                         P(self.tile_order), P(self.sort_ws),
                                         self.sort_ws.numel(), s), "batch_sort_and_bin")
        if side is not None:
            cur.wait_stream(side)
        mark("raster_fwd")
        chk(lib.splat_batch_rasterize_fwd_l2(b, cap, P(self.total), P(self.ids_sorted),
                                             P(self.tile_bins), P(self.tile_order),
                                             P(self.packed), P(self.target), P(self.final_Ts),
                                             P(self.final_idx), P(self.img), P(self.v_img),
                                             P(self.loss), self.chunk, P(self.counter), s),
            "batch_rasterize_fwd_l2")
        mark("raster_bwd")
        chk(lib.splat_batch_rasterize_bwd(b, cap, P(self.total), P(self.ids_sorted),
                                          P(self.tile_bins), P(self.tile_order), P(self.packed),
                                          P(self.final_Ts), P(self.final_idx), P(self.v_img),
                                          P(self.v_alpha), P(self.v_colors), P(self.v_opacity),
                                          P(self.v_xy), P(self.v_conic), self.chunk,
                                          P(self.counter), s), "batch_rasterize_bwd")
        mark("project_bwd")
        chk(lib.splat_batch_project_bwd(b, P(self.means3d), P(self.scales), P(self.quats),
                                        P(self.cov3d), P(self.radii), P(self.conics),
                                        P(self.comp), P(self.v_xy), P(self.v_conic),
                                        P(self.v_mean3d), P(self.v_scale), P(self.v_quat), s),
            "batch_project_bwd")
        mark("end")

    def step_io(self, host_in, host_out):
        """One step from a pinned host copy of ``inputs`` to a pinned host
        block the size of ``outputs``, the copies overlapped with the work:
        the projection's inputs first, then colours, opacities and targets on
        a second stream during the projection and sort; loss and colour /
        opacity gradients back on the second stream during the projection
        backward."""
        if self.capacity is None:
            self.measure_capacity()
        cur = torch.cuda.current_stream(self.dev)
        side = self._side = getattr(self, "_side", None) or torch.cuda.Stream(self.dev)
        a_in = (self.colors.data_ptr() - self.inputs.data_ptr()) // 4
        a_out = (self.v_mean3d.data_ptr() - self.outputs.data_ptr()) // 4
        self.inputs[:a_in].copy_(host_in[:a_in], non_blocking=True)
        side.wait_stream(cur)  # after the first half and the previous step
        with torch.cuda.stream(side):
            self.inputs[a_in:].copy_(host_in[a_in:], non_blocking=True)

        def mark(name):
            if name == "project_bwd":
                side.wait_stream(cur)
                with torch.cuda.stream(side):
                    host_out[:a_out].copy_(self.outputs[:a_out], non_blocking=True)

        self.step(mark=mark, side=side)
        host_out[a_out:].copy_(self.outputs[a_out:], non_blocking=True)
        cur.wait_stream(side)

    def capture_io(self, host_in, host_out):
        if self.capacity is None:
            self.measure_capacity()
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            self.step_io(host_in, host_out)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step_io(host_in, host_out)
        self.graph_io = g
        return g

    def replay_io(self):
        self.graph_io.replay()

    def capture(self):
        if self.capacity is None:
            self.measure_capacity()
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            self.step()
        torch.cuda.current_stream(self.dev).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def check(self) -> int:
        torch.cuda.synchronize(self.dev)
        bits = int(self.status.item())
        count = int(self.total.item())
        if bits:
            self.status.zero_()
            msg = self.lib.splat_device_status_string(bits).decode()
            raise _lib.SplatError(f"device status: {msg} (count {count}, capacity "
                                  f"{self.capacity})")
        return count

    # -- results ---------------------------------------------------------------
    def _pix(self, k):
        v = self.views_host[k]
        return v.pixel_base, v.img_height, v.img_width

    def view_image(self, k):
        b, h, w = self._pix(k)
        return self.img[b:b + h * w].reshape(h, w, 3)

    def view_final(self, k):
        b, h, w = self._pix(k)
        return (self.final_Ts[b:b + h * w].reshape(h, w, 1),
                self.final_idx[b:b + h * w].reshape(h, w, 1))

    def view_entries(self, k):
        """Slice of the per-entry arrays that holds view k's Gaussians."""
        v = self.views_host[k]
        return slice(v.entry_base, v.entry_base + v.num_points)

    def scene_slice(self, s):
        base = sum(self.scene_points[:s])
        return slice(base, base + self.scene_points[s])

    def scene_grads(self, s):
        sl = self.scene_slice(s)
        return dict(means3d=self.v_mean3d[sl], scales=self.v_scale[sl], quats=self.v_quat[sl],
                    colors=self.v_colors[sl], opacities=self.v_opacity[sl])

    # -- tuning ----------------------------------------------------------------
    def time_replays(self, steps: int = 5) -> float:
        """Mean ms of `steps` graph replays (after one)."""
        self.replay()
        torch.cuda.synchronize(self.dev)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(steps):
            self.graph.replay()
        t1.record()
        torch.cuda.synchronize(self.dev)
        return t0.elapsed_time(t1) / steps

    def autotune(self, block_sizes=(8, 12, 16), chunks=(1, 2, 4, 8), steps: int = 3,
                 headroom: float = 1.25, log=None):
        """Measure every (block size, chunk) on this batch; keep the fastest.
        Returns {(bw, chunk): ms}."""
        results = {}
        for bw in block_sizes:
            self._layout(int(bw))
            self.measure_capacity(headroom)
            for ch in chunks:
                self.chunk = int(ch)
                self.graph = None
                self._stream_graphs = None
                self.capture()
                ms = self.time_replays(steps)
                self.check()
                results[(int(bw), int(ch))] = ms
                if log:
                    log(f"autotune bw={bw} chunk={ch}: {ms:.3f} ms")
        best_bw, best_chunk = min(results, key=results.get)
        self._layout(best_bw)
        self.measure_capacity(headroom)
        self.chunk = best_chunk
        self.capture()
        self.best = (best_bw, best_chunk)
        return results
