"""A preallocated, synchronisation-free forward+backward of the render path.

``RenderSession`` holds every buffer of one render (fixed Gaussian count,
camera and image size) and enqueues the whole step -- project, sort and bin,
rasterize forward, L2 loss against a target, rasterize backward, project
backward -- without any host read-back: the intersection count stays on the
device (written by the projection's scan, read by the sort and rasterizer
kernels) and the intersection buffers are sized by a capacity.  The step can
therefore be captured once as a CUDA graph and replayed.

Capacity: by default one eager render measures the count and the capacity
is set to 1.25x that (plus a little).  ``check()`` synchronises and raises if
a step's count ever exceeded the capacity (its outputs are then unusable;
build a new session with a larger capacity).

This is the loop of the reference's fitting example
(examples/single_image.py:26-40): ``mean((render(...) - target)**2)`` and its
gradients with respect to means3d, scales, quats, colors and opacities.
"""

from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib
from ._buffers import block as _block
from ._ops import _status_word
from .streaming import StreamingSteps


class RenderSession(StreamingSteps):
    def __init__(self, num_points: int, *, img_shape, f, c, glob_scale: float = 1.0,
                 clip_thresh: float = 0.01, block_size: int = 16, capacity: int | None = None,
                 device="cuda"):
        self.lib = _lib.load()
        self.dev = torch.device(device)
        if self.dev.index is None:
            self.dev = torch.device("cuda", torch.cuda.current_device())
        n = int(num_points)
        h, w = int(img_shape[0]), int(img_shape[1])
        self.n, self.h, self.w, self.bw = n, h, w, int(block_size)
        self.status = _status_word(self.dev)
        self.params = _lib.make_params(n, (h, w), f, c, glob_scale, clip_thresh, block_size,
                                       self.status.data_ptr())
        f32 = dict(dtype=torch.float32, device=self.dev)
        i32 = dict(dtype=torch.int32, device=self.dev)
        E = torch.empty
        # inputs: views of one block, so that a host copy of the whole step's
        # inputs is one transfer (see INPUTS / upload)
        self.inputs, views = _block(self.input_shapes(), self.dev)
        for name, t in views.items():
            setattr(self, name, t)
        # projection
        self.cov3d, self.xys, self.depths = E(n, 6, **f32), E(n, 2, **f32), E(n, 1, **f32)
        self.radii, self.conics, self.comp = E(n, 1, **i32), E(n, 3, **f32), E(n, 1, **f32)
        self.ntiles, self.cum = E(n, 1, **i32), E(n, 1, **i32)
        self.total = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.proj_ws = E(self.lib.splat_project_fwd_workspace_size(C.byref(self.params)),
                         dtype=torch.uint8, device=self.dev)
        # rasterizer
        tiles = ((w + self.bw - 1) // self.bw) * ((h + self.bw - 1) // self.bw)
        self.tile_bins = E(tiles, 2, **i32)
        self.packed = E(n, 12, **f32)
        self.final_Ts, self.final_idx = E(h, w, 1, **f32), E(h, w, 1, **i32)
        self.img = E(h, w, 3, **f32)
        self.v_img = E(h, w, 3, **f32)
        self.v_alpha = torch.zeros(h, w, 1, **f32)
        # loss and gradients: views of one block (one transfer to the host)
        self.outputs, views = _block(self.output_shapes(), self.dev)
        for name, t in views.items():
            setattr(self, name, t)
        self.v_xy, self.v_conic = E(n, 2, **f32), E(n, 3, **f32)
        self.zeros_n1 = torch.zeros(n, 1, **f32)
        self.capacity = None
        self.graph = None
        self.graph_io = None
        self._stream_graphs = None
        if capacity is not None:
            self._size(int(capacity))

    # -- buffers -------------------------------------------------------------
    def _stream_shapes(self):
        return self.input_shapes(), self.output_shapes()

    def input_shapes(self):
        n, h, w = self.n, self.h, self.w
        # what the projection reads first, then what the rasterizer and the
        # loss read (see step_io)
        return [("means3d", (n, 3)), ("scales", (n, 3)), ("quats", (n, 4)), ("viewmat", (4, 4)),
                ("colors", (n, 3)), ("opacities", (n, 1)), ("background", (3,)),
                ("target", (h, w, 3))]

    def output_shapes(self):
        n = self.n
        # what is final after the rasterizer's backward, then the projection's
        return [("loss", (1,)), ("v_colors", (n, 3)), ("v_opacity", (n, 1)), ("v_mean3d", (n, 3)),
                ("v_scale", (n, 3)), ("v_quat", (n, 4))]

    def host_inputs(self, means3d, scales, quats, colors, opacities, viewmat, background, target):
        """A pinned host block laid out like ``self.inputs`` (for ``upload``)."""
        host, views = _block(self.input_shapes(), "cpu", pin=True)
        src = dict(means3d=means3d, scales=scales, quats=quats, colors=colors,
                   opacities=opacities, viewmat=viewmat, background=background, target=target)
        for name, _ in self.input_shapes():
            views[name].copy_(torch.as_tensor(src[name]).reshape(views[name].shape))
        return host

    def upload(self, host_block):
        """All inputs of a step from a pinned host block (one transfer)."""
        self.inputs.copy_(host_block, non_blocking=True)

    def download(self, host_block):
        """Loss and the five gradients into a pinned host block laid out like
        ``self.outputs`` (one transfer)."""
        host_block.copy_(self.outputs, non_blocking=True)

    def _size(self, capacity: int):
        self.capacity = max(int(capacity), 1)
        self.ids_sorted = torch.empty(self.capacity, dtype=torch.int32, device=self.dev)
        # the forward's per-slot warp bytes for the backward (block width 16)
        self.blend = torch.empty(self.capacity, dtype=torch.uint8, device=self.dev)
        nbytes = self.lib.splat_sort_workspace_size(C.byref(self.params), self.capacity)
        self.sort_ws = torch.empty(nbytes, dtype=torch.uint8, device=self.dev)
        self.graph = None
        self.graph_io = None
        self._stream_graphs = None

    def set_inputs(self, means3d, scales, quats, colors, opacities, viewmat, background, target):
        for dst, src in ((self.means3d, means3d), (self.scales, scales), (self.quats, quats),
                         (self.colors, colors), (self.opacities, opacities),
                         (self.viewmat, viewmat), (self.background, background),
                         (self.target, target)):
            dst.copy_(torch.as_tensor(src).reshape(dst.shape), non_blocking=True)

    def measure_capacity(self, headroom: float = 1.25) -> int:
        """One projection with a host read of the count; sizes the buffers."""
        self._project(cum=True)
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

    def _check(self, rc, what):
        _lib.check(rc, what)

    def _project(self, pack=False, cum=False):
        """The projection; the step reads only the intersection total, so
        cum_tiles_hit is written only when asked (the sizing pass)."""
        P, pr = self._p, C.byref(self.params)
        if pack:  # the packed records too (no separate packing pass), and only the
            # intersection count: the step never reads cum_tiles_hit
            self._check(self.lib.splat_project_fwd_packed(
                pr, P(self.means3d), P(self.scales), P(self.quats), P(self.viewmat),
                P(self.colors), P(self.opacities), P(self.cov3d), P(self.xys), P(self.depths),
                P(self.radii), P(self.conics), P(self.comp), P(self.ntiles), None,
                P(self.total), P(self.packed), P(self.proj_ws), self.proj_ws.numel(),
                self._stream()), "project_fwd_packed")
            return
        self._check(self.lib.splat_project_fwd(
            pr, P(self.means3d), P(self.scales), P(self.quats), P(self.viewmat), P(self.cov3d),
            P(self.xys), P(self.depths), P(self.radii), P(self.conics), P(self.comp),
            P(self.ntiles), P(self.cum) if cum else None, P(self.total), P(self.proj_ws),
            self.proj_ws.numel(), self._stream()), "project_fwd")

    def step(self, mark=None, side=None):
        """Enqueue one forward+backward on the current stream (no host sync).
        ``mark(stage)`` is called before each stage and with "end" after the
        last (e.g. to record CUDA events).  The projection writes the packed
        records too; with ``side`` (a stream on which the colours, opacities,
        background and target are still arriving, see step_io) the packing
        pass instead runs on it once they and the projection are done.  The
        forward rasterizer computes the L2 loss in its epilogue."""
        if self.capacity is None:
            self.measure_capacity()
        P, pr, cap = self._p, C.byref(self.params), self.capacity
        lib = self.lib
        cur = torch.cuda.current_stream(self.dev)
        s = C.c_void_p(cur.cuda_stream)
        mark = mark or (lambda name: None)
        mark("project_fwd")
        self._project(pack=side is None)
        if side is not None:
            projected = torch.cuda.Event()
            projected.record(cur)
            side.wait_event(projected)
            with torch.cuda.stream(side):
                self._check(lib.splat_pack_splats(
                    pr, P(self.xys), P(self.conics), P(self.colors), P(self.opacities),
                    P(self.packed), C.c_void_p(side.cuda_stream)), "pack_splats")
        mark("sort")
        self._check(lib.splat_sort_and_bin(
            pr, cap, P(self.total), P(self.xys), P(self.depths), P(self.radii), P(self.cum),
            P(self.ids_sorted), P(self.tile_bins), None, None, None, P(self.sort_ws),
            self.sort_ws.numel(), s), "sort_and_bin")
        if side is not None:
            cur.wait_stream(side)
        mark("raster_fwd")
        self._check(lib.splat_rasterize_fwd_l2(
            pr, cap, P(self.total), P(self.ids_sorted), P(self.tile_bins), P(self.packed),
            P(self.background), P(self.target), P(self.final_Ts), P(self.final_idx),
            P(self.img), P(self.v_img), P(self.loss), P(self.blend), s), "rasterize_fwd_l2")
        mark("raster_bwd")
        self._check(lib.splat_rasterize_bwd(
            pr, cap, P(self.total), P(self.ids_sorted), P(self.tile_bins), P(self.packed),
            P(self.background), P(self.final_Ts), P(self.final_idx), P(self.v_img),
            P(self.v_alpha), P(self.v_colors), P(self.v_opacity), P(self.v_xy), None,
            P(self.v_conic), P(self.blend), s), "rasterize_bwd")
        mark("project_bwd")
        self._check(lib.splat_project_bwd(
            pr, P(self.means3d), P(self.scales), P(self.quats), P(self.viewmat), P(self.cov3d),
            P(self.radii), P(self.conics), P(self.comp), P(self.v_xy), P(self.zeros_n1),
            P(self.v_conic), P(self.zeros_n1), P(self.v_mean3d), P(self.v_scale),
            P(self.v_quat), None, None, s), "project_bwd")  # the cov cotangents are not returned
        mark("end")

    def count_pairs(self):
        """Work counts of the last step (diagnostic, synchronises): pixel-Gaussian
        pairs the reference's forward and backward evaluate, the contributing
        ones, and (tile, Gaussian) pairs with a contributing pixel
        (splat_count_pairs)."""
        out = torch.zeros(4, dtype=torch.int64, device=self.dev)
        P = self._p
        self._check(self.lib.splat_count_pairs(
            C.byref(self.params), self.capacity, P(self.total), P(self.ids_sorted),
            P(self.tile_bins), P(self.packed), P(self.final_idx), P(out), self._stream()),
            "count_pairs")
        c = [int(x) for x in out.cpu().tolist()]
        return {"fwd_evaluated": c[0], "bwd_evaluated": c[1], "bwd_contributing": c[2],
                "tile_gaussian_contributing": c[3]}

    def _split(self, buf, first):
        """Offset in `buf` (a block) of the view named `first`."""
        return (getattr(self, first).data_ptr() - buf.data_ptr()) // 4

    def step_io(self, host_in, host_out):
        """One step from a pinned host input block (``host_inputs``) to a
        pinned host output block (the size of ``outputs``), with the copies
        overlapped: the projection's inputs go first and the rest (colours,
        opacities, background, target) on a second stream while the
        projection and the sort run; loss and colour/opacity gradients go
        back on the second stream while the projection backward runs."""
        if self.capacity is None:
            self.measure_capacity()
        cur = torch.cuda.current_stream(self.dev)
        side = self._side = getattr(self, "_side", None) or torch.cuda.Stream(self.dev)
        a_in = self._split(self.inputs, "colors")
        a_out = self._split(self.outputs, "v_mean3d")
        self.inputs[:a_in].copy_(host_in[:a_in], non_blocking=True)
        # the second half follows the first (copies in parallel would share the
        # link and delay the projection) but overlaps the projection and sort;
        # waiting on `cur` also orders it after the previous step's readers.
        # The packing pass follows it on the same stream, and the rasterizer
        # waits for both.
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            self.inputs[a_in:].copy_(host_in[a_in:], non_blocking=True)
        def mark(name):
            if name == "project_bwd":  # colour/opacity gradients are final
                side.wait_stream(cur)
                with torch.cuda.stream(side):
                    host_out[:a_out].copy_(self.outputs[:a_out], non_blocking=True)

        self.step(mark=mark, side=side)
        host_out[a_out:].copy_(self.outputs[a_out:], non_blocking=True)
        cur.wait_stream(side)

    def capture_io(self, host_in, host_out):
        """Capture step_io(host_in, host_out) as a CUDA graph (after one eager
        warm-up); replay with replay_io()."""
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
        """Capture step() as a CUDA graph (after one eager warm-up step)."""
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
        """Synchronise; raise if any step overflowed or a device check fired.
        Returns the last step's intersection count."""
        torch.cuda.synchronize(self.dev)
        bits = int(self.status.item())
        count = int(self.total.item())
        if bits:
            self.status.zero_()
            msg = self.lib.splat_device_status_string(bits).decode()
            raise _lib.SplatError(f"device status: {msg} (count {count}, capacity "
                                  f"{self.capacity})")
        return count

    @property
    def grads(self):
        return dict(means3d=self.v_mean3d, scales=self.v_scale, quats=self.v_quat,
                    colors=self.v_colors, opacities=self.v_opacity)
