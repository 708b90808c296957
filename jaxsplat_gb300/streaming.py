"""Consecutive steps with the host copies overlapped (double-buffered I/O).

A session's step reads one input block and writes one output block (views of
single buffers, so that each direction is one host transfer).  ``stream_step``
gives every step its own upload and download but lets step i+1's upload and
step i's download run while step i computes: the session gets a second input
block and a second output block, and one CUDA graph of its ``step()`` per
block pair; the intermediate buffers are shared, since the steps' computations
stay in order on one stream.

Ordering (k = i mod 2): step i's upload waits for step i-2's computation (the
last reader of input block k); step i's computation waits for its upload and
for step i-2's download (the last reader of output block k); its download
waits for its computation.
"""

from __future__ import annotations

import torch

from ._buffers import block


class StreamingSteps:
    """Mixin for RenderSession and BatchSession.  The host class provides
    ``inputs`` / ``outputs`` (blocks), ``_stream_shapes()`` -> (input shapes,
    output shapes), ``step()``, ``capacity`` / ``measure_capacity()``, ``dev``
    and ``check()``, and sets ``_stream_graphs = None`` whenever its buffers
    change."""

    _stream_graphs = None

    def _bind(self, k: int):
        """Point the input and output views at block pair k."""
        self.inputs, self.outputs = self._in_blocks[k], self._out_blocks[k]
        for name, t in list(self._in_views[k].items()) + list(self._out_views[k].items()):
            setattr(self, name, t)

    def capture_stream(self):
        """Prepare ``stream_step`` (second block pair, two graphs)."""
        if self.capacity is None:
            self.measure_capacity()
        if self._stream_graphs is not None:
            return
        if getattr(self, "_in_blocks", None) is None:
            ins, outs = self._stream_shapes()
            views_in = {name: getattr(self, name) for name, _ in ins}
            views_out = {name: getattr(self, name) for name, _ in outs}
            in1, vin1 = block(ins, self.dev)
            out1, vout1 = block(outs, self.dev)
            self._in_blocks, self._out_blocks = [self.inputs, in1], [self.outputs, out1]
            self._in_views, self._out_views = [views_in, vin1], [views_out, vout1]
            self._copy_in = torch.cuda.Stream(self.dev)
            self._copy_out = torch.cuda.Stream(self.dev)
            ev = lambda: [torch.cuda.Event(), torch.cuda.Event()]
            self._in_done, self._comp_done, self._out_done = ev(), ev(), ev()
        self._in_blocks[1].copy_(self._in_blocks[0])
        graphs = []
        for k in (0, 1):
            self._bind(k)
            side = torch.cuda.Stream(self.dev)  # warm-up outside the capture
            side.wait_stream(torch.cuda.current_stream(self.dev))
            with torch.cuda.stream(side):
                self.step()
            torch.cuda.current_stream(self.dev).wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self.step()
            graphs.append(g)
        self._bind(0)
        self._stream_graphs = graphs
        self._stream_i = 0

    def stream_step(self, host_in, host_out):
        """Enqueue one step from pinned ``host_in`` (laid out like ``inputs``)
        to pinned ``host_out`` (like ``outputs``) without waiting for the
        previous steps; ``stream_sync()`` orders the current stream after all
        of them."""
        if self._stream_graphs is None:
            self.capture_stream()
        k = self._stream_i & 1
        cur = torch.cuda.current_stream(self.dev)
        cin, cout = self._copy_in, self._copy_out
        cin.wait_event(self._comp_done[k])
        with torch.cuda.stream(cin):
            self._in_blocks[k].copy_(host_in, non_blocking=True)
        self._in_done[k].record(cin)
        cur.wait_event(self._in_done[k])
        cur.wait_event(self._out_done[k])
        self._stream_graphs[k].replay()
        self._comp_done[k].record(cur)
        cout.wait_event(self._comp_done[k])
        with torch.cuda.stream(cout):
            host_out.copy_(self._out_blocks[k], non_blocking=True)
        self._out_done[k].record(cout)
        self._stream_i += 1

    def stream_sync(self):
        """Order the current stream after every step ``stream_step`` enqueued."""
        if self._stream_graphs is not None:
            torch.cuda.current_stream(self.dev).wait_stream(self._copy_out)
