"""Single-image fitting on this library's kernels -- the loop of the
reference's examples/single_image.py:10-69 as one CUDA-graph step.

Per step: map the raw parameters (quats normalised, colors and opacities
through a sigmoid, single_image.py:143-148), render, L2 loss against the
target, backward, Adam (lr 1e-2 by default, optax defaults) on the raw
parameters.  Initialisation follows single_image.py:72-140 (drawn with numpy
from a seed: jax.random streams cannot be reproduced without jax): means in
[-6, 6] x [-6, 6] x [-1, 1], scales in [0, 0.5], uniformly random unit
quaternions, raw colors in [0, 1], raw opacities in [0.5, 1]; camera at
z = -8 looking down +z, f = c = (W / 2, H / 2), black background.

The intersection buffers are sized with headroom and checked every
``check_every`` steps: when the count nears the capacity the buffers grow and
the step is captured again; a step that overflowed raises.
"""

from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from .session import RenderSession


def random_init(num_points: int, seed: int = 0) -> dict:
    """Raw parameters drawn like single_image.py:72-140."""
    rng = np.random.default_rng(seed)
    n = num_points
    means = rng.uniform([-6.0, -6.0, -1.0], [6.0, 6.0, 1.0], (n, 3)).astype(np.float32)
    scales = rng.uniform(0.0, 0.5, (n, 3)).astype(np.float32)
    u, v, w = rng.uniform(size=(3, n, 1))
    quats = np.hstack([np.sqrt(1 - u) * np.sin(2 * np.pi * v), np.sqrt(1 - u) * np.cos(2 * np.pi * v),
                       np.sqrt(u) * np.sin(2 * np.pi * w), np.sqrt(u) * np.cos(2 * np.pi * w)])
    colors = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    opac = rng.uniform(0.5, 1.0, (n, 1)).astype(np.float32)
    return dict(means3d=means, scales=scales, quats=quats.astype(np.float32), colors=colors,
                opacities=opac)


def random_init_device(num_points: int, seed: int, device) -> dict:
    """random_init's distributions drawn on the device (torch's generator,
    so not the same numbers as the numpy draw of the same seed): no host
    work and no upload when a reused fitter restarts."""
    g = torch.Generator(device=device).manual_seed(int(seed))
    n = num_points
    f32 = dict(dtype=torch.float32, device=device, generator=g)
    lo = torch.tensor([-6.0, -6.0, -1.0], device=device)
    hi = torch.tensor([6.0, 6.0, 1.0], device=device)
    means = lo + (hi - lo) * torch.rand(n, 3, **f32)
    scales = 0.5 * torch.rand(n, 3, **f32)
    u, v, w = torch.rand(3, n, 1, **f32)
    two_pi = 2.0 * math.pi
    quats = torch.cat([torch.sqrt(1 - u) * torch.sin(two_pi * v),
                       torch.sqrt(1 - u) * torch.cos(two_pi * v),
                       torch.sqrt(u) * torch.sin(two_pi * w), torch.sqrt(u) * torch.cos(two_pi * w)],
                      dim=1)
    colors = torch.rand(n, 3, **f32)
    opac = 0.5 + 0.5 * torch.rand(n, 1, **f32)
    return dict(means3d=means, scales=scales, quats=quats, colors=colors, opacities=opac)


def camera(img_shape):
    h, w = img_shape
    viewmat = np.eye(4, dtype=np.float32)
    viewmat[2, 3] = 8.0
    return dict(viewmat=viewmat, f=(w / 2.0, h / 2.0), c=(w / 2.0, h / 2.0), glob_scale=1.0,
                clip_thresh=0.01)


def psnr(mse: float) -> float:
    return float("inf") if mse <= 0 else -10.0 * math.log10(mse)


class Fitter:
    def __init__(self, target, num_points: int | None = None, *, init: dict | None = None,
                 seed: int = 0, lr: float = 1e-2, block_size: int = 16, device="cuda",
                 headroom: float = 1.5):
        self.lib = _lib.load()
        tgt = torch.as_tensor(np.asarray(target, np.float32))
        h, w = int(tgt.shape[0]), int(tgt.shape[1])
        if init is None:
            init = random_init(int(num_points), seed)
        n = int(np.shape(init["means3d"])[0])
        self.n, self.lr, self.headroom = n, float(lr), float(headroom)
        cam = camera((h, w))
        self.sess = RenderSession(n, img_shape=(h, w), f=cam["f"], c=cam["c"],
                                  glob_scale=cam["glob_scale"], clip_thresh=cam["clip_thresh"],
                                  block_size=block_size, device=device)
        dev = self.sess.dev
        f32 = dict(dtype=torch.float32, device=dev)
        self.quats_raw = torch.as_tensor(init["quats"], **f32).contiguous().clone()
        self.colors_raw = torch.as_tensor(init["colors"], **f32).contiguous().clone()
        self.opac_raw = torch.as_tensor(np.reshape(init["opacities"], (n, 1)), **f32).contiguous().clone()
        s = self.sess
        s.set_inputs(init["means3d"], init["scales"], s.quats, s.colors, s.opacities, cam["viewmat"],
                     np.zeros(3, np.float32), tgt)
        self.m = torch.zeros(n, 14, **f32)
        self.v = torch.zeros(n, 14, **f32)
        self.step_count = torch.zeros(1, dtype=torch.int32, device=dev)
        self.steps_done = 0
        self.graph = None
        self._transform()
        s.measure_capacity(self.headroom)

    def reset(self, target=None, init: dict | None = None, seed: int = 0):
        """Start a new fit in the same buffers (the captured graph stays
        valid): a new target and/or new raw parameters (host arrays or device
        tensors; random, drawn on the device, if not given), Adam state
        cleared."""
        s = self.sess
        if target is not None:
            t = target if isinstance(target, torch.Tensor) else torch.as_tensor(np.asarray(target, np.float32))
            s.target.copy_(t.reshape(s.target.shape))
        if init is None:
            init = random_init_device(self.n, seed, s.dev)

        def load(dst, x, cols):
            # device tensors are copied on the device; host arrays uploaded
            if isinstance(x, torch.Tensor):
                dst.copy_(x.reshape(self.n, cols))
            else:
                dst.copy_(torch.as_tensor(np.asarray(x, np.float32)).reshape(self.n, cols))

        load(s.means3d, init["means3d"], 3)
        load(s.scales, init["scales"], 3)
        load(self.quats_raw, init["quats"], 4)
        load(self.colors_raw, init["colors"], 3)
        load(self.opac_raw, init["opacities"], 1)
        self.m.zero_()
        self.v.zero_()
        self.step_count.zero_()
        self.steps_done = 0
        self._transform()
        # the new parameters may hit more tiles: size the buffers for them
        s._project()
        torch.cuda.synchronize(s.dev)
        count = int(s.total.item())
        if count > 0.8 * s.capacity:
            s._size(int(count * self.headroom) + 4096)
            self.graph = None

    def _p(self, t):
        return C.c_void_p(t.data_ptr())

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.sess.dev).cuda_stream)

    def _transform(self):
        s, P = self.sess, self._p
        _lib.check(self.lib.splat_fit_transform(self.n, P(self.quats_raw), P(self.colors_raw),
                                                P(self.opac_raw), P(s.quats), P(s.colors),
                                                P(s.opacities), self._stream()), "fit_transform")

    def _step(self):
        s, P = self.sess, self._p
        self._transform()
        s.step()
        _lib.check(self.lib.splat_fit_adam(
            self.n, self.lr, P(self.step_count), P(s.means3d), P(s.scales), P(self.quats_raw),
            P(self.colors_raw), P(self.opac_raw), P(self.m), P(self.v), P(s.v_mean3d),
            P(s.v_scale), P(s.v_quat), P(s.v_colors), P(s.v_opacity), P(s.quats), P(s.colors),
            P(s.opacities), self._stream()), "fit_adam")

    def capture(self):
        dev = self.sess.dev
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        # warm-up outside the graph: one real step
        with torch.cuda.stream(side):
            self._step()
        torch.cuda.current_stream(dev).wait_stream(side)
        self.steps_done += 1
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._step()
        self.graph = g

    def run(self, steps: int):
        """Enqueue `steps` fitting steps (graph replays); no host sync."""
        if self.graph is None:
            self.capture()
        for _ in range(steps):
            self.graph.replay()
        self.steps_done += steps

    def check(self) -> float:
        """Synchronise, grow the buffers if the count nears capacity, and
        return the PSNR of the last rendered image."""
        count = self.sess.check()
        if count > 0.8 * self.sess.capacity:
            self.sess._size(int(count * self.headroom) + 4096)
            self.graph = None
        return psnr(float(self.sess.loss.item()))

    def fit_until(self, target_psnr: float = 30.0, max_steps: int = 2000, check_every: int = 25):
        """Run until the rendered image reaches target_psnr (dB) or max_steps.
        Returns (reached, steps, seconds, psnr)."""
        torch.cuda.synchronize(self.sess.dev)
        t0 = time.perf_counter()
        p = float("-inf")
        while self.steps_done < max_steps:
            self.run(min(check_every, max_steps - self.steps_done))
            p = self.check()
            if p >= target_psnr:
                break
        return p >= target_psnr, self.steps_done, time.perf_counter() - t0, p

    def params(self) -> dict:
        """Current raw parameters (device tensors)."""
        s = self.sess
        return dict(means3d=s.means3d, scales=s.scales, quats=self.quats_raw,
                    colors=self.colors_raw, opacities=self.opac_raw)

    def check_render(self) -> float:
        """PSNR of the current parameters' render (one eager step; the
        parameters are not updated)."""
        self._transform()
        self.sess.step()
        torch.cuda.synchronize(self.sess.dev)
        return psnr(float(self.sess.loss.item()))

    def render(self):
        """The image of the current parameters."""
        self._transform()
        self.sess.step()
        torch.cuda.synchronize(self.sess.dev)
        return self.sess.img
