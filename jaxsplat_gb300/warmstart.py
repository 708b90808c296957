"""Learned warm start for single-image fitting.

A small convolutional network looks at a 512x512 target image and proposes
all 16384 Gaussians of the fit at once: an encoder of four 3x3 stride-2
convolutions 3->32->64->128->256 (ReLU, BF16 activations and weights, FP32
accumulation) down to a 32x32 grid, and a 1x1 convolution head emitting, per
grid cell, 16 Gaussians x 14 raw parameters.  Every convolution runs as
im2col + the tcgen05 BF16 GEMM of this library (gemm_tc.cu), forward and
backward; in the forward the bias, ReLU and bf16 conversion run in the
GEMM's epilogue.  The surrounding gathers, ReLU gradient and Adam are this
library's kernels too (nn.cu).  torch only holds the buffers.

Training data is what the plain fitting loop itself produces (``Fitter``
from random init on procedural targets): each fitted set is put on the grid
-- a Gaussian goes to the cell that contains its projected centre, a cell
keeps its 16 most opaque Gaussians (empty slots are transparent
placeholders) -- and the network regresses the standardised per-slot
parameters (centre offset within the cell in cell units, depth, |scales|,
sign-normalised unit quaternion, raw colours, raw opacity) with an MSE loss.

Plain fitting from random init stays both the fallback and the yardstick: the
measurement is wall-clock to 30 dB PSNR from the network's proposal versus
from random init, on held-out seeds.
"""

from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from .fit import Fitter, camera, random_init

GRID = 32           # cells per side
SLOTS = 16          # Gaussians per cell
NPARAM = 14         # raw parameters per Gaussian
IMG = 512
CELL = IMG // GRID  # pixels per cell side
CHANNELS = (3, 32, 64, 128, 256)


def _p(t):
    return C.c_void_p(t.data_ptr())


def _kpad(cin):
    return (9 * cin + 7) // 8 * 8


class ConvNet:
    """The encoder + head with fp32 master weights, bf16 copies and Adam
    state; forward/backward through libsplat's kernels on the current
    stream."""

    def __init__(self, device="cuda", seed: int = 0):
        self.lib = _lib.load()
        self.dev = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.layers = []
        for cin, cout in zip(CHANNELS[:-1], CHANNELS[1:]):
            kp = _kpad(cin)
            w = torch.zeros(cout, kp)
            w[:, :9 * cin] = torch.randn(cout, 9 * cin, generator=g) * math.sqrt(2.0 / (9 * cin))
            self.layers.append(self._param(w, torch.zeros(cout), cin, cout, kp))
        wh = torch.randn(SLOTS * NPARAM, CHANNELS[-1], generator=g) * math.sqrt(1.0 / CHANNELS[-1])
        self.head = self._param(wh, torch.zeros(SLOTS * NPARAM), CHANNELS[-1], SLOTS * NPARAM,
                                CHANNELS[-1])
        # the bias gradients (accumulated by atomics) share one buffer, zeroed
        # once per backward; the weight gradients are overwritten by their GEMMs
        params = self.layers + [self.head]
        self.gb_flat = torch.zeros(sum(prm["b"].numel() for prm in params), device=self.dev)
        off = 0
        for prm in params:
            nb = prm["b"].numel()
            prm["gb"] = self.gb_flat[off:off + nb]
            off += nb
        # every weight and bias array as one segment of a single Adam launch
        segs = []
        for prm in params:
            segs.append(_lib.SplatAdamSeg(prm["w"].data_ptr(), prm["mw"].data_ptr(),
                                          prm["vw"].data_ptr(), prm["gw"].data_ptr(),
                                          prm["w16"].data_ptr(), prm["w"].numel()))
            segs.append(_lib.SplatAdamSeg(prm["b"].data_ptr(), prm["mb"].data_ptr(),
                                          prm["vb"].data_ptr(), prm["gb"].data_ptr(), None,
                                          prm["b"].numel()))
        self._adam_segs = (_lib.SplatAdamSeg * len(segs))(*segs)
        self.step_count = 0
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)

    def _param(self, w, b, cin, cout, k):
        d = self.dev
        w = w.to(d).contiguous()
        return dict(w=w, w16=w.to(torch.bfloat16).contiguous(), b=b.to(d).contiguous(),
                    mw=torch.zeros_like(w), vw=torch.zeros_like(w), mb=torch.zeros_like(b.to(d)),
                    vb=torch.zeros_like(b.to(d)), gw=torch.zeros_like(w),
                    gb=torch.zeros_like(b.to(d)), cin=cin, cout=cout, k=k)

    # -- primitives ------------------------------------------------------------
    def _s(self):
        return C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def gemm(self, A, B, Cm, M, N, K, lda, ldb, ldc, acc=False):
        _lib.check(self.lib.splat_gemm_bf16(_p(A), _p(B), _p(Cm), M, N, K, lda, ldb, ldc, int(acc),
                                            _p(self.status), self._s()), "gemm_bf16")

    def gemm_mn(self, A, a_mn, B, b_mn, Cm, M, N, K, lda, ldb, ldc):
        """Cm = op(A) op(B)^T with A stored [K, M] when a_mn (else [M, K]) and
        B stored [K, N] when b_mn (else [N, K])."""
        _lib.check(self.lib.splat_gemm_bf16_mn(_p(A), int(a_mn), _p(B), int(b_mn), _p(Cm), M, N, K,
                                               lda, ldb, ldc, 0, _p(self.status), self._s()),
                   "gemm_bf16_mn")

    def gemm_bias_act(self, A, B, bias, M, N, K, relu, bf16_out=True):
        """act(A B^T + bias) with the bias, ReLU and output conversion fused
        into the GEMM's epilogue: (M, N) bf16 (or fp32)."""
        y = torch.empty(M, N, dtype=torch.bfloat16 if bf16_out else torch.float32,
                        device=self.dev)
        _lib.check(self.lib.splat_gemm_bf16_bias_act(
            _p(A), _p(B), _p(bias), _p(y) if bf16_out else None, None if bf16_out else _p(y),
            M, N, K, K, K, N, int(relu), _p(self.status), self._s()), "gemm_bf16_bias_act")
        return y

    # -- forward / backward ------------------------------------------------------
    def forward(self, x):
        """x: (B, 512, 512, 3) bf16 NHWC -> (B*32*32, 224) fp32."""
        lib, s = self.lib, self._s()
        B = x.shape[0]
        h = x.shape[1]
        self.saved = []
        cur = x.contiguous()
        for L in self.layers:
            ho = (h - 1) // 2 + 1
            P = B * ho * ho
            cols = torch.empty(P, L["k"], dtype=torch.bfloat16, device=self.dev)
            _lib.check(lib.splat_nn_im2col3x3(_p(cur), _p(cols), B, h, h, L["cin"], 2, L["k"], s),
                       "im2col3x3")
            y = self.gemm_bias_act(cols, L["w16"], L["b"], P, L["cout"], L["k"], relu=True)
            self.saved.append((cols, y, h, ho, P))
            cur, h = y, ho
        Hd = self.head
        P = cur.shape[0]
        out = self.gemm_bias_act(cur, Hd["w16"], Hd["b"], P, Hd["cout"], Hd["k"], relu=False,
                                 bf16_out=False)
        self.head_in = cur
        self.batch = B
        return out

    def backward(self, dout):
        """dout: d(loss)/d(forward output), fp32; sets every parameter's
        gradient."""
        lib, s = self.lib, self._s()
        B = self.batch
        Hd = self.head
        P = dout.shape[0]
        self.gb_flat.zero_()
        dz = torch.empty(P, Hd["cout"], dtype=torch.bfloat16, device=self.dev)
        _lib.check(lib.splat_nn_act_grad(_p(dout), None, _p(dz), _p(Hd["gb"]), P, Hd["cout"], 0, s),
                   "act_grad")
        # dWh = dz^T y4 (both stored pixel-major: MN-major operands);
        # dy4 = dz Wh (Wh as stored: MN-major B)
        self.gemm_mn(dz, True, self.head_in, True, Hd["gw"], Hd["cout"], Hd["k"], P,
                     Hd["cout"], Hd["k"], Hd["k"])
        dy = torch.empty(P, Hd["k"], device=self.dev)
        self.gemm_mn(dz, False, Hd["w16"], True, dy, P, Hd["k"], Hd["cout"], Hd["cout"], Hd["k"],
                     Hd["k"])
        L = self.layers[-1]
        y, P = self.saved[-1][1], self.saved[-1][4]
        dz = torch.empty(P, L["cout"], dtype=torch.bfloat16, device=self.dev)
        _lib.check(lib.splat_nn_act_grad(_p(dy), _p(y), _p(dz), _p(L["gb"]), P, L["cout"], 1, s),
                   "act_grad")
        for i in range(len(self.layers) - 1, -1, -1):
            L = self.layers[i]
            cols, y, h, ho, P = self.saved[i]
            self.gemm_mn(dz, True, cols, True, L["gw"], L["cout"], L["k"], P, L["cout"], L["k"],
                         L["k"])
            if i == 0:
                break
            dcols = torch.empty(P, L["k"], device=self.dev)
            self.gemm_mn(dz, False, L["w16"], True, dcols, P, L["k"], L["cout"], L["cout"], L["k"],
                         L["k"])
            # col2im through the previous layer's ReLU: that layer's dz
            prev = self.layers[i - 1]
            dz = torch.empty(B * h * h, L["cin"], dtype=torch.bfloat16, device=self.dev)
            _lib.check(lib.splat_nn_col2im_act3x3(_p(dcols), _p(self.saved[i - 1][1]), _p(dz),
                                                  _p(prev["gb"]), B, h, h, L["cin"], 2, L["k"], s),
                       "col2im_act3x3")

    def adam(self, lr: float):
        self.step_count += 1
        _lib.check(self.lib.splat_nn_adam_multi(self._adam_segs, len(self._adam_segs), lr,
                                                self.step_count, self._s()), "adam_multi")

    def check(self):
        torch.cuda.synchronize(self.dev)
        if int(self.status.item()):
            raise _lib.SplatError("warm-start network: a tensor-core wait ran out")


# ---------------------------------------------------------------------------
# Fitted sets <-> the grid.

def _cam():
    cam = camera((IMG, IMG))
    return cam["f"][0], cam["f"][1], cam["c"][0], cam["c"][1], float(cam["viewmat"][2, 3])


def to_grid(params: dict) -> np.ndarray:
    """A fitted set (raw parameters) -> (32*32, 16*14) per-slot parameters:
    offset of the projected centre from the cell centre (cell units), depth
    coordinate z, |scales|, sign-normalised unit quaternion, raw colours, raw
    opacity (clipped to [-8, 8]); empty slots are transparent (opacity -8)."""
    fx, fy, cx, cy, tz = _cam()
    m = np.asarray(params["means3d"], np.float64)
    zc = m[:, 2] + tz
    px = fx * m[:, 0] / zc + cx
    py = fy * m[:, 1] / zc + cy
    gx = np.clip(np.floor(px / CELL), 0, GRID - 1).astype(np.int64)
    gy = np.clip(np.floor(py / CELL), 0, GRID - 1).astype(np.int64)
    q = np.asarray(params["quats"], np.float64)
    q = q / np.maximum(np.linalg.norm(q, axis=1, keepdims=True), 1e-12)
    q *= np.where(q[:, :1] < 0, -1.0, 1.0)
    op = np.clip(np.asarray(params["opacities"], np.float64).reshape(-1), -8.0, 8.0)
    feat = np.concatenate([
        (px / CELL - gx - 0.5)[:, None], (py / CELL - gy - 0.5)[:, None], m[:, 2:3],
        np.abs(np.asarray(params["scales"], np.float64)), q,
        np.asarray(params["colors"], np.float64), op[:, None]], axis=1)
    out = np.tile(empty_slot(), (GRID * GRID, SLOTS, 1))
    cell = gy * GRID + gx
    order = np.lexsort((-op, cell))  # by cell, most opaque first
    cell_sorted = cell[order]
    starts = np.searchsorted(cell_sorted, np.arange(GRID * GRID))
    rank = np.arange(len(order)) - starts[cell_sorted]
    keep = rank < SLOTS
    out[cell_sorted[keep], rank[keep]] = feat[order[keep]]
    return out.reshape(GRID * GRID, SLOTS * NPARAM).astype(np.float32)


def empty_slot() -> np.ndarray:
    return np.array([0, 0, 0, 0.02, 0.02, 0.02, 1, 0, 0, 0, 0, 0, 0, -8.0])


def from_grid(grid: np.ndarray) -> dict:
    """Inverse of to_grid: (32*32, 16*14) -> raw parameters of 16384
    Gaussians (ready for ``Fitter(init=...)``)."""
    fx, fy, cx, cy, tz = _cam()
    g = np.asarray(grid, np.float64).reshape(GRID, GRID, SLOTS, NPARAM)
    gy, gx = np.meshgrid(np.arange(GRID), np.arange(GRID), indexing="ij")
    px = (gx[..., None] + 0.5 + g[..., 0]) * CELL
    py = (gy[..., None] + 0.5 + g[..., 1]) * CELL
    z = g[..., 2]
    zc = z + tz
    x = (px - cx) * zc / fx
    y = (py - cy) * zc / fy
    means = np.stack([x, y, z], -1).reshape(-1, 3)
    flat = g.reshape(-1, NPARAM)
    q = flat[:, 6:10]
    q = q / np.maximum(np.linalg.norm(q, axis=1, keepdims=True), 1e-6)
    return dict(means3d=means.astype(np.float32), scales=np.abs(flat[:, 3:6]).astype(np.float32),
                quats=q.astype(np.float32), colors=flat[:, 10:13].astype(np.float32),
                opacities=flat[:, 13:14].astype(np.float32))


def from_grid_device(grid: torch.Tensor) -> dict:
    """from_grid on the device in fp32 (grid: (32*32, 16*14) tensor): the
    proposal goes from the network's output to the fitter's buffers without
    a round trip through the host."""
    fx, fy, cx, cy, tz = _cam()
    g = grid.to(torch.float32).reshape(GRID, GRID, SLOTS, NPARAM)
    idx = torch.arange(GRID, device=g.device, dtype=torch.float32)
    gy, gx = torch.meshgrid(idx, idx, indexing="ij")
    px = (gx[..., None] + 0.5 + g[..., 0]) * CELL
    py = (gy[..., None] + 0.5 + g[..., 1]) * CELL
    z = g[..., 2]
    zc = z + tz
    means = torch.stack([(px - cx) * zc / fx, (py - cy) * zc / fy, z], -1).reshape(-1, 3)
    flat = g.reshape(-1, NPARAM)
    q = flat[:, 6:10]
    q = q / torch.clamp(torch.linalg.norm(q, dim=1, keepdim=True), min=1e-6)
    return dict(means3d=means, scales=flat[:, 3:6].abs(), quats=q, colors=flat[:, 10:13],
                opacities=flat[:, 13:14])


# ---------------------------------------------------------------------------
# Data, training, evaluation.

def fit_set(target: np.ndarray, seed: int, steps: int, device="cuda") -> dict:
    """Plain fit (random init, Adam lr 1e-2) for `steps` steps -> raw params."""
    ft = Fitter(target, SLOTS * GRID * GRID, seed=seed, device=device)
    ft.run(steps)
    ft.check()
    return {k: v.detach().cpu().numpy() for k, v in ft.params().items()}


class WarmStart:
    """Trains the network on fitted sets and proposes initial parameters."""

    def __init__(self, device="cuda", seed: int = 0):
        self.dev = torch.device(device)
        self.net = ConvNet(device, seed)
        self.mu = np.zeros(SLOTS * NPARAM, np.float32)
        self.sd = np.ones(SLOTS * NPARAM, np.float32)
        self._stats_dev = None

    def fit_normaliser(self, grids):
        """Per-parameter mean and spread over every slot of every set (numpy
        array or device tensor)."""
        per = torch.as_tensor(grids).reshape(-1, NPARAM)
        mu = torch.zeros(NPARAM, dtype=torch.float64, device=per.device)
        sq = torch.zeros(NPARAM, dtype=torch.float64, device=per.device)
        for c in torch.split(per, 1 << 22):  # in chunks: the fp64 copies stay small
            c = c.double()
            mu += c.sum(0)
            sq += (c * c).sum(0)
        n = per.shape[0]
        mu /= n
        sd = (sq / n - mu * mu).clamp_min(0).sqrt() + 1e-3
        self.mu = np.tile(mu.cpu().numpy(), SLOTS).astype(np.float32)
        self.sd = np.tile(sd.cpu().numpy(), SLOTS).astype(np.float32)
        self._stats_dev = None

    def _img(self, imgs):
        if isinstance(imgs, torch.Tensor):
            return imgs.to(self.dev, torch.bfloat16)
        return torch.as_tensor(np.asarray(imgs, np.float32)).to(self.dev).to(torch.bfloat16)

    def train(self, images, grids, epochs: int = 20, batch: int = 8, lr: float = 1e-3,
              log=None) -> list:
        """images (S, 512, 512, 3), grids (S, 1024, 224) (numpy arrays or
        device tensors; a device tensor of grids is standardised in place)
        -> per-epoch mean loss."""
        lib = _lib.load()
        self.fit_normaliser(grids)
        X = self._img(images)
        mu = torch.as_tensor(self.mu, device=self.dev)
        sd = torch.as_tensor(self.sd, device=self.dev)
        if isinstance(grids, torch.Tensor):
            Y = grids.to(self.dev, torch.float32)
            Y.sub_(mu).div_(sd)
        else:
            Y = (torch.as_tensor(np.asarray(grids, np.float32)).to(self.dev) - mu) / sd
        n = X.shape[0]
        loss = torch.zeros(1, device=self.dev)
        tot = torch.zeros(1, dtype=torch.float64, device=self.dev)
        rng = np.random.default_rng(0)
        hist = []
        for ep in range(epochs):
            perm = rng.permutation(n)
            tot.zero_()
            nb = n // batch
            for b in range(nb):
                idx = torch.as_tensor(perm[b * batch:(b + 1) * batch], device=self.dev)
                out = self.net.forward(X[idx])
                dout = torch.empty_like(out)
                tgt = Y[idx].reshape(-1, SLOTS * NPARAM)
                _lib.check(lib.splat_l2_loss(_p(out), _p(tgt), out.numel(), _p(loss), _p(dout),
                                             C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)),
                           "l2_loss")
                self.net.backward(dout)
                self.net.adam(lr)
                tot += loss  # summed on the device: no host sync per step
            self.net.check()
            hist.append(float(tot.item()) / max(nb, 1))
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.4f}")
        return hist

    def propose(self, image) -> dict:
        """Initial raw parameters of 16384 Gaussians for a target image, as
        device tensors (the network's output de-standardised and decoded on
        the device)."""
        img = image if isinstance(image, torch.Tensor) else np.asarray(image)
        out = self.net.forward(self._img(img[None]))
        mu, sd = self._stats()
        return from_grid_device(out * sd + mu)

    def propose_mean(self, image=None) -> dict:
        """The ablation of ``propose``: the network's output forced to zero,
        i.e. the training sets' mean slot parameters in every cell of the
        grid -- the same grid layout and dataset statistics, nothing taken
        from the target image."""
        mu, _ = self._stats()
        return from_grid_device(mu.expand(GRID * GRID, -1))

    def _stats(self):
        """The standardisation (mean, std per slot parameter) on the device."""
        if self._stats_dev is None:
            self._stats_dev = (torch.as_tensor(np.asarray(self.mu, np.float32), device=self.dev),
                               torch.as_tensor(np.asarray(self.sd, np.float32), device=self.dev))
        return self._stats_dev


def time_to_psnr(fitter: Fitter, target, seed: int = 0, psnr: float = 30.0,
                 max_steps: int = 3000, check_every: int = 5, propose=None):
    """Wall-clock (s) for a reused, graph-captured Fitter to reach `psnr` dB
    on `target`: the proposal (`propose(target)`, else random init from
    `seed`), loading it, and the fitting loop.  Returns (reached, steps,
    seconds, final psnr)."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    init = propose(target) if propose is not None else None
    fitter.reset(target, init=init, seed=seed)
    reached, steps, _, p = fitter.fit_until(psnr, max_steps=max_steps, check_every=check_every)
    torch.cuda.synchronize()
    return reached, steps, time.perf_counter() - t0, p


__all__ = ["ConvNet", "WarmStart", "to_grid", "from_grid", "from_grid_device", "fit_set",
           "time_to_psnr", "random_init"]


def make_dataset(n_sets: int, fit_steps: int, first_seed: int = 0, device="cuda", log=None,
                 concurrent: int = 8):
    """Targets and grid-form fitted sets of `n_sets` procedural images
    (seeds first_seed ..), each fitted by the plain loop for `fit_steps`
    steps from random init, kept on the device (targets as bf16, the
    network's input type; grids as fp32).  `concurrent` fits run at once,
    each a reused Fitter replaying its own captured step graph on its own
    stream: one fit of 16384 Gaussians at 512x512 is a graph of small kernels
    that leaves most of the GPU idle, and independent fits fill it."""
    from .scenes import procedural_target

    dev = torch.device(device)
    k_max = max(1, min(int(concurrent), n_sets))
    fitters, streams = [], []
    imgs = torch.empty(n_sets, IMG, IMG, 3, dtype=torch.bfloat16, device=dev)
    grids = torch.empty(n_sets, GRID * GRID, SLOTS * NPARAM, dtype=torch.float32, device=dev)
    cur = torch.cuda.current_stream(dev)
    for k0 in range(0, n_sets, k_max):
        group = list(range(k0, min(n_sets, k0 + k_max)))
        targets = []
        for j, k in enumerate(group):
            sd = first_seed + k
            tgt = procedural_target(sd, IMG, device=device)
            if j == len(fitters):
                fitters.append(Fitter(tgt.cpu().numpy(), SLOTS * GRID * GRID, seed=sd,
                                      device=device))
                streams.append(torch.cuda.Stream(dev))
            ft = fitters[j]
            ft.reset(tgt, seed=sd)
            if ft.graph is None:
                ft.capture()
            targets.append(tgt)
        for j in range(len(group)):
            streams[j].wait_stream(cur)
        for _ in range(fit_steps):
            for j in range(len(group)):
                with torch.cuda.stream(streams[j]):
                    fitters[j].graph.replay()
        for j, k in enumerate(group):
            cur.wait_stream(streams[j])
            ft = fitters[j]
            ft.steps_done += fit_steps
            ft.check()
            params = {kk: v.detach().cpu().numpy() for kk, v in ft.params().items()}
            imgs[k] = targets[j].to(torch.bfloat16)
            grids[k] = torch.from_numpy(to_grid(params)).to(dev)
        if log and (group[-1] + 1) // 100 > k0 // 100:
            log(f"fitted {group[-1] + 1}/{n_sets}")
    return imgs, grids


def run_experiment(n_train: int = 1000, fit_steps: int = 300, epochs: int = 60,
                   eval_seeds=tuple(range(1_000_000, 1_000_008)), psnr: float = 30.0,
                   check_every: int = 5, device="cuda", log=None, concurrent: int = 16,
                   lr: float = 3e-3) -> dict:
    """Dataset from the plain loop, training, then wall-clock to `psnr` dB on
    held-out seeds from three starts: random init (the plain method), the
    network's proposal, and the ablation that keeps the proposal's grid
    layout and dataset-mean slot parameters but ignores the image
    (``WarmStart.propose_mean``)."""
    from .scenes import procedural_target

    t0 = time.perf_counter()
    imgs, grids = make_dataset(n_train, fit_steps, device=device, log=log, concurrent=concurrent)
    t_data = time.perf_counter() - t0
    ws = WarmStart(device)
    t1 = time.perf_counter()
    hist = ws.train(imgs, grids, epochs=epochs, lr=lr, log=log)
    t_train = time.perf_counter() - t1
    rows = []
    first = procedural_target(eval_seeds[0], IMG, device=device).cpu().numpy()
    ft = Fitter(first, SLOTS * GRID * GRID, seed=0, device=device)
    ft.capture()
    # untimed warm-up of both paths (first-use costs)
    time_to_psnr(ft, first, psnr=psnr, max_steps=20, check_every=check_every)
    time_to_psnr(ft, first, psnr=psnr, max_steps=20, check_every=check_every, propose=ws.propose)
    time_to_psnr(ft, first, psnr=psnr, max_steps=20, check_every=check_every,
                 propose=ws.propose_mean)
    for sd in eval_seeds:
        tgt = procedural_target(sd, IMG, device=device).cpu().numpy()
        plain = time_to_psnr(ft, tgt, seed=sd, psnr=psnr, check_every=check_every)
        learned = time_to_psnr(ft, tgt, seed=sd, psnr=psnr, check_every=check_every,
                               propose=ws.propose)
        mean = time_to_psnr(ft, tgt, seed=sd, psnr=psnr, check_every=check_every,
                            propose=ws.propose_mean)
        ft.reset(tgt, init=ws.propose(tgt))
        init_psnr = ft.check_render()
        ft.reset(tgt, init=ws.propose_mean(tgt))
        mean_init_psnr = ft.check_render()
        rows.append({"seed": int(sd), "plain_s": round(plain[2], 4), "plain_steps": plain[1],
                     "plain_reached": bool(plain[0]), "learned_s": round(learned[2], 4),
                     "learned_steps": learned[1], "learned_reached": bool(learned[0]),
                     "learned_init_psnr": round(init_psnr, 2), "mean_s": round(mean[2], 4),
                     "mean_steps": mean[1], "mean_reached": bool(mean[0]),
                     "mean_init_psnr": round(mean_init_psnr, 2)})
        if log:
            log(str(rows[-1]))
    return {"train_sets": n_train, "fit_steps": fit_steps, "epochs": epochs, "lr": lr,
            "data_s": round(t_data, 1), "train_s": round(t_train, 1),
            "loss_first": round(hist[0], 4), "loss_last": round(hist[-1], 4), "eval": rows}

