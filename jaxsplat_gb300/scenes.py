"""Seeded synthetic Gaussian scenes with the shapes and value distributions of
the workloads this library is measured on.

Every scene is drawn with numpy's PCG64 generator, so the same seed gives the
same arrays on any machine.  The distributions follow the benchmark
definitions of the render path (camera at the origin looking down +z,
identity view matrix):

  means     x ~ U[-xr, xr], y ~ U[-yr, yr], z ~ U[z0, z1]
  scales    exp(N(-4.0, 0.5)) per axis
  quats     N(0, 1)^4, normalised (w, x, y, z order)
  colors    U[0, 1]^3
  opacities sigmoid(N(0, 1)), shape (N, 1)
  target    U[0, 1]^(H, W, 3) (the L2 loss target)
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class SceneSpec:
    name: str
    num_points: int
    img_shape: tuple[int, int]  # (H, W)
    f: tuple[float, float]
    c: tuple[float, float]
    x_range: float = 2.0
    y_range: float = 2.0
    z_range: tuple[float, float] = (2.0, 8.0)
    glob_scale: float = 1.0
    clip_thresh: float = 0.01
    block_width: int = 16
    background: tuple[float, float, float] = (0.0, 0.0, 0.0)


# The named workloads.  "small" is the 100k-Gaussian 256x256 case, "hd" the
# 1M-Gaussian 1920x1080 headline case, "uhd" its 6M-Gaussian 3840x2160
# variant, "gradcheck" the 20k-Gaussian 128x128 finite-difference case.
SPECS = {
    "small": SceneSpec("small", 100_000, (256, 256), (256.0, 256.0), (128.0, 128.0)),
    "hd": SceneSpec(
        "hd", 1_000_000, (1080, 1920), (1200.0, 1200.0), (960.0, 540.0),
        x_range=4.0, y_range=2.5, z_range=(2.0, 12.0),
    ),
    "uhd": SceneSpec(
        "uhd", 6_000_000, (2160, 3840), (2400.0, 2400.0), (1920.0, 1080.0),
        x_range=4.0, y_range=2.5, z_range=(2.0, 12.0),
    ),
    "gradcheck": SceneSpec("gradcheck", 20_000, (128, 128), (128.0, 128.0), (64.0, 64.0)),
}


@dataclass
class Scene:
    spec: SceneSpec
    means3d: np.ndarray
    scales: np.ndarray
    quats: np.ndarray
    colors: np.ndarray
    opacities: np.ndarray
    viewmat: np.ndarray
    background: np.ndarray
    target: np.ndarray
    extra: dict = field(default_factory=dict)

    @property
    def kwargs(self) -> dict:
        s = self.spec
        return dict(
            img_shape=tuple(s.img_shape), f=tuple(s.f), c=tuple(s.c),
            glob_scale=s.glob_scale, clip_thresh=s.clip_thresh,
        )


def make_scene(spec: SceneSpec | str, seed: int = 0, num_points: int | None = None,
               img_shape: tuple[int, int] | None = None, block_width: int | None = None) -> Scene:
    """Draw a scene.  ``num_points`` / ``img_shape`` / ``block_width`` override
    the spec (the focal length and principal point then follow the image
    size the way the named specs do: f = W (or the spec's f scaled), c = centre)."""
    if isinstance(spec, str):
        spec = SPECS[spec]
    if num_points is not None or img_shape is not None or block_width is not None:
        h, w = img_shape if img_shape is not None else spec.img_shape
        sh, sw = spec.img_shape
        spec = SceneSpec(
            spec.name, num_points if num_points is not None else spec.num_points, (h, w),
            (spec.f[0] * w / sw, spec.f[1] * w / sw), (w / 2.0, h / 2.0),
            spec.x_range, spec.y_range, spec.z_range, spec.glob_scale, spec.clip_thresh,
            block_width if block_width is not None else spec.block_width, spec.background,
        )
    rng = np.random.default_rng(seed)
    n = spec.num_points
    means = np.empty((n, 3), np.float32)
    means[:, 0] = rng.uniform(-spec.x_range, spec.x_range, n)
    means[:, 1] = rng.uniform(-spec.y_range, spec.y_range, n)
    means[:, 2] = rng.uniform(spec.z_range[0], spec.z_range[1], n)
    scales = np.exp(rng.normal(-4.0, 0.5, (n, 3))).astype(np.float32)
    q = rng.normal(0.0, 1.0, (n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    quats = q.astype(np.float32)
    colors = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    opac = (1.0 / (1.0 + np.exp(-rng.normal(0.0, 1.0, (n, 1))))).astype(np.float32)
    h, w = spec.img_shape
    target = rng.uniform(0.0, 1.0, (h, w, 3)).astype(np.float32)
    return Scene(
        spec=spec, means3d=means, scales=scales, quats=quats, colors=colors, opacities=opac,
        viewmat=np.eye(4, dtype=np.float32), background=np.asarray(spec.background, np.float32),
        target=target,
    )


def look_at(eye, target=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Row-major world -> camera matrix of a camera at `eye` looking at
    `target` (+z forward, +y down in the image, world +y as the down
    direction, like the identity view matrix)."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    d = np.array([0.0, 1.0, 0.0])
    r = np.cross(d, f)
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    V = np.eye(4)
    V[:3, :3] = R
    V[:3, 3] = -R @ eye
    return V.astype(np.float32)


# The batched workload: 4 scenes (Gaussian counts below, distributions of the
# "small" scene), 8 cameras per scene on a circle of radius 6 around the
# origin looking at it, poses jittered by seed, image sizes cycling through
# 512x512, 1280x720 and 1920x1080, f = 0.625 W (the 1920x1080 scene's
# field of view), principal point at the centre.
BATCH_POINTS = (50_000, 200_000, 800_000, 2_000_000)
BATCH_SIZES = ((512, 512), (720, 1280), (1080, 1920))


def make_batch(seed: int = 0, scene_points=BATCH_POINTS, views_per_scene: int = 8,
               sizes=BATCH_SIZES, radius: float = 6.0):
    """Returns (scenes, views, targets): scene dicts with means3d, scales,
    quats, colors, opacities; view dicts with scene, viewmat, img_shape, f,
    c, background; one U[0,1] target image per view."""
    rng = np.random.default_rng(seed)
    scenes, views, targets = [], [], []
    for s, n in enumerate(scene_points):
        sc = make_scene("small", seed=seed * 1000 + s, num_points=int(n))
        scenes.append(dict(means3d=sc.means3d, scales=sc.scales, quats=sc.quats,
                           colors=sc.colors, opacities=sc.opacities))
        for v in range(views_per_scene):
            th = 2.0 * np.pi * v / views_per_scene + rng.uniform(-0.1, 0.1)
            eye = (radius * np.sin(th), rng.uniform(-0.3, 0.3), -radius * np.cos(th))
            h, w = sizes[(s + v) % len(sizes)]
            f = 0.625 * w
            views.append(dict(scene=s, viewmat=look_at(eye), img_shape=(h, w), f=(f, f),
                              c=(w / 2.0, h / 2.0), background=np.zeros(3, np.float32)))
            targets.append(rng.uniform(0.0, 1.0, (h, w, 3)).astype(np.float32))
    return scenes, views, targets


def _procedural_params(seed: int, size: int, blobs: int, gratings: int):
    rng = np.random.default_rng(seed)
    bl = []
    for _ in range(blobs):
        cx, cy = rng.uniform(0, size, 2)
        sx, sy = np.exp(rng.uniform(np.log(size / 64), np.log(size / 6), 2))
        th = rng.uniform(0, np.pi)
        bl.append((cx, cy, sx, sy, th, rng.uniform(0, 1, 3)))
    gr = []
    for _ in range(gratings):
        cycles = rng.uniform(2, 20)
        th = rng.uniform(0, np.pi)
        phase = rng.uniform(0, 2 * np.pi)
        gr.append((cycles, th, phase, rng.uniform(0, 0.5, 3)))
    return bl, gr


def procedural_target(seed: int, size: int = 512, blobs: int = 64, gratings: int = 3,
                      device=None) -> np.ndarray:
    """A (size, size, 3) fp32 image in [0, 1] drawn from a seed: a sum of
    `blobs` random anisotropic 2D Gaussian blobs with random colours plus
    `gratings` sinusoidal gratings (2-20 cycles across the image, random
    orientation, phase and colour), rescaled into [0, 1].  With a torch
    `device` the image is evaluated there in fp32 and returned as a tensor
    (same draws; numpy evaluates in fp64)."""
    bl, gr = _procedural_params(seed, size, blobs, gratings)
    if device is not None:
        import torch

        ar = torch.arange(size, dtype=torch.float32, device=device) + 0.5
        yy, xx = torch.meshgrid(ar, ar, indexing="ij")
        img = torch.zeros(size, size, 3, device=device)
        cos, sin = math.cos, math.sin
    else:
        yy, xx = np.meshgrid(np.arange(size, dtype=np.float64) + 0.5,
                             np.arange(size, dtype=np.float64) + 0.5, indexing="ij")
        img = np.zeros((size, size, 3))
        cos, sin = np.cos, np.sin
    lib = np if device is None else __import__("torch")
    for cx, cy, sx, sy, th, col in bl:
        c, s_ = cos(th), sin(th)
        dx, dy = xx - cx, yy - cy
        u = (c * dx + s_ * dy) / sx
        v = (-s_ * dx + c * dy) / sy
        img = img + lib.exp(-0.5 * (u * u + v * v))[..., None] * _as(col, img)
    for cycles, th, phase, col in gr:
        w = 2 * np.pi * cycles / size
        g = 0.5 + 0.5 * lib.sin(w * (cos(th) * xx + sin(th) * yy) + phase)
        img = img + g[..., None] * _as(col, img)
    lo, hi = img.min(), img.max()
    if device is not None:
        return ((img - lo) / max(float(hi - lo), 1e-12)).float()
    return ((img - lo) / max(hi - lo, 1e-12)).astype(np.float32)


def _as(col, like):
    if isinstance(like, np.ndarray):
        return col
    import torch

    return torch.as_tensor(np.asarray(col, np.float32), device=like.device)
