"""Generate the golden fixtures in tests/golden/ from the reference's own kernels.

Run on a machine with a GPU, after ``python oracle/build.py`` has produced
oracle/_ref/*.cubin (compiled from the reference's lib/kernels sources) and
the harness:

    python tests/golden/make_golden.py --out tests/golden

For each case the reference's four custom calls are chained exactly as
``jax.grad(mean((render(...) - target)**2))`` dispatches them (see
oracle/ref.py), and the sort/bin intermediates are taken from the same
kernels.  Small cases store every input and output array (``<case>.npz``);
the 100k-Gaussian 256x256 case stores sha256 digests and summary statistics
(``small.json``) because its arrays are large.
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from jaxsplat_gb300.scenes import make_scene  # noqa: E402


def _viewmat_tilted() -> np.ndarray:
    """A rigid world-to-camera transform with a non-trivial rotation."""
    ay, ax = 0.21, -0.13
    ry = np.array([[np.cos(ay), 0, np.sin(ay)], [0, 1, 0], [-np.sin(ay), 0, np.cos(ay)]])
    rx = np.array([[1, 0, 0], [0, np.cos(ax), -np.sin(ax)], [0, np.sin(ax), np.cos(ax)]])
    v = np.eye(4)
    v[:3, :3] = rx @ ry
    v[:3, 3] = [0.3, -0.2, 0.5]
    return v.astype(np.float32)


def tiny_inputs(seed: int = 11) -> dict:
    """~700 Gaussians on a 70x45 image (not a multiple of any tile width),
    with planted edge cases appended after the random ones."""
    sc = make_scene("small", seed=seed, num_points=700, img_shape=(45, 70))
    means, scales, quats = sc.means3d.copy(), sc.scales.copy(), sc.quats.copy()
    colors, opac = sc.colors.copy(), sc.opacities.copy()
    extra_m, extra_s = [], []
    extra_m.append([0.0, 0.0, -1.0]); extra_s.append([0.05, 0.05, 0.05])      # behind camera
    extra_m.append([0.0, 0.0, 0.005]); extra_s.append([0.05, 0.05, 0.05])     # inside near clip
    extra_m.append([40.0, 0.0, 4.0]); extra_s.append([0.02, 0.02, 0.02])      # off screen
    extra_m.append([-1.2, 0.0, 4.0]); extra_s.append([0.08, 0.08, 0.08])      # straddles border
    extra_m.append([0.1, -0.1, 6.0]); extra_s.append([1.5, 1.2, 0.9])         # covers every tile
    extra_m.append([0.3, 0.2, 3.0]); extra_s.append([0.01, 0.01, 0.01])       # tiny
    k = len(extra_m)
    # the planted positions are camera-space; map them back to world space
    vm = _viewmat_tilted().astype(np.float64)
    cam = np.asarray(extra_m, np.float64)
    extra_m = ((cam - vm[:3, 3]) @ vm[:3, :3]).tolist()
    rng = np.random.default_rng(seed + 1)
    q = rng.normal(size=(k, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    means = np.concatenate([means, np.asarray(extra_m, np.float32)])
    scales = np.concatenate([scales, np.asarray(extra_s, np.float32)])
    quats = np.concatenate([quats, q.astype(np.float32)])
    colors = np.concatenate([colors, rng.uniform(size=(k, 3)).astype(np.float32)])
    opac = np.concatenate([opac, rng.uniform(0.3, 0.99, size=(k, 1)).astype(np.float32)])
    # exact duplicates of two random Gaussians: equal depth keys, so the
    # stable sort must order them by Gaussian index
    dup = [6, 17]
    means = np.concatenate([means, means[dup]])
    scales = np.concatenate([scales, scales[dup]])
    quats = np.concatenate([quats, quats[dup]])
    colors = np.concatenate([colors, colors[::-1][:2]])
    opac = np.concatenate([opac, opac[dup]])
    h, w = 45, 70
    return dict(
        means3d=means, scales=scales, quats=quats, colors=colors, opacities=opac,
        viewmat=_viewmat_tilted(), background=np.asarray([0.1, 0.2, 0.3], np.float32),
        target=rng.uniform(size=(h, w, 3)).astype(np.float32),
        img_shape=np.asarray([h, w]), f=np.asarray([60.0, 55.0]), c=np.asarray([35.5, 22.25]),
        glob_scale=np.asarray(1.0), clip_thresh=np.asarray(0.01),
    )


def spec_inputs(name: str, seed: int) -> dict:
    sc = make_scene(name, seed=seed)
    return dict(
        means3d=sc.means3d, scales=sc.scales, quats=sc.quats, colors=sc.colors,
        opacities=sc.opacities, viewmat=sc.viewmat, background=sc.background, target=sc.target,
        img_shape=np.asarray(sc.spec.img_shape), f=np.asarray(sc.spec.f),
        c=np.asarray(sc.spec.c), glob_scale=np.asarray(sc.spec.glob_scale),
        clip_thresh=np.asarray(sc.spec.clip_thresh),
    )


CASES = {
    # name: (input builder, block width)
    "tiny_bw16": (lambda: tiny_inputs(), 16),
    "tiny_bw8": (lambda: tiny_inputs(), 8),
    "tiny_bw12": (lambda: tiny_inputs(), 12),
    "gradcheck": (lambda: spec_inputs("gradcheck", 3), 16),
}
HASHED = {"small": (lambda: spec_inputs("small", 0), 16)}

INPUT_KEYS = ("means3d", "scales", "quats", "colors", "opacities", "viewmat", "background",
              "target")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def render_kwargs(inp: dict, bw: int) -> dict:
    return dict(img_shape=tuple(int(x) for x in inp["img_shape"]),
                f=tuple(float(x) for x in inp["f"]), c=tuple(float(x) for x in inp["c"]),
                glob_scale=float(inp["glob_scale"]), clip_thresh=float(inp["clip_thresh"]),
                block_size=bw)


def l2_cotangent(img, target):
    """d/d img of mean((img - target)^2)."""
    return 2.0 * (img - target) / img.numel()


def run_reference(ref, inp: dict, bw: int) -> dict:
    import torch

    dev = "cuda"
    t = {k: torch.from_numpy(np.ascontiguousarray(inp[k])).to(dev) for k in INPUT_KEYS}
    kw = render_kwargs(inp, bw)
    fwd = ref.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                     viewmat=t["viewmat"], background=t["background"], **kw)
    v_img = l2_cotangent(fwd["img"], t["target"]).contiguous()
    out = ref.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                     viewmat=t["viewmat"], background=t["background"], v_img=v_img, **kw)
    s = ref.sort_and_bin(out["xys"], out["depths"], out["radii"], out["cum_tiles_hit"],
                         img_shape=kw["img_shape"], block_width=bw)
    out.update(s)
    out["v_img"] = v_img
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    ap.add_argument("--dump-full", action="store_true",
                    help="also write the hashed cases' full arrays (for offline analysis)")
    a = ap.parse_args()
    from oracle.ref import RefKernels

    ref = RefKernels()
    os.makedirs(a.out, exist_ok=True)
    for name, (mk, bw) in CASES.items():
        inp = mk()
        res = run_reference(ref, inp, bw)
        arrays = {f"in_{k}": np.asarray(v) for k, v in inp.items()}
        arrays.update({f"out_{k}": v for k, v in res.items()})
        arrays["block_width"] = np.asarray(bw)
        np.savez_compressed(os.path.join(a.out, f"{name}.npz"), **arrays)
        print(name, "I =", res["isect_ids"].size)
    for name, (mk, bw) in HASHED.items():
        inp = mk()
        res = run_reference(ref, inp, bw)
        rec = {"block_width": bw,
               "inputs_sha256": {k: digest(np.asarray(inp[k])) for k in INPUT_KEYS},
               "sha256": {k: digest(v) for k, v in res.items()},
               "stats": {k: {"sum": float(np.asarray(v, np.float64).sum()),
                             "abs_sum": float(np.abs(np.asarray(v, np.float64)).sum()),
                             "max_abs": float(np.abs(np.asarray(v, np.float64)).max())
                             if v.size else 0.0, "shape": list(v.shape)}
                         for k, v in res.items()}}
        with open(os.path.join(a.out, f"{name}.json"), "w") as fh:
            json.dump(rec, fh, indent=1, sort_keys=True)
        if a.dump_full:
            arrays = {f"in_{k}": np.asarray(v) for k, v in inp.items()}
            arrays.update({f"out_{k}": v for k, v in res.items()})
            np.savez_compressed(os.path.join(a.out, f"{name}_full.npz"), **arrays)
        print(name, "I =", res["isect_ids"].size)


if __name__ == "__main__":
    main()
