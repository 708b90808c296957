import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, GOLDEN)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsplat.so")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


GOLDEN_CASES = ["tiny_bw16", "tiny_bw8", "tiny_bw12", "gradcheck"]


def load_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return {k: z[k] for k in z.files}


def golden_kwargs(g: dict) -> dict:
    return dict(img_shape=tuple(int(x) for x in g["in_img_shape"]),
                f=tuple(float(x) for x in g["in_f"]), c=tuple(float(x) for x in g["in_c"]),
                glob_scale=float(g["in_glob_scale"]), clip_thresh=float(g["in_clip_thresh"]))


def load_small_digests() -> dict:
    with open(os.path.join(GOLDEN, "small.json")) as fh:
        return json.load(fh)


# Output groups and their parity bar (the benchmark spec): integer/index outputs
# bit-exact; image within 1e-5 absolute; gradients within 1e-4 relative
# (normwise: max |a - b| / max |b|).
INT_KEYS = ["radii", "num_tiles_hit", "cum_tiles_hit", "isect_ids", "gaussian_ids",
            "isect_ids_sorted", "gaussian_ids_sorted", "tile_bins", "final_idx"]
PROJ_FLOAT_KEYS = ["xys", "depths", "cov3d", "conics", "compensation"]
IMG_KEYS = ["img", "final_Ts"]
GRAD_KEYS = ["v_colors", "v_opacity", "v_xy", "v_conic", "v_mean3d", "v_scale", "v_quat"]
IMG_ATOL = 1e-5
GRAD_RTOL = 1e-4


def normwise_rel(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    denom = np.abs(b).max() if b.size else 0.0
    if denom == 0.0:
        return float(np.abs(a).max()) if a.size else 0.0
    return float(np.abs(a - b).max() / denom)
