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


# Output groups and their parity bar: integer/index outputs
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


# Element-wise bar for gradients, beside the normwise one: over the entries
# whose reference magnitude is at least ELEM_FLOOR x the array's largest, the
# relative error |a - b| / |b| has its 99th percentile within ELEM_P99 and its
# maximum within ELEM_MAX.  Two fp32 implementations that sum the same terms
# in different orders (the reference's atomics, this library's reductions)
# were measured at p99 <= 8.2e-6 and max <= 6.8e-4 on every case (100k to 6M
# Gaussians, batched views, block widths 8-16); the bar keeps ~4x headroom.
ELEM_FLOOR = 1e-3
ELEM_P99 = 3e-5
ELEM_MAX = 3e-3


def elementwise_rel(a, b, floor: float = ELEM_FLOOR):
    """(max, p99, count) of |a - b| / |b| over entries with |b| >= floor *
    max|b|.  Works on numpy arrays or torch tensors (kept on their device)."""
    try:
        import torch

        if isinstance(a, torch.Tensor):
            a64 = a.detach().reshape(-1).double()
            b64 = b.detach().reshape(-1).double().to(a64.device)
            if b64.numel() == 0:
                return 0.0, 0.0, 0
            m = b64.abs() >= floor * b64.abs().max()
            r = ((a64[m] - b64[m]).abs() / b64[m].abs())
            n = int(r.numel())
            if n == 0:
                return 0.0, 0.0, 0
            k = max(1, int(np.ceil(0.99 * n)))
            return float(r.max()), float(torch.kthvalue(r.cpu(), k).values), n
    except ImportError:  # pragma: no cover
        pass
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    if b.size == 0:
        return 0.0, 0.0, 0
    m = np.abs(b) >= floor * np.abs(b).max()
    if not m.any():
        return 0.0, 0.0, 0
    r = np.abs(a[m] - b[m]) / np.abs(b[m])
    return float(r.max()), float(np.percentile(r, 99)), int(m.sum())


def assert_elementwise(a, b, label: str, p99: float = ELEM_P99, mx: float = ELEM_MAX):
    emax, ep99, n = elementwise_rel(a, b)
    print(f"{label}: element-wise rel err over {n} entries: max {emax:.3g} p99 {ep99:.3g}")
    assert ep99 <= p99 and emax <= mx, f"{label}: max {emax:.3g} p99 {ep99:.3g}"
    return emax, ep99
