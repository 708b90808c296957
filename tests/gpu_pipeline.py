"""Helpers shared by the GPU tests: run this library's CUDA path stage by
stage on numpy inputs and return numpy outputs named like the golden
fixtures."""

import numpy as np
import torch

from jaxsplat_gb300 import _ops

INPUT_KEYS = ("means3d", "scales", "quats", "colors", "opacities", "viewmat", "background")


def to_dev(inp: dict) -> dict:
    return {k: torch.from_numpy(np.ascontiguousarray(inp[k], np.float32)).cuda()
            for k in INPUT_KEYS if k in inp}


def run_cuda(inp: dict, kw: dict, bw: int, v_img=None, with_abs=True, device=False,
             blend=True) -> dict:
    """project -> sort/bin (with intermediates) -> rasterize fwd [-> bwd chain].
    Returns numpy arrays, or the CUDA tensors themselves with ``device``;
    ``v_img`` may be a numpy array or a CUDA tensor.  With ``blend`` (block
    width 16) the backward walks the forward's per-slot warp bytes."""
    t = to_dev(inp)
    p = _ops.project_fwd(t["means3d"], t["scales"], t["quats"], t["viewmat"], block_width=bw,
                         **kw)
    n = t["means3d"].shape[0]
    count = _ops.read_counts(n, p["cum_tiles_hit"], p["total"], device=t["means3d"].device)
    s = _ops.sort_and_bin(count, p["xys"], p["depths"], p["radii"], p["cum_tiles_hit"],
                          img_shape=kw["img_shape"], block_width=bw, intermediates=True)
    packed = _ops.pack_splats(p["xys"], p["conics"], t["colors"], t["opacities"],
                              img_shape=kw["img_shape"], block_width=bw)
    r = _ops.rasterize_fwd(count, s["gaussian_ids_sorted"], s["tile_bins"], packed,
                           t["background"], img_shape=kw["img_shape"], block_width=bw,
                           blend=blend)
    blend_bytes = r.pop("blend", None)
    out = {**p, **s, **r}
    out.pop("total")
    out["count"] = torch.tensor(count)
    if v_img is not None:
        h, w = kw["img_shape"]
        vi = (v_img.contiguous() if isinstance(v_img, torch.Tensor)
              else torch.from_numpy(np.ascontiguousarray(v_img, np.float32)).cuda())
        rb = _ops.rasterize_bwd(count, s["gaussian_ids_sorted"], s["tile_bins"], packed,
                                t["background"], r["final_Ts"], r["final_idx"], vi,
                                torch.zeros(h, w, 1, device="cuda"), img_shape=kw["img_shape"],
                                block_width=bw, with_abs=with_abs, blend=blend_bytes)
        z = torch.zeros(n, 1, device="cuda")
        pb = _ops.project_bwd(t["means3d"], t["scales"], t["quats"], t["viewmat"], p["cov3d"],
                              p["radii"], p["conics"], p["compensation"], rb["v_xy"], z,
                              rb["v_conic"], z, block_width=bw, **kw)
        out.update(rb)
        out.update(pb)
    torch.cuda.synchronize()
    if device:
        return out
    return {k: v.cpu().numpy() for k, v in out.items()}
