"""The fitting loop (examples/single_image.py on this library's kernels):
the fused parameter maps + Adam kernel against torch, and a short fit."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_adam_kernel_matches_torch_adam():
    import torch

    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    n, lr = 1000, 1e-2
    g = torch.Generator(device="cpu").manual_seed(0)
    raw = {k: torch.randn(n, d, generator=g).cuda() for k, d in
           (("means", 3), ("scales", 3), ("quats", 4), ("colors", 3), ("opac", 1))}
    grads = [torch.randn(n, d, generator=g).cuda() * 1e-3 for d in (3, 3, 4, 3, 1)]
    # torch reference: the same maps, autograd, torch.optim.Adam (same update rule as optax.adam)
    ref = {k: v.clone().requires_grad_(True) for k, v in raw.items()}
    opt = torch.optim.Adam(list(ref.values()), lr=lr, betas=(0.9, 0.999), eps=1e-8)
    mapped = {k: v.clone() for k, v in raw.items()}
    m = torch.zeros(n, 14, device="cuda")
    v = torch.zeros(n, 14, device="cuda")
    step = torch.zeros(1, dtype=torch.int32, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(3):
        opt.zero_grad()
        q = ref["quats"] / ref["quats"].norm(dim=-1, keepdim=True)
        outs = [ref["means"], ref["scales"], q, torch.sigmoid(ref["colors"]),
                torch.sigmoid(ref["opac"])]
        torch.autograd.backward(outs, grads)
        opt.step()
        assert lib.splat_fit_transform(n, P(raw["quats"]),
                                       P(raw["colors"]), P(raw["opac"]), P(mapped["quats"]),
                                       P(mapped["colors"]), P(mapped["opac"]), stream) == 0
        assert lib.splat_fit_adam(n, lr, P(step), P(raw["means"]), P(raw["scales"]),
                                  P(raw["quats"]), P(raw["colors"]), P(raw["opac"]), P(m), P(v),
                                  *[P(t) for t in grads], P(mapped["quats"]),
                                  P(mapped["colors"]), P(mapped["opac"]), stream) == 0
    torch.cuda.synchronize()
    assert int(step.item()) == 3
    for k in raw:
        torch.testing.assert_close(raw[k], ref[k].detach(), rtol=1e-5, atol=1e-6)


def test_fit_improves_psnr():
    from jaxsplat_gb300.fit import Fitter
    from jaxsplat_gb300.scenes import make_scene

    # a smooth target: a few blurred blobs
    h, w = 64, 96
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    target = np.zeros((h, w, 3), np.float32)
    rng = np.random.default_rng(3)
    for _ in range(6):
        cx, cy, r = rng.uniform(0, w), rng.uniform(0, h), rng.uniform(5, 20)
        target += np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * r * r))[..., None] * rng.uniform(0, 1, 3)
    target = np.clip(target, 0, 1)
    fit = Fitter(target, 3000, seed=1)
    fit.run(1)
    p0 = fit.check()
    reached, steps, secs, p = fit.fit_until(target_psnr=60.0, max_steps=300, check_every=50)
    assert steps == 300
    assert p > p0 + 5.0, (p0, p)
