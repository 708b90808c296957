"""The fitted-set <-> grid mapping of the warm start (CPU): a set with at most
16 Gaussians per cell comes back unchanged (up to quaternion sign/scale and
|scales|), empty slots are transparent, and over-full cells keep their 16
most opaque Gaussians."""

import numpy as np


def _set(n, seed, spread=5.0):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    return dict(means3d=np.c_[rng.uniform(-spread, spread, (n, 2)), rng.uniform(-1, 1, n)],
                scales=rng.uniform(-0.3, 0.3, (n, 3)), quats=q * rng.uniform(0.5, 2, (n, 1)),
                colors=rng.normal(size=(n, 3)), opacities=rng.uniform(-4, 4, (n, 1)))


def _canon(p):
    q = p["quats"] / np.linalg.norm(p["quats"], axis=1, keepdims=True)
    q *= np.where(q[:, :1] < 0, -1, 1)
    return np.c_[p["means3d"], np.abs(p["scales"]), q, p["colors"], p["opacities"]]


def test_round_trip_of_sparse_set():
    from jaxsplat_gb300.warmstart import GRID, NPARAM, SLOTS, from_grid, to_grid

    p = _set(500, 0)
    g = to_grid(p)
    assert g.shape == (GRID * GRID, SLOTS * NPARAM)
    back = from_grid(g)
    live = back["opacities"].reshape(-1) > -7.9
    assert live.sum() == 500
    a = _canon(p)
    b = _canon({k: v[live] for k, v in back.items()})
    # same multiset of Gaussians: match by opacity (distinct values)
    ia, ib = np.argsort(a[:, -1]), np.argsort(b[:, -1])
    np.testing.assert_allclose(a[ia], b[ib], rtol=1e-4, atol=1e-4)


def test_full_cells_keep_the_most_opaque():
    from jaxsplat_gb300.warmstart import SLOTS, from_grid, to_grid

    p = _set(40, 1, spread=0.01)
    p["means3d"][:, :2] += 0.1  # all inside one cell (pixel ~ (259, 259))
    back = from_grid(to_grid(p))
    live = np.sort(back["opacities"].reshape(-1)[back["opacities"].reshape(-1) > -7.9])
    top = np.sort(p["opacities"].reshape(-1))[-SLOTS:]
    np.testing.assert_allclose(live, top, atol=1e-5)


def test_device_decoding_matches_host_decoding():
    """from_grid_device (the proposal's decoding, run here on CPU tensors)
    gives from_grid's parameters to fp32 rounding."""
    import torch

    from jaxsplat_gb300.warmstart import from_grid, from_grid_device, to_grid

    g = to_grid(_set(3000, 2))
    host = from_grid(g)
    dev = from_grid_device(torch.as_tensor(g))
    for k, v in host.items():
        np.testing.assert_allclose(dev[k].numpy(), v, rtol=1e-5, atol=1e-5, err_msg=k)


def test_device_random_init_has_the_reference_ranges():
    """random_init_device draws random_init's distributions (on CPU here):
    means in [-6, 6]^2 x [-1, 1], scales in [0, 0.5], unit quaternions,
    colours in [0, 1], opacities in [0.5, 1]."""
    import torch

    from jaxsplat_gb300.fit import random_init_device

    p = random_init_device(20000, 3, torch.device("cpu"))
    m = p["means3d"].numpy()
    assert m.shape == (20000, 3)
    assert (np.abs(m[:, :2]) <= 6).all() and (np.abs(m[:, 2]) <= 1).all()
    assert m[:, 0].min() < -5.9 and m[:, 0].max() > 5.9
    s = p["scales"].numpy()
    assert (s >= 0).all() and (s <= 0.5).all()
    np.testing.assert_allclose(np.linalg.norm(p["quats"].numpy(), axis=1), 1.0, atol=1e-5)
    c, o = p["colors"].numpy(), p["opacities"].numpy()
    assert (c >= 0).all() and (c <= 1).all() and (o >= 0.5).all() and (o <= 1).all()
    again = random_init_device(20000, 3, torch.device("cpu"))
    assert torch.equal(again["means3d"], p["means3d"])  # seeded
