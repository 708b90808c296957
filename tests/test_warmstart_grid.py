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
