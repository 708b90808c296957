"""FP64 central finite differences against the render path's hand-written
adjoints (the 20k-Gaussian 128x128 gradient-check scene, eps = 1e-3).

The loss is mean((render - target)^2).  200 seed-chosen scalar entries are
checked, 40 per parameter group.  The render is piecewise smooth: tile sets
change with the radius, and a Gaussian's contribution switches at the
alpha < 1/255 and T <= 1e-4 cut-offs; the reference's adjoint also differs
from the true derivative where the forward's 0.999 alpha clamp and its
1.3 tan(fov) frustum clamp apply (backward.cu:261 and 446-452 use 0.99 and
no clamp).  Entries whose central difference changes by more than 1% when
the step is halved are flagged as non-smooth and reported, not compared.
"""

import numpy as np
import pytest

from conftest import golden_kwargs, load_golden
from oracle.oracle import Oracle

GROUPS = {"means3d": "v_mean3d", "scales": "v_scale", "quats": "v_quat", "colors": "v_colors",
          "opacities": "v_opacity"}
EPS = 1e-3
PER_GROUP = 40
# median / 90th-percentile relative error bounds per group on smooth entries
BOUNDS = {"means3d": (1e-2, 0.1), "scales": (1e-2, 0.1), "quats": (1e-3, 1e-2),
          "colors": (1e-6, 1e-5), "opacities": (1e-6, 1e-5)}


@pytest.fixture(scope="module")
def setup():
    o = Oracle("f64")
    g = load_golden("gradcheck")
    kw = golden_kwargs(g)
    P = {k: g["in_" + k].astype(np.float64) for k in GROUPS}
    target = g["in_target"].astype(np.float64)

    def render(P, v_img=None):
        return o.render(P["means3d"], P["scales"], P["quats"], P["colors"], P["opacities"],
                        viewmat=g["in_viewmat"], background=g["in_background"], block_size=16,
                        v_img=v_img, **kw)

    img = render(P)["img"]
    full = render(P, v_img=2.0 * (img - target) / img.size)
    return render, P, target, full


def _loss(render, P, target):
    return float(np.mean((render(P)["img"] - target) ** 2))


def _fd(render, P, target, grp, i, j, eps):
    Pp = {k: v.copy() for k, v in P.items()}
    Pm = {k: v.copy() for k, v in P.items()}
    Pp[grp][i, j] += eps
    Pm[grp][i, j] -= eps
    return (_loss(render, Pp, target) - _loss(render, Pm, target)) / (2.0 * eps)


@pytest.mark.parametrize("grp", list(GROUPS))
def test_fd_gradcheck_fp64(setup, grp):
    render, P, target, full = setup
    an = full[GROUPS[grp]]
    scale = float(np.abs(an).max())
    rng = np.random.default_rng(20_000 + list(GROUPS).index(grp))
    visible = np.nonzero(full["radii"].ravel() > 0)[0]
    rels, flagged = [], 0
    for _ in range(PER_GROUP):
        i = int(rng.choice(visible))
        j = int(rng.integers(P[grp].shape[1]))
        f1 = _fd(render, P, target, grp, i, j, EPS)
        f2 = _fd(render, P, target, grp, i, j, EPS / 2)
        if abs(f1 - f2) > 0.01 * max(abs(f1), abs(f2)) + 1e-4 * scale:
            flagged += 1
            continue
        a = float(an[i, j])
        rels.append(abs(f1 - a) / max(abs(f1), abs(a), 1e-3 * scale))
    r = np.asarray(rels)
    med, p90 = float(np.median(r)), float(np.percentile(r, 90))
    print(f"\n{grp}: {len(r)} smooth entries, {flagged} flagged; rel err median {med:.3g} "
          f"p90 {p90:.3g} max {r.max():.3g}")
    assert flagged <= PER_GROUP // 2
    assert med <= BOUNDS[grp][0] and p90 <= BOUNDS[grp][1]
