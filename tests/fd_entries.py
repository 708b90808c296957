"""FP64 central finite differences of the render loss at 200 seed-chosen
scalar entries of the 20k-Gaussian 128x128 gradient-check scene (test
infrastructure, shared by the oracle-adjoint test and the CUDA-adjoint test).

The loss is mean((render - target)^2), rendered by the fp64 build of the
oracle.  For each entry the central difference is taken at eps = 1e-3 and
again at eps/2 and eps/4.  Richardson extrapolation, R(h) = (4 D(h/2) -
D(h)) / 3, cancels the O(eps^2) term of a smooth loss; where the loss is
smooth the two extrapolations R(eps) and R(eps/2) agree to ~1e-8 relative and
R(eps/2) is the derivative to that accuracy.  The render is only piecewise
smooth (tile sets change with the radius, a Gaussian's contribution switches
on at alpha >= 1/255 and stops at T <= 1e-4); an entry with such a switch
inside the stencil makes the extrapolations disagree and is flagged as
non-smooth instead of compared.  Entries on Gaussians whose camera-space
position is clamped to the frustum in the forward (forward.cu:498-501) are
flagged too: the reference's adjoint omits that clamp (backward.cu:421-524),
so there it is not the derivative of the forward.
"""

from __future__ import annotations

import functools

import numpy as np

from conftest import golden_kwargs, load_golden

GROUPS = {"means3d": "v_mean3d", "scales": "v_scale", "quats": "v_quat", "colors": "v_colors",
          "opacities": "v_opacity"}
EPS = 1e-3
PER_GROUP = 40
SMOOTH_RTOL = 1e-4  # agreement of the two Richardson extrapolations


def gradcheck_inputs():
    g = load_golden("gradcheck")
    return g, golden_kwargs(g)


def _frustum_clamped(g, kw):
    vm = g["in_viewmat"].astype(np.float64)
    t = g["in_means3d"].astype(np.float64) @ vm[:3, :3].T + vm[:3, 3]
    h, w = kw["img_shape"]
    fx, fy = kw["f"]
    lim_x, lim_y = 1.3 * 0.5 * w / fx, 1.3 * 0.5 * h / fy
    return (np.abs(t[:, 0] / t[:, 2]) > lim_x) | (np.abs(t[:, 1] / t[:, 2]) > lim_y)


@functools.lru_cache(maxsize=1)
def fd_table():
    """{group: list of dict(i, j, d1, d2, d4, deriv, smooth, clamped)} plus the
    oracle's fp64 adjoint under key "_adjoint" and the loss cotangent's
    scale under "_scale"."""
    from oracle.oracle import Oracle

    o = Oracle("f64")
    g, kw = gradcheck_inputs()
    P = {k: g["in_" + k].astype(np.float64) for k in GROUPS}
    target = g["in_target"].astype(np.float64)

    def render(P, v_img=None):
        return o.render(P["means3d"], P["scales"], P["quats"], P["colors"], P["opacities"],
                        viewmat=g["in_viewmat"], background=g["in_background"], block_size=16,
                        v_img=v_img, **kw)

    def loss(P):
        return float(np.mean((render(P)["img"] - target) ** 2))

    def cdiff(grp, i, j, eps):
        Pp = {k: v.copy() for k, v in P.items()}
        Pm = {k: v.copy() for k, v in P.items()}
        Pp[grp][i, j] += eps
        Pm[grp][i, j] -= eps
        return (loss(Pp) - loss(Pm)) / (2.0 * eps)

    img = render(P)["img"]
    full = render(P, v_img=2.0 * (img - target) / img.size)
    clamped = _frustum_clamped(g, kw)
    visible = np.nonzero(full["radii"].ravel() > 0)[0]
    table = {"_adjoint": {grp: full[GROUPS[grp]] for grp in GROUPS}}
    for gi, grp in enumerate(GROUPS):
        scale = float(np.abs(full[GROUPS[grp]]).max())
        rng = np.random.default_rng(20_000 + gi)
        rows = []
        for _ in range(PER_GROUP):
            i = int(rng.choice(visible))
            j = int(rng.integers(P[grp].shape[1]))
            d1, d2, d4 = (cdiff(grp, i, j, EPS / k) for k in (1, 2, 4))
            r1, r2 = (4 * d2 - d1) / 3, (4 * d4 - d2) / 3
            smooth = abs(r1 - r2) <= SMOOTH_RTOL * max(abs(r1), abs(r2)) + 1e-9 * scale
            rows.append(dict(i=i, j=j, d1=d1, d2=d2, d4=d4, deriv=r2, smooth=smooth,
                             clamped=bool(clamped[i]) and grp in ("means3d", "scales", "quats"),
                             scale=scale))
        table[grp] = rows
    return table


def compare(rows, grad, floor=1e-3):
    """Relative errors of ``grad`` at the usable entries: |a - d| / max(|a|,
    |d|, floor * scale).  Returns (errors of the extrapolated derivative,
    errors of the plain eps = 1e-3 central difference, flagged count)."""
    rich, plain, flagged = [], [], 0
    for r in rows:
        if not r["smooth"] or r["clamped"]:
            flagged += 1
            continue
        a = float(grad[r["i"], r["j"]])
        fl = floor * r["scale"]
        rich.append(abs(a - r["deriv"]) / max(abs(a), abs(r["deriv"]), fl))
        plain.append(abs(a - r["d1"]) / max(abs(a), abs(r["d1"]), fl))
    return np.asarray(rich), np.asarray(plain), flagged
