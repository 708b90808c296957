"""Pin the CPU oracle against the reference kernels' own outputs.

The golden fixtures were produced by the reference's CUDA kernels (built from
its sources, run through oracle/ref_harness.cu; see
tests/golden/make_golden.py).  The fp32 oracle must reproduce every integer
and index output bit for bit, and the float outputs within the tolerances
of the render path; the fp64 transcription within the same tolerances.
"""

import numpy as np
import pytest

from conftest import (GOLDEN_CASES, GRAD_KEYS, GRAD_RTOL, IMG_ATOL, INT_KEYS, golden_kwargs,
                      load_golden, load_small_digests, normwise_rel)
from oracle.oracle import Oracle


@pytest.fixture(scope="module")
def o32():
    return Oracle("f32")


@pytest.fixture(scope="module")
def o64():
    return Oracle("f64")


def _render(o, g):
    return o.render(g["in_means3d"], g["in_scales"], g["in_quats"], g["in_colors"],
                    g["in_opacities"], viewmat=g["in_viewmat"], background=g["in_background"],
                    block_size=int(g["block_width"]), v_img=g["out_v_img"], **golden_kwargs(g))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_f32_integer_outputs_bit_exact(o32, case):
    g = load_golden(case)
    out = _render(o32, g)
    for k in INT_KEYS:
        np.testing.assert_array_equal(out[k], g["out_" + k], err_msg=k)
    # the projected centres and depths feed the keys: also bit-exact
    np.testing.assert_array_equal(out["xys"], g["out_xys"])
    np.testing.assert_array_equal(out["depths"], g["out_depths"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_float_outputs_within_tolerance(o32, o64, case, prec):
    g = load_golden(case)
    out = _render(o32 if prec == "f32" else o64, g)
    for k in ("img", "final_Ts"):
        assert np.abs(out[k] - g["out_" + k]).max() <= IMG_ATOL, k
    for k in ("cov3d", "conics", "compensation"):
        assert normwise_rel(out[k], g["out_" + k]) <= 1e-5, k
    for k in GRAD_KEYS + ["v_xy_abs", "v_cov2d", "v_cov3d"]:
        assert normwise_rel(out[k], g["out_" + k]) <= GRAD_RTOL, k


def test_oracle_f64_integer_outputs(o64):
    """The FP64 transcription reaches the same tile counts and sort order on
    the 20k-Gaussian case (no decision sits on a rounding boundary there)."""
    g = load_golden("gradcheck")
    out = _render(o64, g)
    for k in ("radii", "num_tiles_hit", "gaussian_ids_sorted", "tile_bins"):
        np.testing.assert_array_equal(out[k], g["out_" + k], err_msg=k)


def test_oracle_matches_reference_digests_100k(o32):
    """100k Gaussians at 256x256 (the small benchmark scene): the oracle's
    integer outputs hash to the reference's digests."""
    import hashlib

    from make_golden import INPUT_KEYS, spec_inputs

    d = load_small_digests()
    inp = spec_inputs("small", 0)
    for k in INPUT_KEYS:
        h = hashlib.sha256(np.ascontiguousarray(inp[k]).tobytes()).hexdigest()
        if h != d["inputs_sha256"][k]:
            pytest.skip(f"seeded input {k} differs from the fixture's (numpy RNG stream changed)")
    kw = dict(img_shape=tuple(int(x) for x in inp["img_shape"]), f=tuple(inp["f"]),
              c=tuple(inp["c"]), glob_scale=float(inp["glob_scale"]),
              clip_thresh=float(inp["clip_thresh"]))
    out = o32.render(inp["means3d"], inp["scales"], inp["quats"], inp["colors"],
                     inp["opacities"], viewmat=inp["viewmat"], background=inp["background"],
                     block_size=16, **kw)
    for k in INT_KEYS:
        got = hashlib.sha256(np.ascontiguousarray(out[k]).tobytes()).hexdigest()
        assert got == d["sha256"][k], k
    st = d["stats"]["img"]
    assert abs(float(out["img"].astype(np.float64).sum()) - st["sum"]) <= 1e-5 * out["img"].size
