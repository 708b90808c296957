"""FP64 central finite differences against the oracle's fp64 adjoint (the
restatement of the reference's hand-written backward) on the 20k-Gaussian
128x128 gradient-check scene: 200 seed-chosen scalar entries, 40 per
parameter group.  How the differences are taken and which entries are
flagged as non-smooth: tests/fd_entries.py.

Bounds, on the entries that are not flagged: the Richardson-extrapolated
difference agrees with the adjoint to 1e-6 relative at every entry (measured
at most ~2e-7); the plain eps = 1e-3 central difference to 2e-3 (its own
O(eps^2) error, ~5e-4 at the 90th percentile for means and scales)."""

import numpy as np
import pytest

from fd_entries import GROUPS, PER_GROUP, compare, fd_table

RICH_MAX = 1e-6
PLAIN_MAX = 2e-3
# scales change tile sets (through the radius) most often: up to 3/4 of the
# sampled scale entries have a switch inside the stencil
MIN_SMOOTH = {"means3d": 20, "scales": 10, "quats": 20, "colors": 20, "opacities": 20}


@pytest.mark.parametrize("grp", list(GROUPS))
def test_fd_gradcheck_fp64(grp):
    table = fd_table()
    rich, plain, flagged = compare(table[grp], table["_adjoint"][grp])
    print(f"\n{grp}: {rich.size} smooth entries, {flagged} flagged; extrapolated rel err max "
          f"{rich.max():.3g}; eps=1e-3 rel err median {np.median(plain):.3g} max {plain.max():.3g}")
    assert rich.size + flagged == PER_GROUP
    assert rich.size >= MIN_SMOOTH[grp]
    assert rich.max() <= RICH_MAX
    assert plain.max() <= PLAIN_MAX
