"""The total-variation term of HashGridEncoder (models/encoders.py:236-254) in the CPU oracle: pinned
to the reference's own encoder (fixtures tv_*.npz, made by running models/encoders.py), its
gradient checked by central differences, and the saturating float-to-uint32 conversion of grid
coordinates at the grid's low faces and below the grid."""
import numpy as np
import pytest

from golden_inputs import TV_CASES, tv_inputs
from oracle import hashgrid as H

from tests.golden_util import load


@pytest.mark.parametrize("case", TV_CASES, ids=lambda c: c["tag"])
def test_tv_golden(case):
    """The float32 restatement gives the reference's value bit for bit, the FP64 one within 1e-6."""
    pos, lat, tab, b = tv_inputs(case)
    want = float(load(case["tag"])["tv"])
    assert float(H.total_variation(pos, lat, b, tab, case["tv_scale"])) == want
    t64 = float(H.total_variation(pos, lat, b, tab, case["tv_scale"], dtype=np.float64))
    assert abs(t64 - want) <= 1e-6 * abs(want)


def test_tv_off():
    pos, lat, tab, b = tv_inputs(TV_CASES[0])
    assert H.total_variation(pos, lat, b, tab, 0.0) == 0


def test_tv_grad_central_differences():
    """TV is quadratic in the table: central differences of the FP64 value equal the gradient."""
    rng = np.random.default_rng(5)
    tab = H.LevelTable(4, 2 ** 10, 2, 4, 32)   # two dense levels, two hashed
    pos = rng.uniform(-1.1, 1.1, size=(300, 3)).astype(np.float32)   # some outside the box
    lat = rng.uniform(-1, 1, size=(tab.n_params, 2))
    s = 0.7
    g = H.total_variation_grad(pos, lat, 1.0, tab, s)
    rows = rng.choice(np.nonzero(np.abs(g).sum(1))[0], 40, replace=False)
    h = 1e-4
    for r in rows:
        for f in range(2):
            lp, lm = lat.copy(), lat.copy()
            lp[r, f] += h
            lm[r, f] -= h
            fd = (H.total_variation(pos, lp, 1.0, tab, s, dtype=np.float64)
                  - H.total_variation(pos, lm, 1.0, tab, s, dtype=np.float64)) / (2 * h)
            assert abs(fd - g[r, f]) <= 1e-9 * max(1.0, abs(g[r, f])), (r, f)


def test_tv_low_face_neighbours_saturate():
    """A point on the grid's low faces has floor(pos_scaled) = 0 on every axis at every level: its
    -1 neighbours convert to coordinate 0, i.e. corner 0's own row, and add nothing to TV."""
    tab = H.LevelTable(6, 2 ** 12, 2, 16, 256)
    pos = np.array([[-1.0, -1.0, -1.0]], np.float32)
    r0, ra = H.tv_rows(H.normalize(pos, 1.0), tab)
    assert (ra[:, :, 3:] == r0[:, :, None]).all()
    assert (ra[:, :, :3] != r0[:, :, None]).all()


def test_corners_below_the_grid_saturate():
    """A coordinate below the grid converts to 0 for both corners of the axis (floor - 0 and
    floor + 1 are both <= 0), so x-neighbour corners share rows; inside the box they differ."""
    tab = H.LevelTable(4, 2 ** 12, 2, 16, 64)
    pos = np.array([[-1.5, 0.1, 0.2], [0.3, 0.1, 0.2]], np.float32)
    idx, _, ps = H.corner_indices(H.normalize(pos, 1.0), tab)
    assert (np.floor(ps[:, 0, 0]) <= -1).all()
    assert (idx[:, 0, :4] == idx[:, 0, 4:]).all()
    assert (idx[:, 1, :4] != idx[:, 1, 4:]).all()
    assert np.array_equal(H.coords_u32(np.array([-3.0, -1.0, -0.0, 0.0, 5.0, np.nan, 5e9])),
                          np.array([0, 0, 0, 0, 5, 0, 4294967295], np.uint32))
