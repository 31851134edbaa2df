"""The CPU restatements behind the training-step parity tests (no GPU): the optax chain and its
schedule (oracle/optim.py, app/nerf/_utils.py:19-77), the occupancy-grid maintenance
(oracle/ogrid.py, utils/types.py:1149-1362) and the FP32-kernel emulation of the field forward
(oracle.field.forward_fma32)."""
import math

import numpy as np
import pytest

from oracle import field as Fd
from oracle import ogrid as OG
from oracle import optim as OP


@pytest.mark.parametrize("count,want", [(0, 1e-2), (9999, 1e-2), (10000, 1e-2), (19999, 1e-2), (20000, 1e-2 / 3),
                                        (29999, 1e-2 / 3), (30000, 1e-2 / 9), (50000, 1e-2 / 81),
                                        (60000, 1e-4), (10 ** 6, 1e-4)])
def test_reference_schedule(count, want):
    """exponential_decay(1e-2, 10k, 1/3, staircase, begin 10k, end 1e-4): held for 20k steps, then
    a third every 10k steps, floored at lr/100."""
    assert abs(OP.reference_lr(count) - want) <= 1e-6 * want


def test_adam_restatement_against_float64():
    rng = np.random.default_rng(0)
    n = 4096
    p = rng.uniform(-1, 1, n).astype(np.float32)
    g = (rng.normal(size=n) * 1e-3).astype(np.float32)
    m = (rng.normal(size=n) * 1e-4).astype(np.float32)
    v = (rng.uniform(size=n) * 1e-7).astype(np.float32)
    for count, wd in ((0, 0.0), (7, 1e-6), (25000, 1e-6)):
        lr = OP.reference_lr(count)
        p1, m1, v1 = OP.adam_update(p, g, m, v, count, lr, weight_decay=wd)
        # float64 with the float32 constants the chain uses (0.9f is 0.899999976...)
        b1, b2 = float(np.float32(0.9)), float(np.float32(0.99))
        P, Gd, M, Vd = (x.astype(np.float64) for x in (p, g, m, v))
        M = (1 - b1) * Gd + b1 * M
        Vd = (1 - b2) * Gd * Gd + b2 * Vd
        t = count + 1
        u = (M / (1 - b1 ** t)) / (np.sqrt(Vd / (1 - b2 ** t) + 1e-15) + 1e-15)
        P = P - lr * u + wd * P
        assert np.abs(m1 - M).max() <= 1e-6 * np.abs(M).max()
        assert np.abs(v1 - Vd).max() <= 1e-6 * np.abs(Vd).max()
        assert np.all(np.abs(p1 - P) <= 1e-6 * (np.abs(P) + lr))


def test_ogrid_decay_max_threshold():
    G = 4
    d = np.array([-1.0, 0.0, 2.0, 10.0] * (G ** 3 // 4), np.float32)
    d2 = OG.decay(d, 0, G)
    assert (d2[d < 0] == -1).all() and np.allclose(d2[d >= 0], d[d >= 0] * np.float32(0.95))
    cells = np.array([1, 1, 2, 5], np.int64)
    sig = np.array([3.0, 4.0, 1.0, 0.5], np.float32)
    d3 = OG.max_update(d2, 0, G, cells, sig)
    assert d3[1] == 4.0 and d3[2] == np.float32(2.0) * np.float32(0.95) and d3[5] == 0.5
    live = d3[d3 >= 0]
    assert OG.threshold(d3, G, 1024, 1.0) == pytest.approx(min(0.01 * 1024 / (2 * math.sqrt(3)), live.mean()))
    assert OG.threshold_step(1024, 1.0) == pytest.approx(2.9559, rel=1e-4)


def test_cell_points_base():
    """types.py:1195-1199: cell i of G maps to (i/(G-1)*2-1)*(mip_bound - hcw), so the jittered
    point (+-hcw) stays inside [-mip_bound, mip_bound]."""
    G = 8
    cells = np.arange(G ** 3, dtype=np.uint32)
    base, hcw = OG.cell_points_base(cells, 0, G, 1.0)
    assert hcw == pytest.approx(1 / 8)
    assert np.abs(base).max() + hcw <= 1.0 + 1e-6
    assert base.min() == pytest.approx(-(1 - 1 / 8))


def _look_at(pos):
    pos = np.asarray(pos, np.float64)
    fwd = -pos / np.linalg.norm(pos)
    right = np.cross(fwd, (0.0, 0.0, 1.0))
    if np.linalg.norm(right) < 1e-8:
        right = np.cross(fwd, (0.0, 1.0, 0.0))
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    R = np.stack([right, up, -fwd], axis=1)
    return np.concatenate([R.reshape(-1), pos]).astype(np.float32)


def test_mark_untrained_geometry():
    """One narrow camera on the +x axis looking at the origin: the cells around the origin are
    seen, the cells of the box's far corners outside its frustum are not; and the result equals a
    float64 projection of each cell's 8 corners except within float rounding of the frustum."""
    G, bound = 16, 1.0
    W = H = 32
    f = (W / 2) / math.tan(math.radians(10) / 2)
    tf = _look_at((6.0, 0.0, 0.0))[None]
    alive = OG.mark_untrained(1, G, bound, tf, W, H, f, f, W / 2, H / 2)
    from oracle import volrend as V
    xyz = V.morton3d_invert(np.arange(G ** 3, dtype=np.uint32)).astype(np.float64)
    lo = (xyz / G - 0.5) * 2 * bound
    centre = lo + bound / G
    assert alive[np.argmin(np.linalg.norm(centre, axis=1))]
    far = np.argmax(np.abs(centre[:, 1]) + np.abs(centre[:, 2]))
    assert not alive[far]
    R = tf[0, :9].reshape(3, 3).astype(np.float64)
    t = tf[0, 9:].astype(np.float64)
    seen = np.zeros(G ** 3, bool)
    margin = np.zeros(G ** 3)
    for k in range(8):
        v = lo + (2 * bound / G) * np.array([(k >> 2) & 1, (k >> 1) & 1, k & 1])
        pc = (v - t) @ R
        u = (pc[:, 0] / -pc[:, 2] * f + W / 2) / W
        w = (pc[:, 1] / -pc[:, 2] * f + H / 2) / H
        ok = (pc[:, 2] < 0) & (u >= 0) & (u < 1) & (w >= 0) & (w < 1)
        seen |= ok
        margin = np.maximum(margin, np.minimum.reduce([u, 1 - u, w, 1 - w]))
    near_edge = np.abs(margin) < 1e-5
    assert np.array_equal(alive[~near_edge], seen[~near_edge])
    assert 0 < alive.mean() < 1


def test_forward_fma32_matches_fp64():
    """The FP32-kernel emulation is a float32 evaluation: within float32 rounding of FP64."""
    rng = np.random.default_rng(1)
    n = 2048
    enc = rng.normal(scale=0.5, size=(n, 32)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    dirs = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    w = Fd.init_weights(3)
    a, cache = Fd.forward_fma32(enc, dirs, w)
    b, c64 = Fd.forward(enc, dirs, w, dtype=np.float64)
    assert (np.abs(a - b).max(0) / np.abs(b).max(0)).max() <= 1e-6
    assert np.abs(Fd.sh4_fma32(dirs) - Fd.sh4(dirs.astype(np.float64))).max() <= 1e-6
    for k in ("a1", "a2", "a3"):
        assert np.abs(cache[k] - c64[k]).max() <= 1e-5 * np.abs(c64[k]).max()
