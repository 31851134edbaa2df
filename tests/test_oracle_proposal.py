"""CPU checks of the proposal oracle's own invariants (no reference counterpart exists)."""
import numpy as np

from golden_inputs import make_rays
from oracle import proposal as P


def blob_bitfield(G, centres, radius):
    """Occupancy bits (Morton order) of the cells whose centre lies within `radius` of a centre."""
    g = (np.arange(G) + 0.5) / G * 2 - 1
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    occ = np.zeros((G, G, G), bool)
    for c in centres:
        occ |= (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 < radius ** 2
    idx = np.arange(G)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    bits = np.zeros(G ** 3, np.uint8)
    bits[P._morton3(I, J, K)] = occ
    return np.packbits(bits, bitorder="little")


CENTRES = [(0.3, -0.2, 0.1), (-0.4, 0.35, -0.3)]


def test_coarse_grid_covers_occupied_cells():
    G = 64
    bits = blob_bitfield(G, CENTRES, 0.15)
    coarse = P.coarse_grid(bits, G)
    Gc = G // 8
    occ = np.unpackbits(bits, bitorder="little").astype(bool)
    idx = np.arange(G)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    dense = occ[P._morton3(I, J, K)]
    for x, y, z in zip(*np.nonzero(dense)):
        assert coarse[x // 8 + (y // 8) * Gc + (z // 8) * Gc * Gc]
    assert 0 < coarse.mean() < 0.5


def test_interval_contains_every_occupied_crossing():
    """Dense point sampling of each ray never finds an occupied fine cell outside [t_a, t_b]."""
    G = 64
    bits = blob_bitfield(G, CENTRES, 0.15)
    coarse = P.coarse_grid(bits, G)
    occ = np.unpackbits(bits, bitorder="little").astype(bool)
    rng = np.random.default_rng(0)
    o, d, t0, t1 = make_rays(rng, 300, 1.0)
    hits = 0
    for i in range(len(o)):
        hit, ta, tb = P.ray_interval(o[i], d[i], t0[i], t1[i], coarse, G // 8, 1.0)
        ts = np.linspace(t0[i], t1[i], 2000)
        pts = o[i][None] + ts[:, None] * d[i][None]
        c = np.clip(np.floor((pts + 1) / 2 * G).astype(int), 0, G - 1)
        inside = occ[P._morton3(c[:, 0], c[:, 1], c[:, 2])]
        if inside.any():
            assert hit
            assert ta <= ts[inside].min() + 1e-6 and ts[inside].max() <= tb + 1e-6
        hits += hit
    assert 0 < hits < len(o)


def test_samples_are_sorted_and_follow_the_density():
    rng = np.random.default_rng(1)
    x = np.full(P.N_BINS, -8.0, np.float32)
    x[40:44] = 3.0           # a dense slab in bins 40..43
    t, ds = P.sample_ray(x, 1.0, 3.0, np.full(P.N_SAMPLES, 0.5, np.float32))
    assert np.all(np.diff(t) >= 0) and np.all(ds >= 0)
    assert t[0] >= 1.0 and t[-1] <= 3.0
    lo, hi = 1.0 + 40 * 2.0 / 64, 1.0 + 44 * 2.0 / 64
    assert ((t >= lo) & (t <= hi)).mean() > 0.8
    # the uniform mixture still reaches every part of the interval
    t2, _ = P.sample_ray(np.full(P.N_BINS, -30.0, np.float32), 1.0, 3.0, rng.uniform(size=P.N_SAMPLES))
    assert np.allclose(np.sort(t2), t2) and t2.min() < 1.2 and t2.max() > 2.8


def test_mlp_backward_matches_finite_differences():
    rng = np.random.default_rng(2)
    w = P.init_weights(3)
    e = rng.normal(size=(20, 8))
    g = rng.normal(size=20)
    _, cache = P.mlp_forward(e, w, dtype=np.float64)
    de, gw = P.mlp_backward(g, cache, w)
    h = 1e-6
    for k in ("P0", "P1", "P2"):
        for _ in range(5):
            i, j = rng.integers(w[k].shape[0]), rng.integers(w[k].shape[1])
            wp = {a: b.astype(np.float64).copy() for a, b in w.items()}
            wm = {a: b.astype(np.float64).copy() for a, b in w.items()}
            wp[k][i, j] += h
            wm[k][i, j] -= h
            fd = ((P.mlp_forward(e, wp, np.float64)[0] - P.mlp_forward(e, wm, np.float64)[0]) @ g) / (2 * h)
            assert abs(fd - gw[k][i, j]) <= 1e-6 * max(1.0, abs(fd))
    ep, em = e.copy(), e.copy()
    ep[3, 5] += h
    em[3, 5] -= h
    fd = ((P.mlp_forward(ep, w, np.float64)[0] - P.mlp_forward(em, w, np.float64)[0]) @ g) / (2 * h)
    assert abs(fd - de[3, 5]) <= 1e-6 * max(1.0, abs(fd))
