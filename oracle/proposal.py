"""CPU oracle for the learned proposal sampler.  TEST INFRASTRUCTURE ONLY.

The reference has no proposal sampler (it marches the occupancy grid only); this module restates
the project's own algorithm so the GPU kernels have a checker:

  coarse grid   a byte per block of 8^3 fine occupancy cells: 1 when any fine cell of the block,
                grown by one fine cell on every side, is occupied (cascade 0, Morton-ordered bits
                as in the reference's bitfield, marching.cu:79-98)
  interval      a 3D DDA over the coarse grid from t_start to t_end; the ray's interval runs from
                the entry of its first occupied block to the exit of its last; no occupied block
                means no samples (the ray is valid and shows its background)
  bins          N_BINS equal bins over the interval; the proposal field (4-level hash grid, MLP
                8 -> 64 -> 64 -> 1, relu, exp density) at the bin centres
  samples       weights w_i = T_i (1 - exp(-sigma_i delta)) with T_i = exp(-delta sum_{k<i} sigma_k)
                (1 - exp as -expm1), normalised (uniform when they are all zero) and mixed with MIX
                of a uniform density, form a piecewise-constant pdf; its inverse CDF at
                u_0 = 0, u_k = (k - 1/2 + xi_k) / N_SAMPLES (0 < k < N_SAMPLES), u_N = 1 gives
                N_SAMPLES + 1 edges from t_a to t_b; sample k sits at the midpoint of
                [e_k, e_{k+1}] and stands for that interval, so the samples' intervals partition
                [t_a, t_b] and crowd where the pdf is high
  training      the proposal's log density regresses the field's log density at the field's own
                samples (and at points drawn in occupied cells): L = mean w (x - log(sigma_f + EPS))^2
                with w = UNDER when the proposal is below the target, else 1

Float32 throughout, one rounding per operation in the order written here (the GPU file is built
without FMA contraction); exp differs from CUDA's by an ulp, so tests compare within tolerance.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

from . import hashgrid as H

N_BINS = 64
N_SAMPLES = 48
MIX = np.float32(0.1)
EPS = np.float32(1e-3)
UNDER = np.float32(2.0)
SHAPES = {"P0": (8, 64), "P1": (64, 64), "P2": (64, 1)}
N_WEIGHTS = 8 * 64 + 64 * 64 + 64


def table(bound: float = 1.0) -> H.LevelTable:
    """4 levels, 2^16 rows per level, resolutions 16..128 (scale 2 per level)."""
    return H.LevelTable(4, 1 << 16, 2, 16, 128)


def init_weights(seed: int = 0) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    out = {}
    for k, (a, b) in SHAPES.items():
        lim = np.sqrt(6.0 / (a + b))
        out[k] = rng.uniform(-lim, lim, size=(a, b)).astype(np.float32)
    return out


def pack(w: Dict[str, np.ndarray]) -> np.ndarray:
    return np.concatenate([w[k].ravel() for k in SHAPES]).astype(np.float32)


def unpack(flat: np.ndarray) -> Dict[str, np.ndarray]:
    out, off = {}, 0
    for k, (a, b) in SHAPES.items():
        out[k] = np.asarray(flat[off:off + a * b], np.float32).reshape(a, b)
        off += a * b
    return out


# ------------------------------------------------------------------------------ coarse grid

def _morton3(x, y, z):
    def expand(v):
        v = np.asarray(v, np.uint64)
        v = (v * 0x00010001) & 0xFF0000FF
        v = (v * 0x00000101) & 0x0F00F00F
        v = (v * 0x00000011) & 0xC30C30C3
        v = (v * 0x00000005) & 0x49249249
        return v
    return (expand(x) | (expand(y) << 1) | (expand(z) << 2)).astype(np.uint32)


def coarse_grid(bits: np.ndarray, G: int) -> np.ndarray:
    """u8 [Gc^3], index x + y Gc + z Gc^2 with Gc = G / 8."""
    occ = np.unpackbits(np.asarray(bits, np.uint8), bitorder="little").astype(bool)
    g = np.arange(G)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    dense = occ[_morton3(X, Y, Z)]                       # [x, y, z]
    grown = dense.copy()
    for axis in range(3):                                 # dilate by one fine cell
        a = grown.copy()
        sl_lo = [slice(None)] * 3
        sl_hi = [slice(None)] * 3
        sl_lo[axis], sl_hi[axis] = slice(0, G - 1), slice(1, G)
        a[tuple(sl_lo)] |= grown[tuple(sl_hi)]
        a[tuple(sl_hi)] |= grown[tuple(sl_lo)]
        grown = a
    Gc = G // 8
    blocks = grown.reshape(Gc, 8, Gc, 8, Gc, 8).any(axis=(1, 3, 5))   # [cx, cy, cz]
    return np.ascontiguousarray(blocks.transpose(2, 1, 0)).reshape(-1).astype(np.uint8)


def ray_interval(o, d, t0, t1, coarse: np.ndarray, Gc: int, mb: float):
    """(hit, t_a, t_b) of one ray: the coarse-grid DDA."""
    f = np.float32
    o = np.asarray(o, f)
    d = np.asarray(d, f)
    t0, t1, mb = f(t0), f(t1), f(mb)
    if not t0 < t1:
        return False, f(0), f(0)
    scale = f(Gc) / (f(2) * mb)
    cell, tmax, tdel, step = [0] * 3, [f(0)] * 3, [f(0)] * 3, [0] * 3
    for a in range(3):
        g = (o[a] + t0 * d[a] + mb) * scale
        c = int(np.floor(g))
        cell[a] = min(max(c, 0), Gc - 1)
        if d[a] > 0:
            step[a] = 1
            tmax[a] = ((f(cell[a] + 1) / scale - mb) - o[a]) / d[a]
            tdel[a] = (f(1) / scale) / d[a]
        elif d[a] < 0:
            step[a] = -1
            tmax[a] = ((f(cell[a]) / scale - mb) - o[a]) / d[a]
            tdel[a] = (f(-1) / scale) / d[a]
        else:
            step[a] = 0
            tmax[a] = f(np.inf)
            tdel[a] = f(np.inf)
    t = t0
    hit, ta, tb = False, f(0), f(0)
    for _ in range(3 * Gc + 3):
        if not t < t1:
            break
        # first axis reaching the smallest boundary, in x, y, z order on ties
        m = min(tmax)
        a = 0 if tmax[0] == m else (1 if tmax[1] == m else 2)
        tn = min(m, t1)
        if coarse[cell[0] + cell[1] * Gc + cell[2] * Gc * Gc]:
            if not hit:
                ta = t
            hit, tb = True, tn
        cell[a] += step[a]
        if cell[a] < 0 or cell[a] >= Gc:
            break
        t = m
        tmax[a] = f(tmax[a] + tdel[a])
    return hit and tb > ta, ta, tb


# ------------------------------------------------------------------------------ proposal MLP

def mlp_forward(enc: np.ndarray, w: Dict[str, np.ndarray], dtype=np.float32):
    w = {k: np.asarray(v, dtype) for k, v in w.items()}
    e = np.asarray(enc, dtype)
    a1 = e @ w["P0"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ w["P1"]
    h2 = np.maximum(a2, 0)
    x = (h2 @ w["P2"])[:, 0]
    return x, dict(e=e, a1=a1, h1=h1, a2=a2, h2=h2)


def mlp_backward(dx: np.ndarray, cache, w: Dict[str, np.ndarray], dtype=np.float64):
    w = {k: np.asarray(v, dtype) for k, v in w.items()}
    c = {k: np.asarray(v, dtype) for k, v in cache.items()}
    g = np.asarray(dx, dtype)[:, None]
    grads = {"P2": c["h2"].T @ g}
    d2 = (g @ w["P2"].T) * (c["a2"] > 0)
    grads["P1"] = c["h1"].T @ d2
    d1 = (d2 @ w["P1"].T) * (c["a1"] > 0)
    grads["P0"] = c["e"].T @ d1
    return d1 @ w["P0"].T, grads


def loss_grad(x: np.ndarray, sigma_f: np.ndarray, n: int) -> Tuple[np.ndarray, float]:
    """dL/dx and the loss sum for the log-density regression over n points."""
    f = np.float32
    y = np.log(np.asarray(sigma_f, f) + EPS).astype(f)
    r = (np.asarray(x, f) - y).astype(f)
    w = np.where(r < 0, UNDER, f(1)).astype(f)
    g = (f(2) * w * r / f(n)).astype(f)
    return g, float((w * r * r).sum())


# ------------------------------------------------------------------------------ sampling

def bin_points(o, d, ta, tb):
    f = np.float32
    o, d = np.asarray(o, f), np.asarray(d, f)
    delta = (f(tb) - f(ta)) / f(N_BINS)
    c = np.array([f(ta) + (f(i) + f(0.5)) * delta for i in range(N_BINS)], f)
    return (o[None, :] + c[:, None] * d[None, :]).astype(f), delta


def sample_ray(x_bins: np.ndarray, ta: float, tb: float, xi: np.ndarray, n_samples: int = N_SAMPLES, mix=MIX):
    """Returns (t [n_samples], ds [n_samples]) for one ray; xi[k] jitters edge k (0 < k < n_samples)."""
    f = np.float32
    ta, tb = f(ta), f(tb)
    delta = (tb - ta) / f(N_BINS)
    w = np.empty(N_BINS, f)
    acc = f(0)
    W = f(0)
    for i in range(N_BINS):
        s = f(np.exp(np.clip(f(x_bins[i]), f(-15), f(15))))
        T = f(np.exp(-(delta * acc)))
        a = f(-np.expm1(-(s * delta)))
        w[i] = T * a
        W = W + w[i]
        acc = acc + s
    p = np.empty(N_BINS, f)
    for i in range(N_BINS):
        wi = (w[i] / W) if W > 0 else f(1) / f(N_BINS)
        p[i] = (f(1) - f(mix)) * wi + f(mix) / f(N_BINS)
    e = np.empty(n_samples + 1, f)
    e[0], e[n_samples] = ta, tb
    b, c_lo, c_hi = 0, f(0), p[0]
    for k in range(1, n_samples):
        u = (f(k) - f(0.5) + f(xi[k])) / f(n_samples)
        while u >= c_hi and b < N_BINS - 1:
            b += 1
            c_lo = c_hi
            c_hi = c_hi + p[b]
        frac = min(max((u - c_lo) / p[b], f(0)), f(1))
        e[k] = ta + (f(b) + frac) * delta
    t = ((e[:-1] + e[1:]) * f(0.5)).astype(f)
    ds = (e[1:] - e[:-1]).astype(f)
    return t, ds


MISS_LIMIT = 0.01


def missed_transmittance(x_bins: np.ndarray, ta: float, tb: float, o, d, bits: np.ndarray, G: int, bound: float,
                         threshold: float) -> float:
    """The per-ray fallback test (ngp_proposal_judge), in float64: the occupancy grid marks the bins
    whose cell holds density >= threshold; where the proposal's density sigma_i is below that the
    proposal misses mass, and the transmittance it misses is
    sum over occupied bins of T_i (1 - exp(-(threshold - sigma_i) delta)), T_i = exp(-delta
    sum_{j<i} sigma_j).  A ray is marched instead when this exceeds MISS_LIMIT."""
    f = np.float32
    occ = np.unpackbits(np.asarray(bits, np.uint8), bitorder="little").astype(bool)
    ta64, tb64 = float(f(ta)), float(f(tb))
    delta = (tb64 - ta64) / N_BINS
    s = np.exp(np.clip(np.asarray(x_bins, np.float64), -15, 15))
    acc = np.concatenate([[0.0], np.cumsum(s)[:-1]])
    T = np.exp(-delta * acc)
    mb = min(1.0, float(bound))
    t = ta64 + (np.arange(N_BINS) + 0.5) * delta
    pos = np.asarray(o, np.float64)[None, :] + t[:, None] * np.asarray(d, np.float64)[None, :]
    g = np.clip(np.floor((pos / mb + 1.0) * 0.5 * G), 0, G - 1).astype(np.int64)
    cell_occ = occ[_morton3(g[:, 0], g[:, 1], g[:, 2])]
    short = np.maximum(threshold - s, 0.0)
    return float(np.sum(np.where(cell_occ, T * -np.expm1(-short * delta), 0.0)))
