"""Deterministic inputs shared by the golden-fixture generator and the tests.

Large inputs (hash tables, MLP weights, query points) are rebuilt here from the seeds recorded in
the fixtures, so the fixtures only hold outputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from oracle.hashgrid import LevelTable  # noqa: E402
from oracle.field import init_weights  # noqa: E402

# Hash-grid cases: the training configuration (L=16, F=2, T=2^19, N_min=16, N_max=2048*bound),
# a small all-levels-dense table, and a bound-2 scene.
HASHGRID_CASES = [
    dict(tag="ngp_b1", L=16, T=2**19, F=2, N_min=16, N_max=2048, bound=1.0, n=2048, seed=11),
    dict(tag="small_dense", L=4, T=2**14, F=2, N_min=4, N_max=16, bound=1.0, n=1024, seed=12),
    dict(tag="ngp_b2", L=16, T=2**16, F=2, N_min=16, N_max=4096, bound=2.0, n=1024, seed=13),
]

# Total-variation cases (encoders.py:236-254 with tv_scale > 0): a small table with dense and hashed
# levels and the training configuration.  Points keep clear of the grid's low faces, where the -1
# neighbour's float-to-uint32 conversion is the platform's (the tests cover that case separately).
TV_CASES = [
    dict(tag="tv_small", L=8, T=2**12, F=2, N_min=16, N_max=512, bound=1.0, n=1024, seed=31, tv_scale=0.37),
    dict(tag="tv_ngp", L=16, T=2**19, F=2, N_min=16, N_max=2048, bound=1.0, n=2048, seed=32, tv_scale=1e-3),
]

FIELD_CASE = dict(L=16, T=2**19, F=2, N_min=16, N_max=2048, bound=1.0, n=1024, seed=21,
                  weight_seed=22)


def tv_inputs(case):
    """Returns (positions [n,3], latents [P,F], LevelTable, bound) for a TV case: positions with
    (pos + bound) / (2 bound) >= 0.075, so floor(pos_scaled) >= 1 at every level (N_min = 16)."""
    tab = LevelTable(case["L"], case["T"], case["F"], case["N_min"], case["N_max"])
    rng = np.random.default_rng(case["seed"])
    b = case["bound"]
    pos = rng.uniform(-0.85 * b, 0.95 * b, size=(case["n"], 3)).astype(np.float32)
    latents = rng.uniform(-1, 1, size=(tab.n_params, tab.F)).astype(np.float32)
    return pos, latents, tab, b


def hashgrid_inputs(case):
    """Returns (positions [n,3] in [-bound, bound], latents [P,F], LevelTable, bound)."""
    tab = LevelTable(case["L"], case["T"], case["F"], case["N_min"], case["N_max"])
    rng = np.random.default_rng(case["seed"])
    b = case["bound"]
    pos = rng.uniform(-b, b, size=(case["n"], 3)).astype(np.float32)
    # edge positions: the box corners and faces, and points on cell boundaries of level 0
    edge = np.array([[-b, -b, -b], [b, b, b], [b, -b, 0.0], [0.0, 0.0, 0.0], [-b, b, b]],
                    np.float32)
    pos[: len(edge)] = edge
    latents = rng.uniform(-1e-4, 1e-4, size=(tab.n_params, tab.F)).astype(np.float32)
    # larger values in a few rows so that every corner contributes visibly
    latents *= np.float32(1e4)
    return pos, latents, tab, b


def field_inputs(case):
    """Returns (positions, unit directions, latents, MLP weights, LevelTable, bound)."""
    tab = LevelTable(case["L"], case["T"], case["F"], case["N_min"], case["N_max"])
    rng = np.random.default_rng(case["seed"])
    b = case["bound"]
    pos = rng.uniform(-b, b, size=(case["n"], 3)).astype(np.float32)
    d = rng.normal(size=(case["n"], 3))
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    latents = rng.uniform(-1, 1, size=(tab.n_params, tab.F)).astype(np.float32)
    w = init_weights(case["weight_seed"])
    return pos, dirs, latents, w, tab, b


def near_far(bound: float, o: np.ndarray, d: np.ndarray):
    """models/renderers/cuda.py:56-97 in float32."""
    eps = np.float32(1e-15)
    d = np.where(np.signbit(d), np.minimum(d, -eps), np.maximum(d, eps)).astype(np.float32)
    b = np.float32(bound)
    t0 = (-b - o) / d
    t1 = (b - o) / d
    ts = np.maximum(np.float32(0), np.minimum(t0, t1).max(-1)).astype(np.float32)
    te = np.maximum(t0, t1).min(-1).astype(np.float32)
    return ts, te


def make_rays(rng: np.random.Generator, n: int, bound: float):
    """Rays from a sphere of radius 3*bound towards random points in the box."""
    o = rng.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=-1, keepdims=True) * 3 * bound
    tgt = rng.uniform(-0.9 * bound, 0.9 * bound, size=(n, 3))
    d = tgt - o
    d = d / np.linalg.norm(d, axis=-1, keepdims=True)
    o, d = o.astype(np.float32), d.astype(np.float32)
    t0, t1 = near_far(bound, o, d)
    return o, d, t0, t1


def random_bitfield(rng: np.random.Generator, K: int, G: int, density: float) -> np.ndarray:
    n = K * G ** 3
    if density <= 0:
        return np.zeros(n // 8, np.uint8)
    if density >= 1:
        return np.full(n // 8, 255, np.uint8)
    return np.packbits(rng.uniform(size=n) < density, bitorder="little")
