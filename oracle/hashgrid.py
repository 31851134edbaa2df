"""CPU oracle for the multiresolution hash-grid encoder.  TEST INFRASTRUCTURE ONLY.

A NumPy restatement of ``HashGridEncoder`` (models/encoders.py:58-256) and of the gradient JAX
derives for it (the transpose of the gather at encoders.py:226, a scatter-add into the table).

Float32 evaluation follows the reference's operation order with one rounding per operation:
``pos = (pos + bound) / (2*bound)`` (:87), ``pos_scaled = pos * float32(scale_l) + 0.5`` (:216-218),
corner = floor + {0,1}^3 converted to uint32 (:116-123), dense index ``x + y*res + z*res^2`` for the first
``first_hash_level`` levels (:134-155), hash ``x ^ y*2654435761 ^ z*805459861`` (:157-177), both in
wrapping uint32 arithmetic, then ``mod T`` and ``+ offsets[l]`` (:179-189); lerp weight
``prod_d((1-o_d) + (2 o_d - 1) * frac_d)`` (:191-213); corner sum in corner order (:231); output
column ``l*F + f`` (:233).  A gather index past the table end is clamped to the last row, which is
what JAX's gather does with out-of-range indices.

The float-to-uint32 conversion of the grid coordinates (``astype(jnp.uint32)`` at :123 and :132) is
the one XLA performs on the GPU the reference runs on: it saturates, so a coordinate below the grid
(a point outside the box, or the -1 neighbour of the TV term at the grid's low face) becomes 0 and
NaN becomes 0 (PTX ``cvt.rzi.u32.f32`` clamps to the destination range).  Inside the box every
coordinate is non-negative and the conversion is exact.

The total-variation term (:236-254) and its gradient are ``total_variation`` and
``total_variation_grad``.

``encode(..., dtype=np.float64)`` gives the FP64 twin used for gradient checks.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np

PRIMES = (1, 2654435761, 805459861)
CORNERS = np.array([[(c >> 2) & 1, (c >> 1) & 1, c & 1] for c in range(8)], dtype=np.uint32)
# the six axis neighbours of a cell's corner 0 in the TV term, in the reference's order (:35-49)
ADJACENT = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0], [0, 0, -1], [0, -1, 0], [-1, 0, 0]], dtype=np.int64)


def coords_u32(v: np.ndarray) -> np.ndarray:
    """Float grid coordinates to uint32 as XLA converts them on the GPU: saturating (negative and
    NaN give 0, values past the range give 2^32 - 1), exact for coordinates in range."""
    v = np.asarray(v, np.float64)
    return np.where(v > 0, np.minimum(v, 4294967295.0), 0.0).astype(np.uint32)


def grid_rows(v: np.ndarray, l: int, tab: "LevelTable") -> np.ndarray:
    """Table rows of uint32 grid vertices v [..., 3] at level l: dense ``x + y*res + z*res^2`` or
    hashed ``x ^ y*p1 ^ z*p2`` in wrapping uint32 arithmetic (:134-177), ``mod T`` and
    ``+ offsets[l]`` (:179-189), then clamped to the table like JAX's gather."""
    with np.errstate(over="ignore"):
        if l < tab.first_hash_level:
            r = np.uint32(tab.resolutions[l])
            i = v[..., 0] + v[..., 1] * r + v[..., 2] * (r * r)
        else:
            i = v[..., 0] ^ (v[..., 1] * np.uint32(PRIMES[1])) ^ (v[..., 2] * np.uint32(PRIMES[2]))
        i = i % np.uint32(tab.T) + np.uint32(tab.offsets[l])
    return np.minimum(i, np.uint32(tab.n_params - 1))


@dataclass(frozen=True)
class LevelTable:
    """encoders.py:77-114: per-level scale, resolution, table offsets."""
    L: int
    T: int
    F: int
    N_min: int
    N_max: int
    per_level_scale: float | None = None
    dim: int = 3

    @property
    def b(self) -> float:
        if self.per_level_scale is not None:
            return float(self.per_level_scale)
        return math.exp((math.log(self.N_max) - math.log(self.N_min)) / (self.L - 1))

    def _build(self):
        scales, res, offs, first_hash = [], [], [0], 0
        for i in range(self.L):
            s = self.N_min * (self.b ** i) - 1
            scales.append(s)
            r = math.ceil(s) + 1
            res.append(r)
            n = (r ** self.dim + 7) // 8 * 8
            if n <= self.T:
                first_hash += 1
            else:
                n = self.T
            offs.append(offs[-1] + n)
        return scales, res, offs, first_hash

    @property
    def scales(self) -> List[float]:
        return self._build()[0]

    @property
    def resolutions(self) -> List[int]:
        return self._build()[1]

    @property
    def offsets(self) -> List[int]:
        return self._build()[2]

    @property
    def first_hash_level(self) -> int:
        return self._build()[3]

    @property
    def n_params(self) -> int:
        return self.offsets[-1]


def normalize(pos: np.ndarray, bound: float, dtype=np.float32) -> np.ndarray:
    """encoders.py:87."""
    pos = np.asarray(pos, dtype)
    return (pos + dtype(bound)) / dtype(2 * bound)


def corner_indices(pos01: np.ndarray, tab: LevelTable, dtype=np.float32):
    """Returns (indices [L, N, 8] uint32, weights [L, N, 8], pos_scaled [L, N, 3])."""
    scales = np.asarray(tab.scales, dtype)
    ps = pos01[None, :, :] * scales[:, None, None] + dtype(0.5)
    fl = np.floor(ps)
    vert = coords_u32(fl[:, :, None, :] + CORNERS[None, None, :, :].astype(fl.dtype))   # [L, N, 8, 3]
    idx = np.empty(vert.shape[:3], np.uint32)
    for l in range(tab.L):
        idx[l] = grid_rows(vert[l], l, tab)
    frac = np.modf(ps)[0]
    o = CORNERS.astype(dtype)
    w3 = (dtype(1) - o)[None, None] + (dtype(2) * o - dtype(1))[None, None] * frac[:, :, None, :]
    w3 = np.clip(w3, dtype(0), dtype(1))
    w = (w3[..., 0] * w3[..., 1]) * w3[..., 2]
    return idx, w.astype(dtype), ps


def encode(pos: np.ndarray, latents: np.ndarray, bound: float, tab: LevelTable, dtype=np.float32):
    """HashGridEncoder.__call__ without the TV term: returns enc [N, L*F]."""
    p01 = normalize(pos, bound, dtype)
    idx, w, _ = corner_indices(p01, tab, dtype)
    lat = np.asarray(latents, dtype)
    acc = lat[idx[:, :, 0]] * w[:, :, 0, None]
    for c in range(1, 8):
        acc = acc + lat[idx[:, :, c]] * w[:, :, c, None]
    n = p01.shape[0]
    return np.ascontiguousarray(acc.transpose(1, 0, 2).reshape(n, tab.L * tab.F))


def encode_as_f32(pos: np.ndarray, latents: np.ndarray, bound: float, tab: LevelTable) -> np.ndarray:
    """The float32 encoder's corners and weights (the ones the GPU and the reference compute) applied
    to float64 latents: the encoder as a function of the table, for central differences."""
    p01 = normalize(pos, bound, np.float32)
    idx, w, _ = corner_indices(p01, tab, np.float32)
    lat = np.asarray(latents, np.float64)
    w = w.astype(np.float64)
    acc = lat[idx[:, :, 0]] * w[:, :, 0, None]
    for c in range(1, 8):
        acc = acc + lat[idx[:, :, c]] * w[:, :, c, None]
    n = p01.shape[0]
    return np.ascontiguousarray(acc.transpose(1, 0, 2).reshape(n, tab.L * tab.F))


def encode_backward(pos: np.ndarray, dL_denc: np.ndarray, bound: float, tab: LevelTable,
                    dtype=np.float64) -> np.ndarray:
    """dL/dlatents [P, F]: scatter-add of w * dL/denc (the transpose of the gather)."""
    p01 = normalize(pos, bound, np.float32)
    idx, w, _ = corner_indices(p01, tab, np.float32)
    n = p01.shape[0]
    g = np.asarray(dL_denc, dtype).reshape(n, tab.L, tab.F).transpose(1, 0, 2)  # [L, N, F]
    out = np.zeros((tab.n_params, tab.F), dtype)
    for c in range(8):
        np.add.at(out, idx[:, :, c].reshape(-1), (w[:, :, c, None].astype(dtype) * g).reshape(-1, tab.F))
    return out


def tv_rows(pos01: np.ndarray, tab: LevelTable, dtype=np.float32):
    """(corner-0 rows [L, N], neighbour rows [L, N, 6]) of the TV term (:236-242): the neighbours
    are floor(pos_scaled) + ADJACENT converted like the corners."""
    scales = np.asarray(tab.scales, dtype)
    ps = pos01[None] * scales[:, None, None] + dtype(0.5)
    fl = np.floor(ps)
    v0 = coords_u32(fl)
    va = coords_u32(fl[:, :, None, :] + ADJACENT[None, None].astype(fl.dtype))
    r0 = np.stack([grid_rows(v0[l], l, tab) for l in range(tab.L)])
    ra = np.stack([grid_rows(va[l], l, tab) for l in range(tab.L)])
    return r0, ra


def total_variation(pos, latents, bound, tab: LevelTable, tv_scale: float, dtype=np.float32):
    """encoders.py:236-254 (0 unless tv_scale > 0): tv_scale * (lat[neighbour] - lat[corner 0])^2
    summed over the six neighbours and the features, averaged over levels and points."""
    if tv_scale <= 0:
        return dtype(0)
    p01 = normalize(pos, bound, np.float32)
    r0, ra = tv_rows(p01, tab)
    lat = np.asarray(latents, dtype)
    d = lat[ra] - lat[r0][:, :, None, :]                       # [L, N, 6, F]
    return (dtype(tv_scale) * d * d).sum(axis=(-2, -1)).mean()


def total_variation_grad(pos, latents, bound, tab: LevelTable, tv_scale: float, dtype=np.float64):
    """d total_variation / d latents [P, F]: 2 s (lat[a] - lat[c0]) / (L N) added to each
    neighbour's row and subtracted from corner 0's."""
    p01 = normalize(pos, bound, np.float32)
    r0, ra = tv_rows(p01, tab)
    lat = np.asarray(latents, dtype)
    n = p01.shape[0]
    d = (lat[ra] - lat[r0][:, :, None, :]) * (2.0 * tv_scale / (tab.L * n))   # [L, N, 6, F]
    out = np.zeros((tab.n_params, tab.F), dtype)
    np.add.at(out, ra.reshape(-1), d.reshape(-1, tab.F))
    np.add.at(out, r0.reshape(-1), -d.sum(axis=2).reshape(-1, tab.F))
    return out
