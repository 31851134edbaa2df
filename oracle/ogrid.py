"""CPU restatement of the reference's occupancy-grid maintenance.  TEST INFRASTRUCTURE ONLY.

utils/types.py:1149-1225 (update_ogrid_density), :1227-1239 (threshold_ogrid), :1241-1362
(mark_untrained_density_grid) and :143-144 (mean_density_up_to_cascade), in float32 with the
reference's operation order.  Grids are flat [K * G^3] arrays in Morton order per cascade; cells
marked untrainable hold density -1 (their "alive" index set is the cells with density >= 0).
"""
from __future__ import annotations

import math

import numpy as np

from . import volrend as V

f32 = np.float32


def threshold_step(diagonal_n_steps: int, bound: float) -> float:
    """NeRFState.density_threshold_from_min_step_size (types.py:1367-1369)."""
    return 0.01 * diagonal_n_steps / (2 * min(bound, 1) * 3 ** 0.5)


def decay(density: np.ndarray, cas: int, G: int, factor: float = 0.95) -> np.ndarray:
    """types.py:1161-1162: the cascade's live cells times `factor`."""
    d = np.array(density, np.float32, copy=True)
    G3 = G ** 3
    sl = d[cas * G3:(cas + 1) * G3]
    alive = sl >= 0
    sl[alive] = sl[alive] * f32(factor)
    return d


def cell_points_base(cells: np.ndarray, cas: int, G: int, bound: float):
    """types.py:1195-1199 before the jitter: cell coordinates mapped to
    [-mip_bound + hcw, mip_bound - hcw]; returns (points [M,3], half cell width)."""
    xyz = V.morton3d_invert(np.asarray(cells, np.uint32)).astype(np.float32)
    xyz = xyz / f32(G - 1) * f32(2) - f32(1)
    mip_bound = min(bound, 2.0 ** cas)
    hcw = mip_bound / G
    xyz = xyz * f32(mip_bound - hcw)
    return xyz.astype(np.float32), float(f32(hcw))


def max_update(density: np.ndarray, cas: int, G: int, cells: np.ndarray, sigma: np.ndarray) -> np.ndarray:
    """types.py:1218-1220: density[cell] = max(density[cell], sigma) at the sampled cells.  For a
    cell drawn more than once, jnp's `.at[].set` keeps one of the candidate maxima (unspecified
    which); the largest one is kept here, as an order-independent max does."""
    d = np.array(density, np.float32, copy=True)
    G3 = G ** 3
    sl = d[cas * G3:(cas + 1) * G3]
    np.maximum.at(sl, np.asarray(cells, np.int64), np.asarray(sigma, np.float32))
    return d


def mean_density(density: np.ndarray, G: int) -> float:
    """mean_density_up_to_cascade(1) (types.py:143-144): mean over cascade 0's live cells."""
    d0 = np.asarray(density[:G ** 3], np.float64)
    return float(d0[d0 >= 0].mean())


def threshold(density: np.ndarray, G: int, diagonal_n_steps: int, bound: float) -> float:
    """threshold_ogrid (types.py:1227-1231): min(threshold step, mean live density of cascade 0)."""
    return min(threshold_step(diagonal_n_steps, bound), mean_density(density, G))


def mark_untrained(K: int, G: int, bound: float, transforms: np.ndarray, width: int, height: int, fx: float, fy: float,
                   cx: float, cy: float) -> np.ndarray:
    """types.py:1241-1336 for undistorted pinhole cameras: True for the cells that at least one
    camera sees (one of the cell's 8 corners in front of it and projected inside its image).
    `transforms`: [V, 12] camera-to-world, rotation rows then position."""
    G3 = G ** 3
    n = K * G3
    idx = np.arange(n, dtype=np.uint32)
    level, pos_idcs = idx // G3, idx % G3
    mip_bound = np.minimum(2.0 ** level, bound).astype(np.float32)
    cell_width = (f32(2) * mip_bound / f32(G)).astype(np.float32)
    xyz = V.morton3d_invert(pos_idcs).astype(np.float32)
    xyz /= f32(G)
    xyz -= f32(0.5)
    xyz *= (f32(2) * mip_bound)[:, None]
    offsets = np.array([[0, 0, 0], [0, 0, 1], [0, 1, 0], [0, 1, 1], [1, 0, 0], [1, 0, 1], [1, 1, 0], [1, 1, 1]],
                       np.float32)
    verts = xyz[:, None, :] + cell_width[:, None, None] * offsets[None]   # [n, 8, 3]
    alive = np.zeros(n, bool)
    wh = np.array([width, height], np.float32)
    for T in np.asarray(transforms, np.float32):
        R = T[:9].reshape(3, 3)
        t = T[9:12]
        p = verts - t
        # p_cam = (p[..., None, :] * R.T).sum(-1): component i = p0 R[0][i] + p1 R[1][i] + p2 R[2][i]
        p_cam = (p[..., 0:1] * R[0][None, None, :] + p[..., 1:2] * R[1][None, None, :]) + p[..., 2:3] * R[2][None, None, :]
        in_front = p_cam[..., 2] < 0
        u = p_cam[..., 0] / -p_cam[..., 2]
        v = p_cam[..., 1] / -p_cam[..., 2]
        uv = np.stack([u * f32(fx) + f32(cx), v * f32(fy) + f32(cy)], -1) / wh
        inside = ((uv >= 0) & (uv < 1)).all(-1)
        alive |= (in_front & inside).any(-1)
        if alive.all():
            break
    return alive
