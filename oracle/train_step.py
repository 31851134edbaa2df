"""CPU restatement of the plain NGP training step.  TEST INFRASTRUCTURE ONLY: it is the CPU
baseline that bench.py times beside the GPU path, and nothing in the product imports it.

The reference's training step (app/nerf/_utils.py:80-170, models/renderers/cuda.py:100-162) has
no CPU implementation: its volrendjax ops register GPU lowerings only
(deps/volume-rendering-jax/src/volrendjax/marching/impl.py:12-13), and JAX is not installed here.
This port composes the oracle's pieces in the reference's order:
    rays from pixel indices (_utils.py:97-115), near/far (renderers/cuda.py:56-97), jitter, random
    background, target blend (utils/data.py:443-465)         NumPy float32
    march_rays, integrate_rays(+backward)                    oracle/volrend_oracle.c (OpenMP)
    hash-grid encoder forward / scatter-add backward         oracle/hashgrid.py (NumPy float32)
    MLP forward / backward                                    oracle/field.py (NumPy float32)
    masked Huber loss (_utils.py:151-156)                     NumPy
    Adam + decayed weights (_utils.py:19-77)                  NumPy float32
    occupancy-grid refresh (utils/types.py:1149-1239)         NumPy + oracle packbits
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import field as Fd
from . import hashgrid as H
from . import volrend as V


@dataclass
class CpuScene:
    """Camera intrinsics, per-view camera-to-world [V, 12], and a colour lookup for pixels."""
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float
    transforms: np.ndarray
    bound: float
    near: float = 0.3


def rays_from_pixels(sc: CpuScene, perm: np.ndarray):
    n_pix = sc.width * sc.height
    view, pix = perm // n_pix, perm % n_pix
    x = (pix % sc.width).astype(np.float32)
    y = (pix // sc.width).astype(np.float32)
    d = np.stack([((x + np.float32(0.5)) - np.float32(sc.cx)) / np.float32(sc.fx),
                  -(((y + np.float32(0.5)) - np.float32(sc.cy)) / np.float32(sc.fy)),
                  -np.ones_like(x)], -1)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    T = sc.transforms[view]
    R = T[:, :9].reshape(-1, 3, 3)
    d_world = (d[:, None, :] * R).sum(-1).astype(np.float32)
    o = np.ascontiguousarray(T[:, 9:12], np.float32)
    return o, np.ascontiguousarray(d_world)


def near_far(bound: float, o: np.ndarray, d: np.ndarray):
    eps = np.float32(1e-15)
    d = np.where(np.signbit(d), np.minimum(d, -eps), np.maximum(d, eps)).astype(np.float32)
    t0 = (-np.float32(bound) - o) / d
    t1 = (np.float32(bound) - o) / d
    ts = np.maximum(np.float32(0), np.minimum(t0, t1).max(-1)).astype(np.float32)
    te = np.maximum(t0, t1).min(-1).astype(np.float32)
    return ts, te


class CpuTrainer:
    def __init__(self, sc: CpuScene, targets: np.ndarray, bitfield: np.ndarray, density: np.ndarray,
                 total_samples: int, n_rays: int, G: int = 128, dns: int = 1024, lr: float = 1e-2, seed: int = 0,
                 table: H.LevelTable | None = None):
        self.sc, self.targets = sc, targets
        self.S, self.R, self.G, self.dns, self.lr = total_samples, n_rays, G, dns, lr
        self.tab = table or H.LevelTable(16, 2 ** 19, 2, 16, int(2048 * sc.bound))
        rng = np.random.default_rng(seed)
        self.rng = rng
        self.lat = rng.uniform(-1e-4, 1e-4, size=(self.tab.n_params, 2)).astype(np.float32)
        self.w = Fd.init_weights(seed)
        self.m = {k: np.zeros_like(v) for k, v in self.w.items()}
        self.v = {k: np.zeros_like(v) for k, v in self.w.items()}
        self.m_lat, self.v_lat = np.zeros_like(self.lat), np.zeros_like(self.lat)
        self.bits, self.density = bitfield, density
        self.step_count = 1000  # steady-state cadence: partial occupancy-grid updates every 16 steps
        self.timing = {}

    def _t(self, name, t0):
        self.timing[name] = self.timing.get(name, 0.0) + time.perf_counter() - t0

    def sample_work(self, perm: np.ndarray):
        """Everything of one step that scales with the batch: rays -> loss -> gradients.
        Returns (n_valid_rays, samples used, dL/dlatents, dL/dW)."""
        sc, R, S = self.sc, self.R, self.S
        t = time.perf_counter()
        o, d = rays_from_pixels(sc, perm)
        t0, t1 = near_far(sc.bound, o, d)
        noise = self.rng.uniform(size=R).astype(np.float32)
        bg = self.rng.uniform(size=(R, 3)).astype(np.float32)
        rgba = self.targets[perm].astype(np.float32) / 255
        gt = rgba[:, :3] * rgba[:, 3:] + bg * (1 - rgba[:, 3:])
        self._t("rays", t)
        t = time.perf_counter()
        # the reference's kernel run one thread at a time in ray order (the training march's
        # schedule): the rays before the budget filled keep their results, later rays are dropped
        m, valid, ns, st, idcs, xyzs, dirs, dss, zs = V.march_rays(S, self.dns, 1, self.G, sc.bound, 0.0, o, d, t0, t1,
                                                                   noise, self.bits, early_exit=True)
        used = int(m)
        self._t("march", t)
        t = time.perf_counter()
        enc = H.encode(xyzs[:used], self.lat, sc.bound, self.tab)
        drgb_u, cache = Fd.forward(enc, dirs[:used], self.w, dtype=np.float32)
        drgbs = np.zeros((S, 4), np.float32)
        drgbs[:used] = drgb_u
        self._t("field_fwd", t)
        t = time.perf_counter()
        _, rgbd, opac = V.integrate_rays(sc.near, st, ns, bg, dss, zs, drgbs)
        e = rgbd[:, :3] - gt
        ae = np.abs(e)
        delta = np.float32(0.1)
        g = np.where(ae <= delta, e, delta * np.sign(e)) / np.float32(3)
        nv = max(int(valid.sum()), 1)
        g = np.where(valid[:, None], g, 0).astype(np.float32) / np.float32(nv)
        g4 = np.concatenate([g, np.zeros((R, 1), np.float32)], -1)
        _, _, g_drgbs = V.integrate_rays_backward(sc.near, st, ns, bg, dss, zs, drgbs, rgbd, opac, g4)
        self._t("integrate", t)
        t = time.perf_counter()
        denc, gw = Fd.backward(g_drgbs[:used], cache, self.w, dtype=np.float32)
        self._t("field_bwd", t)
        t = time.perf_counter()
        glat = H.encode_backward(xyzs[:used], denc, sc.bound, self.tab, dtype=np.float32)
        self._t("table_bwd", t)
        return int(valid.sum()), used, glat, gw

    def adam(self, glat, gw):
        """Dense Adam over every parameter (optax updates all entries every step)."""
        t = time.perf_counter()
        c = self.step_count + 1
        b1, b2 = np.float32(0.9), np.float32(0.99)
        bc1, bc2 = np.float32(1 - 0.9 ** c), np.float32(1 - 0.99 ** c)
        lr = np.float32(self.lr)

        def upd(p, g, m, v, wd):
            m *= b1
            m += (1 - b1) * g
            v *= b2
            v += (1 - b2) * g * g
            u = -lr * (m / bc1) / (np.sqrt(v / bc2 + np.float32(1e-15)) + np.float32(1e-15))
            if wd:
                u += np.float32(wd) * p
            p += u
        upd(self.lat, glat, self.m_lat, self.v_lat, 0.0)
        for k in self.w:
            upd(self.w[k], gw[k], self.m[k], self.v[k], 1e-6)
        self.step_count += 1
        self._t("adam", t)

    def update_ogrid(self):
        """types.py:1149-1239 for one cascade without update_all: decay, half uniform cells and
        half occupied cells, jittered point per cell, density query, max, threshold, packbits."""
        t = time.perf_counter()
        G, G3 = self.G, self.G ** 3
        alive = self.density >= 0
        self.density[alive] *= np.float32(0.95)
        M = max(1, int(alive.sum()) // 2)
        alive_idx = np.nonzero(alive)[0]
        occ_idx = np.nonzero(alive & np.unpackbits(self.bits, bitorder="little").astype(bool))[0]
        cells = np.concatenate([self.rng.choice(alive_idx, M // 2),
                                self.rng.choice(occ_idx if len(occ_idx) else alive_idx, M // 2)]).astype(np.uint32)
        xyz = V.morton3d_invert(cells).astype(np.float32)
        xyz = xyz / np.float32(G - 1) * 2 - 1
        mb = min(self.sc.bound, 1.0)
        hcw = mb / G
        xyz = xyz * np.float32(mb - hcw) + self.rng.uniform(-hcw, hcw, xyz.shape).astype(np.float32)
        sig = np.empty(len(cells), np.float32)
        for s in range(0, len(cells), 1 << 18):
            enc = H.encode(xyz[s:s + (1 << 18)], self.lat, self.sc.bound, self.tab)
            sig[s:s + (1 << 18)] = Fd.density_only(enc, self.w)
        np.maximum.at(self.density, cells, sig)
        mean = self.density[self.density >= 0].mean()
        thr = min(0.01 * self.dns / (2 * min(self.sc.bound, 1) * math.sqrt(3)), float(mean))
        _, self.bits = V.packbits(np.float32(thr), self.density)
        self._t("ogrid", t)


def analytic_occupancy(density_fn, G: int, bound: float, dns: int = 1024):
    """Occupancy grid from a known density field (cell centres, K = 1), thresholded as
    threshold_ogrid does: min(0.01 * diag / (2 min(bound,1) sqrt3), mean density)."""
    idx = np.arange(G ** 3, dtype=np.uint32)
    xyz = V.morton3d_invert(idx).astype(np.float64)
    centres = ((xyz + 0.5) / G - 0.5) * 2 * min(bound, 1.0)
    dens = np.empty(G ** 3, np.float32)
    for s in range(0, G ** 3, 1 << 18):
        dens[s:s + (1 << 18)] = density_fn(centres[s:s + (1 << 18)])
    thr = min(0.01 * dns / (2 * min(bound, 1) * math.sqrt(3)), float(dens.mean()))
    _, bits = V.packbits(np.float32(thr), dens)
    return dens, bits
