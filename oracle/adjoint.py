"""FP64 forwards and central differences for the adjoint checks.  TEST INFRASTRUCTURE ONLY.

integrate_forward64 restates integrating.cu:24-104 of the reference (front-to-back compositing,
early stop once T <= 1e-4, colour and depth normalised by the opacity for a stopped ray, the
background blended in otherwise) in float64, vectorised over copies of one ray so that central
differences of every input of the ray take one pass.
"""
from __future__ import annotations

import numpy as np

T_THRESHOLD = 1e-4


def integrate_forward64(sigma, rgb, dt, z, bg):
    """sigma, dt, z [..., n]; rgb [..., n, 3]; bg [..., 3] (leading dims are copies of a ray).
    Returns (out [..., 4] = rgb + depth, opacity [...], n_used [...])."""
    sigma, dt, z = (np.asarray(a, np.float64) for a in (sigma, dt, z))
    rgb, bg = np.asarray(rgb, np.float64), np.asarray(bg, np.float64)
    lead = sigma.shape[:-1]
    n = sigma.shape[-1]
    T = np.ones(lead)
    acc = np.zeros(lead + (4,))
    used = np.zeros(lead, np.int64)
    for k in range(n):
        live = T > T_THRESHOLD
        a = 1.0 - np.exp(-sigma[..., k] * dt[..., k])
        w = np.where(live, T * a, 0.0)
        acc[..., :3] += w[..., None] * rgb[..., k, :]
        acc[..., 3] += w * z[..., k]
        T = np.where(live, T * (1.0 - a), T)
        used += live
    op = 1.0 - T
    stopped = T <= T_THRESHOLD
    out = acc.copy()
    out[..., :3] = np.where(stopped[..., None], acc[..., :3] / np.maximum(op, 1e-300)[..., None],
                            acc[..., :3] + T[..., None] * bg)
    out[..., 3] = np.where(stopped, acc[..., 3] / np.maximum(op, 1e-300), acc[..., 3])
    return out, op, used


def ray_fd64(sigma, rgb, dt, z, bg, g, h=1e-6):
    """Central differences of L = g . out for one ray.  Returns (dL/dsigma [n], dL/drgb [n, 3],
    dL/dz [n], dL/dbg [3])."""
    n = len(sigma)
    base = dict(sigma=np.asarray(sigma, np.float64), rgb=np.asarray(rgb, np.float64),
                dt=np.asarray(dt, np.float64), z=np.asarray(z, np.float64), bg=np.asarray(bg, np.float64))
    g = np.asarray(g, np.float64)

    def batch(name, count, perturb):
        cp = {k: np.broadcast_to(v, (2 * count,) + v.shape).copy() for k, v in base.items()}
        for j in range(count):
            perturb(cp[name], j, 2 * j, +h)
            perturb(cp[name], j, 2 * j + 1, -h)
        out, _, _ = integrate_forward64(cp["sigma"], cp["rgb"], cp["dt"], cp["z"], cp["bg"])
        L = out @ g
        return (L[0::2] - L[1::2]) / (2 * h)

    def at_sample(arr, j, row, d):
        arr[row, j] += d

    d_sigma = batch("sigma", n, at_sample)
    d_z = batch("z", n, at_sample)
    d_rgb = np.stack([batch("rgb", n, lambda arr, j, row, d, c=c: arr.__setitem__((row, j, c), arr[row, j, c] + d))
                      for c in range(3)], 1)
    d_bg = batch("bg", 3, lambda arr, j, row, d: arr.__setitem__((row, j), arr[row, j] + d))
    return d_sigma, d_rgb, d_z, d_bg


def ray_adjoint64(sigma, rgb, dt, z, bg, g):
    """The exact adjoint written out (the formula ngp_integrate_rays_backward_exact evaluates), in
    float64: with norm = 1 for a ray reaching the background and its opacity for a stopped ray,
    dL/dsigma_k = dt_k sum_c g_c (T_{k+1} x_kc - (out_c - cur_kc)) / norm, dL/dx_kc = w_k g_c / norm
    (x = rgb, or z for the depth channel), dL/dbg = T_N g[:3] (not stopped) or 0."""
    out, op, used = integrate_forward64(sigma, rgb, dt, z, bg)
    n = len(sigma)
    T = 1.0
    cur = np.zeros(4)
    stopped = (1.0 - op) <= T_THRESHOLD
    norm = op if stopped else 1.0
    gs = np.zeros(n)
    grgb = np.zeros((n, 3))
    gz = np.zeros(n)
    for k in range(int(used)):
        a = 1.0 - np.exp(-sigma[k] * dt[k])
        w = T * a
        x = np.concatenate([rgb[k], [z[k]]])
        cur += w * x
        T *= 1.0 - a
        gs[k] = dt[k] * (g @ (T * x - (out - cur))) / norm
        grgb[k] = w * g[:3] / norm
        gz[k] = w * g[3] / norm
    gbg = (1.0 - op) * g[:3] if not stopped else np.zeros(3)
    return gs, grgb, gz, gbg
