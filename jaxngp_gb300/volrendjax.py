"""Drop-in replacements for the public ops of volrendjax, on CUDA torch tensors.

Signatures, argument meaning, return tuples, broadcasting and shape/dtype checks follow
deps/volume-rendering-jax/src/volrendjax:

* ``packbits``                 packbits/__init__.py:8-28, packbits/abstract.py:7-38
* ``march_rays``               marching/__init__.py:8-93, marching/abstract.py:7-72
* ``march_rays_inference``     marching/__init__.py:96-157, marching/abstract.py:75-121
* ``morton3d(_invert)``        morton3d/__init__.py:6-10, morton3d/abstract.py:6-45
* ``integrate_rays``           integrating/__init__.py:11-59, with the custom VJP of
                               integrating/impl.py:50-146 as a torch.autograd.Function
* ``integrate_rays_inference`` integrating/__init__.py:62-110

JAX's uint32 arrays are int32 tensors here (same bits; every value on this path is < 2^31), and
the scalar results are 0-d device tensors, so nothing forces a host synchronisation.
Errors the reference reports through chex/NotImplementedError are raised as ValueError /
NotImplementedError before any kernel runs.
"""
from __future__ import annotations

from typing import Tuple

import torch

from . import _lib as L

u32 = torch.int32


def _as_u32(t: torch.Tensor) -> torch.Tensor:
    if t.dtype == torch.uint32:
        return t.view(torch.int32)
    if t.dtype != torch.int32:
        raise TypeError(f"expected a uint32 (int32) tensor, got {t.dtype}")
    return t


def _f32(t: torch.Tensor, name: str) -> torch.Tensor:
    if t.dtype != torch.float32:
        raise NotImplementedError(f"{name} is only implemented for float32 inputs, got {t.dtype}")
    return t.contiguous()


def _check_shape(t: torch.Tensor, shape, name: str):
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: expected shape {tuple(shape)}, got {tuple(t.shape)}")


# ------------------------------------------------------------------------------------ packbits

def packbits(density_threshold, density_grid: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
    """Pack `density_grid > density_threshold` into a uint8 bitfield (bit k of byte i is cell
    8i+k).  Returns (occ_mask bool [N], occ_bitfield uint8 [N//8])."""
    grid = _f32(density_grid, "packbits")
    if grid.dim() != 1:
        raise ValueError("packbits expects a rank-1 density grid")
    n_bits = grid.shape[0]
    if n_bits % 8 != 0:
        raise ValueError(f"pack_density_into_bits expects size of density grid to be divisible by 8, got {n_bits}")
    thr = torch.as_tensor(density_threshold, dtype=torch.float32, device=grid.device)
    mask = torch.empty(n_bits, dtype=torch.bool, device=grid.device)
    bits = torch.empty(n_bits // 8, dtype=torch.uint8, device=grid.device)
    desc = L.PackbitsDescriptor(n_bits // 8)
    if thr.numel() == 1:
        L.call("ngp_packbits_scalar", [thr.reshape(1).contiguous(), grid, mask, bits], desc)
    else:
        thr = torch.broadcast_to(thr, grid.shape).contiguous()
        L.call("pack_density_into_bits", [thr, grid, mask, bits], desc)
    return mask, bits


# ---------------------------------------------------------------------------------- marching

def march_rays(total_samples: int, diagonal_n_steps: int, K: int, G: int, bound: float,
               stepsize_portion: float, rays_o: torch.Tensor, rays_d: torch.Tensor,
               t_starts: torch.Tensor, t_ends: torch.Tensor, noises, occupancy_bitfield: torch.Tensor,
               return_counters: bool = False):
    """Generate samples along each ray, skipping empty space by the occupancy bitfield.

    Returns (measured_batch_size_before_compaction, ray_is_valid, rays_n_samples,
    rays_sample_startidx, idcs, xyzs, dirs, dss, z_vals), as marching/__init__.py:93.
    """
    rays_o, rays_d = _f32(rays_o, "march_rays"), _f32(rays_d, "march_rays")
    n_rays = rays_o.shape[0]
    _check_shape(rays_o, (n_rays, 3), "rays_o")
    _check_shape(rays_d, (n_rays, 3), "rays_d")
    t_starts, t_ends = _f32(t_starts, "t_starts"), _f32(t_ends, "t_ends")
    _check_shape(t_starts, (n_rays,), "t_starts")
    _check_shape(t_ends, (n_rays,), "t_ends")
    noises = torch.broadcast_to(torch.as_tensor(noises, dtype=torch.float32, device=rays_o.device), (n_rays,)).contiguous()
    if occupancy_bitfield.dtype != torch.uint8:
        raise TypeError("occupancy_bitfield must be uint8")
    _check_shape(occupancy_bitfield, (K * G * G * G // 8,), "occupancy_bitfield")
    for v, nm in [(total_samples, "total_samples"), (diagonal_n_steps, "diagonal_n_steps"), (K, "K"), (G, "G")]:
        if int(v) <= 0:
            raise ValueError(f"{nm} must be positive")
    if bound <= 0 or stepsize_portion < 0:
        raise ValueError("bound must be positive and stepsize_portion non-negative")
    dev = rays_o.device
    counters = torch.empty(2, dtype=u32, device=dev)
    valid = torch.empty(n_rays, dtype=torch.bool, device=dev)
    n_samples = torch.empty(n_rays, dtype=u32, device=dev)
    startidx = torch.empty(n_rays, dtype=u32, device=dev)
    idcs = torch.empty(total_samples, dtype=u32, device=dev)
    xyzs = torch.empty(total_samples, 3, dtype=torch.float32, device=dev)
    dirs = torch.empty(total_samples, 3, dtype=torch.float32, device=dev)
    dss = torch.empty(total_samples, dtype=torch.float32, device=dev)
    z_vals = torch.empty(total_samples, dtype=torch.float32, device=dev)
    desc = L.MarchingDescriptor(n_rays, total_samples, diagonal_n_steps, K, G, bound, stepsize_portion)
    L.call("march_rays", [rays_o, rays_d, t_starts, t_ends, noises, occupancy_bitfield.contiguous(),
                          counters[0:1], counters[1:2], valid, n_samples, startidx, idcs, xyzs, dirs, dss,
                          z_vals], desc)
    measured = counters[0] - counters[1]
    out = (measured, valid, n_samples, startidx, idcs, xyzs, dirs, dss, z_vals)
    return (out, counters) if return_counters else out


def march_rays_inference(diagonal_n_steps: int, K: int, G: int, march_steps_cap: int, bound: float,
                         stepsize_portion: float, rays_o: torch.Tensor, rays_d: torch.Tensor,
                         t_starts: torch.Tensor, t_ends: torch.Tensor, occupancy_bitfield: torch.Tensor,
                         next_ray_index_in: torch.Tensor, terminated: torch.Tensor, indices: torch.Tensor):
    """One refill-and-march iteration of the inference renderer.

    Returns (next_ray_index, indices, n_samples, t_starts, xyzs, dss, z_vals) where t_starts is the
    input with the advanced values scattered back (marching/__init__.py:156)."""
    rays_o, rays_d = _f32(rays_o, "march_rays_inference"), _f32(rays_d, "march_rays_inference")
    n_total = rays_o.shape[0]
    n_rays = terminated.shape[0]
    _check_shape(rays_d, (n_total, 3), "rays_d")
    _check_shape(t_starts, (n_total,), "t_starts")
    _check_shape(t_ends, (n_total,), "t_ends")
    _check_shape(occupancy_bitfield, (K * G * G * G // 8,), "occupancy_bitfield")
    _check_shape(next_ray_index_in, (1,), "next_ray_index_in")
    _check_shape(indices, (n_rays,), "indices")
    if terminated.dtype != torch.bool:
        raise TypeError("terminated must be bool")
    dev = rays_o.device
    cap = int(march_steps_cap)
    nri = torch.empty(1, dtype=u32, device=dev)
    idx_out = torch.empty(n_rays, dtype=u32, device=dev)
    n_samples = torch.empty(n_rays, dtype=u32, device=dev)
    t_out = torch.empty(n_rays, dtype=torch.float32, device=dev)
    xyzs = torch.empty(n_rays, cap, 3, dtype=torch.float32, device=dev)
    dss = torch.empty(n_rays, cap, dtype=torch.float32, device=dev)
    z_vals = torch.empty(n_rays, cap, dtype=torch.float32, device=dev)
    desc = L.MarchingInferenceDescriptor(n_total, n_rays, diagonal_n_steps, K, G, cap, bound, stepsize_portion)
    L.call("march_rays_inference", [rays_o, rays_d, _f32(t_starts, "t_starts"), _f32(t_ends, "t_ends"),
                                    occupancy_bitfield.contiguous(), _as_u32(next_ray_index_in).contiguous(),
                                    terminated.contiguous(), _as_u32(indices).contiguous(), nri, idx_out,
                                    n_samples, t_out, xyzs, dss, z_vals], desc)
    t_new = t_starts.clone()
    ok = idx_out < n_total
    t_new.index_put_((idx_out[ok].long(),), t_out[ok])
    return nri, idx_out, n_samples, t_new, xyzs, dss, z_vals


def morton3d(xyzs: torch.Tensor) -> torch.Tensor:
    """uint32 [N,3] grid coordinates -> uint32 [N] Morton codes."""
    xyzs = _as_u32(xyzs).contiguous()
    n = xyzs.shape[0]
    out = torch.empty(n, dtype=u32, device=xyzs.device)
    L.call("morton3d", [xyzs, out], L.Morton3DDescriptor(n))
    return out


def morton3d_invert(idcs: torch.Tensor) -> torch.Tensor:
    """uint32 [N] Morton codes -> uint32 [N,3] grid coordinates."""
    idcs = _as_u32(idcs).contiguous()
    n = idcs.shape[0]
    out = torch.empty(n, 3, dtype=u32, device=idcs.device)
    L.call("morton3d_invert", [idcs, out], L.Morton3DDescriptor(n))
    return out


# ------------------------------------------------------------------------------- integrating

def _integrate_forward(startidx, n_samples, bgs, dss, z_vals, drgbs):
    n = startidx.shape[0]
    s = dss.shape[0]
    dev = drgbs.device
    measured = torch.empty(1, dtype=u32, device=dev)
    rgbds = torch.empty(n, 4, dtype=torch.float32, device=dev)
    opac = torch.empty(n, dtype=torch.float32, device=dev)
    L.call("integrate_rays", [startidx, n_samples, bgs, dss, z_vals, drgbs, measured, rgbds, opac],
           L.IntegratingDescriptor(n, s))
    return measured, rgbds, opac


def integrate_rays_backward(near_distance: float, rays_sample_startidx, rays_n_samples, bgs, dss, z_vals, drgbs,
                            final_rgbds, final_opacities, dL_dfinal_rgbds, exact: bool = False):
    """The reference's backward kernel (integrating/impl.py:109-141), or with `exact` the exact
    adjoint of the forward (ngp_integrate_rays_backward_exact).  Returns
    (dL_dbgs [R,3], dL_dz_vals [S], dL_ddrgbs [S,4])."""
    startidx, n_samples = _as_u32(rays_sample_startidx).contiguous(), _as_u32(rays_n_samples).contiguous()
    n = startidx.shape[0]
    s = dss.shape[0]
    dev = drgbs.device
    bgs = torch.broadcast_to(bgs, (n, 3)).contiguous().float()
    g_bgs = torch.empty(n, 3, dtype=torch.float32, device=dev)
    g_z = torch.empty(s, dtype=torch.float32, device=dev)
    g_c = torch.empty(s, 4, dtype=torch.float32, device=dev)
    if near_distance < 0:
        raise ValueError("near_distance must be non-negative")
    L.call("ngp_integrate_rays_backward_exact" if exact else "integrate_rays_backward",
           [startidx, n_samples, bgs, dss.contiguous(), z_vals.contiguous(),
                                       drgbs.contiguous(), final_rgbds.contiguous(), final_opacities.contiguous(),
                                       dL_dfinal_rgbds.contiguous(), g_bgs, g_z, g_c],
           L.IntegratingBackwardDescriptor(n, s, near_distance))
    return g_bgs, g_z, g_c


class _IntegrateRays(torch.autograd.Function):
    """custom_vjp of integrating/impl.py:50-146: gradients for bgs, z_vals and drgbs; none for
    near_distance, the index arrays or dss (impl.py:126-141)."""

    @staticmethod
    def forward(ctx, near_distance, startidx, n_samples, bgs, dss, z_vals, drgbs, exact=False):
        measured, rgbds, opac = _integrate_forward(startidx, n_samples, bgs, dss, z_vals, drgbs)
        ctx.near_distance = float(near_distance)
        ctx.exact = bool(exact)
        ctx.save_for_backward(startidx, n_samples, bgs, dss, z_vals, drgbs, rgbds, opac)
        ctx.mark_non_differentiable(measured)
        return measured, rgbds, opac

    @staticmethod
    def backward(ctx, _g_measured, g_rgbds, _g_opac):
        startidx, n_samples, bgs, dss, z_vals, drgbs, rgbds, opac = ctx.saved_tensors
        if g_rgbds is None:
            g_rgbds = torch.zeros_like(rgbds)
        g_bgs, g_z, g_c = integrate_rays_backward(ctx.near_distance, startidx, n_samples, bgs, dss, z_vals, drgbs,
                                                  rgbds, opac, g_rgbds.contiguous(), exact=ctx.exact)
        return None, None, None, g_bgs, None, g_z, g_c, None


def integrate_rays(near_distance: float, rays_sample_startidx: torch.Tensor, rays_n_samples: torch.Tensor,
                   bgs: torch.Tensor, dss: torch.Tensor, z_vals: torch.Tensor, drgbs: torch.Tensor,
                   exact_adjoint: bool = False):
    """Front-to-back compositing with early termination at T <= 1e-4.

    Returns (measured_batch_size, final_rgbds [R,4], final_opacities [R]); differentiable w.r.t.
    bgs, z_vals and drgbs, through the reference's backward, or with `exact_adjoint` through the
    exact adjoint of the forward."""
    startidx, n_samples = _as_u32(rays_sample_startidx).contiguous(), _as_u32(rays_n_samples).contiguous()
    n = startidx.shape[0]
    s = dss.shape[0]
    _check_shape(n_samples, (n,), "rays_n_samples")
    _check_shape(z_vals, (s,), "z_vals")
    _check_shape(drgbs, (s, 4), "drgbs")
    _f32(drgbs, "integrate_rays")
    bgs = torch.broadcast_to(torch.as_tensor(bgs, dtype=torch.float32, device=drgbs.device), (n, 3)).contiguous()
    measured, rgbds, opac = _IntegrateRays.apply(near_distance, startidx, n_samples, bgs, dss.contiguous(),
                                                 z_vals.contiguous(), drgbs.contiguous(), exact_adjoint)
    return measured[0], rgbds, opac


def integrate_rays_inference(rays_bg: torch.Tensor, rays_rgbd: torch.Tensor, rays_T: torch.Tensor,
                             n_samples: torch.Tensor, indices: torch.Tensor, dss: torch.Tensor,
                             z_vals: torch.Tensor, drgbs: torch.Tensor):
    """Continue compositing the rays in flight.  Returns (terminate_cnt, terminated, rays_rgbd,
    rays_T) with the per-slot results scattered into the full arrays
    (integrating/__init__.py:108-110)."""
    n_total = rays_rgbd.shape[0]
    n_rays, cap = dss.shape
    _check_shape(rays_bg, (n_total, 3), "rays_bg")
    _check_shape(rays_T, (n_total,), "rays_T")
    _check_shape(z_vals, (n_rays, cap), "z_vals")
    _check_shape(drgbs, (n_rays, cap, 4), "drgbs")
    dev = drgbs.device
    cnt = torch.empty(1, dtype=u32, device=dev)
    term = torch.empty(n_rays, dtype=torch.bool, device=dev)
    rgbd_out = torch.empty(n_rays, 4, dtype=torch.float32, device=dev)
    T_out = torch.empty(n_rays, dtype=torch.float32, device=dev)
    indices = _as_u32(indices).contiguous()
    L.call("integrate_rays_inference", [rays_bg.contiguous(), rays_rgbd.contiguous(), rays_T.contiguous(),
                                        _as_u32(n_samples).contiguous(), indices, dss.contiguous(),
                                        z_vals.contiguous(), _f32(drgbs, "drgbs"), cnt, term, rgbd_out, T_out],
           L.IntegratingInferenceDescriptor(n_total, n_rays, cap))
    new_rgbd, new_T = rays_rgbd.clone(), rays_T.clone()
    ok = indices < n_total
    li = indices[ok].long()
    new_rgbd.index_put_((li,), rgbd_out[ok])
    new_T.index_put_((li,), T_out[ok])
    return cnt[0], term, new_rgbd, new_T


__all__ = ["integrate_rays", "integrate_rays_inference", "march_rays", "march_rays_inference", "morton3d",
           "morton3d_invert", "packbits"]
