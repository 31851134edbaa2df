"""HashGridEncoder on the GPU kernels, with the interface of the reference's flax module.

Mirrors ``HashGridEncoder`` of models/encoders.py:58-256: fields (L, T, F, N_min, N_max,
tv_scale, param_dtype), the parameter named "latent codes stored on grid vertices" of shape
[offsets[-1], F] initialised ~U(-1e-4, 1e-4) (encoders.py:105-114), and
``__call__(pos, bound) -> (encodings [N, L*F], tv)``.  The gradient w.r.t. the table is the
scatter-add of the gather's transpose; positions get no gradient (the reference never
differentiates w.r.t. sample positions: they come from march_rays, which has no JVP).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional

import torch

from . import _lib as L
from . import precision as P

PARAM_NAME = "latent codes stored on grid vertices"


@dataclass(frozen=True)
class LevelTable:
    """encoders.py:77-103, computed on the host in float64 as the reference does."""
    L: int
    T: int
    F: int
    N_min: int
    N_max: int
    per_level_scale: Optional[float] = None
    dim: int = 3

    @property
    def b(self) -> float:
        if self.per_level_scale is not None:
            return float(self.per_level_scale)
        return math.exp((math.log(self.N_max) - math.log(self.N_min)) / (self.L - 1))

    def levels(self):
        scales: List[float] = []
        res: List[int] = []
        offsets = [0]
        first_hash = 0
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
            offsets.append(offsets[-1] + n)
        return scales, res, offsets, first_hash

    @property
    def n_params(self) -> int:
        return self.levels()[2][-1]

    def descriptor(self, n_coords: int, bound: float, accumulate: bool = False) -> L.NgpHashGridDescriptor:
        if self.L > L.MAX_LEVELS:
            raise ValueError(f"at most {L.MAX_LEVELS} levels are supported")
        if self.F != 2:
            raise NotImplementedError("the GPU encoder supports F = 2 features per level")
        scales, res, offsets, first_hash = self.levels()
        if offsets[-1] >= 2 ** 32:
            raise ValueError("table too large for 32-bit indices")
        d = L.NgpHashGridDescriptor()
        d.n_coords = n_coords
        d.L, d.F, d.T = self.L, self.F, self.T
        d.first_hash_level = first_hash
        d.n_params = offsets[-1]
        d.bound = bound
        d.two_bound = 2 * bound
        d.accumulate = 1 if accumulate else 0
        for i in range(self.L):
            d.scales[i] = scales[i]           # float64 -> float32, as jnp.asarray(scales, float32)
            d.resolutions[i] = res[i] & 0xFFFFFFFF
        for i in range(self.L + 1):
            d.offsets[i] = offsets[i]
        return d


def mixed_descriptor(desc: L.NgpHashGridDescriptor, table: int, encodings: int) -> L.NgpHashGridMixedDescriptor:
    m = L.NgpHashGridMixedDescriptor()
    m.grid, m.table, m.encodings = desc, table, encodings
    return m


def forward_call(desc: L.NgpHashGridDescriptor, latents: torch.Tensor, out: torch.Tensor):
    """(entry point, descriptor) of the encoder forward for these storage types."""
    if latents.dtype == torch.float32 and out.dtype == torch.float32:
        return "ngp_hashgrid_forward", desc
    return "ngp_hashgrid_forward_mixed", mixed_descriptor(desc, P.dtype_code(latents), P.dtype_code(out))


def backward_call(desc: L.NgpHashGridDescriptor, dL_denc: torch.Tensor):
    """(entry point, descriptor) of the encoder backward for this gradient type."""
    if dL_denc.dtype == torch.float32:
        return "ngp_hashgrid_backward", desc
    return "ngp_hashgrid_backward_mixed", mixed_descriptor(desc, L.DTYPE_F32, P.dtype_code(dL_denc))


def hashgrid_forward(table: LevelTable, pos: torch.Tensor, latents: torch.Tensor, bound: float,
                     count: Optional[torch.Tensor] = None, out: Optional[torch.Tensor] = None,
                     enc_dtype: torch.dtype = torch.float32) -> torch.Tensor:
    """Encodings of `pos`.  A 16-bit `latents` (a working copy of the FP32 table) and/or 16-bit
    encodings go through ngp_hashgrid_forward_mixed."""
    pos = pos.contiguous()
    n = pos.shape[0]
    if out is None:
        out = torch.empty(n, table.L * table.F, dtype=enc_dtype, device=pos.device)
    desc = table.descriptor(n, bound)
    if latents.dtype == torch.float32 and out.dtype == torch.float32:
        L.call("ngp_hashgrid_forward", [pos, latents, count, out], desc)
    else:
        L.call("ngp_hashgrid_forward_mixed", [pos, latents, count, out],
               mixed_descriptor(desc, P.dtype_code(latents), P.dtype_code(out)))
    return out


def hashgrid_backward(table: LevelTable, pos: torch.Tensor, dL_denc: torch.Tensor, bound: float,
                      count: Optional[torch.Tensor] = None, out: Optional[torch.Tensor] = None,
                      accumulate: bool = False) -> torch.Tensor:
    """FP32 dL/dlatents from FP32 or 16-bit dL/dencodings."""
    n = pos.shape[0]
    if out is None:
        out = torch.empty(table.n_params, table.F, dtype=torch.float32, device=pos.device)
    desc = table.descriptor(n, bound, accumulate)
    if dL_denc.dtype == torch.float32:
        L.call("ngp_hashgrid_backward", [pos.contiguous(), dL_denc.contiguous(), count, out], desc)
    else:
        L.call("ngp_hashgrid_backward_mixed", [pos.contiguous(), dL_denc.contiguous(), count, out],
               mixed_descriptor(desc, L.DTYPE_F32, P.dtype_code(dL_denc)))
    return out


def hashgrid_tv(table: LevelTable, pos: torch.Tensor, latents: torch.Tensor, bound: float, tv_scale: float,
                grad: Optional[torch.Tensor] = None, grad_scale: Optional[torch.Tensor] = None,
                out: Optional[torch.Tensor] = None, scratch: Optional[torch.Tensor] = None) -> torch.Tensor:
    """The TV term of encoders.py:236-254 as a device f32[1] (0 when tv_scale <= 0).  With `grad`
    ([P, F] FP32), d tv / d latents -- times the device scalar `grad_scale` when given -- is added
    into it."""
    pos = pos.contiguous()
    if out is None:
        out = torch.empty(1, dtype=torch.float32, device=pos.device)
    if scratch is None:
        scratch = torch.empty(1, dtype=torch.float64, device=pos.device)
    desc = L.NgpHashGridTVDescriptor(table.descriptor(pos.shape[0], bound), float(tv_scale), int(grad is not None))
    L.call("ngp_hashgrid_tv", [pos, latents, grad_scale, out, grad, scratch], desc)
    return out


class _HashGridTVFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, latents, table, bound, tv_scale):
        ctx.table, ctx.bound, ctx.tv_scale = table, bound, tv_scale
        ctx.save_for_backward(pos, latents)
        return hashgrid_tv(table, pos, latents, bound, tv_scale)[0]

    @staticmethod
    def backward(ctx, g):
        pos, latents = ctx.saved_tensors
        grad = torch.zeros_like(latents)
        g1 = g.reshape(1).to(torch.float32).contiguous()   # the upstream scalar stays on the device
        hashgrid_tv(ctx.table, pos, latents, ctx.bound, ctx.tv_scale, grad=grad, grad_scale=g1)
        return None, grad, None, None, None


class _HashGridFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, latents, table, bound):
        ctx.table, ctx.bound = table, bound
        ctx.save_for_backward(pos)
        return hashgrid_forward(table, pos, latents, bound)

    @staticmethod
    def backward(ctx, g):
        (pos,) = ctx.saved_tensors
        return None, hashgrid_backward(ctx.table, pos, g.contiguous(), ctx.bound), None, None


class HashGridEncoder(torch.nn.Module):
    """models/encoders.py:58-256 on libngp_gb300."""

    def __init__(self, L: int, T: int, F: int, N_min: int, N_max: int, tv_scale: float = 0.0,
                 param_dtype: torch.dtype = torch.float32, per_level_scale: Optional[float] = None,
                 device="cuda", generator: Optional[torch.Generator] = None):
        super().__init__()
        if param_dtype != torch.float32:
            raise NotImplementedError("the FP32 encoder stores float32 latents")
        self.table = LevelTable(L, T, F, N_min, N_max, per_level_scale)
        self.L, self.T, self.F, self.N_min, self.N_max = L, T, F, N_min, N_max
        self.tv_scale = tv_scale
        lat = torch.empty(self.table.n_params, F, dtype=torch.float32, device=device)
        lat.uniform_(-1e-4, 1e-4, generator=generator)
        self.register_parameter(PARAM_NAME, torch.nn.Parameter(lat))

    @property
    def latents(self) -> torch.nn.Parameter:
        return getattr(self, PARAM_NAME)

    @property
    def b(self) -> float:
        return self.table.b

    def forward(self, pos: torch.Tensor, bound: float):
        """(encodings [N, L*F], tv): tv is a differentiable device scalar when tv_scale > 0, else 0
        (encoders.py:236-256)."""
        if pos.dtype != torch.float32 or pos.dim() != 2 or pos.shape[-1] != 3:
            raise ValueError("pos must be float32 [N, 3]")
        enc = _HashGridFn.apply(pos, self.latents, self.table, float(bound))
        tv = _HashGridTVFn.apply(pos, self.latents, self.table, float(bound), float(self.tv_scale)) \
            if self.tv_scale > 0 else 0.0
        return enc, tv


def spherical_harmonics_encoding(coord: torch.Tensor, degree: int) -> torch.Tensor:
    """shjax.spherical_harmonics_encoding (deps/spherical-harmonics-encoding-jax/src/shjax/
    __init__.py:120-134): [n, 3] unit directions -> [n, degree^2] float32, the real spherical
    harmonics of degrees 0..degree-1 (degree in 1..8).  Like the reference's op it has no
    gradient: directions come from the ray batch, not from parameters."""
    if coord.dtype != torch.float32 or coord.dim() != 2 or coord.shape[-1] != 3:
        raise ValueError("coord must be float32 [n, 3]")
    if int(degree) < 0:
        raise ValueError("degree must be non-negative")
    coord = coord.contiguous()
    n = coord.shape[0]
    out = torch.empty(n, int(degree) ** 2, dtype=torch.float32, device=coord.device)
    L.call("spherical_harmonics_encoding_cuda_f32", [coord, out], L.SphericalHarmonicsEncodingDescriptor(n, int(degree)))
    return out


class SphericalHarmonicsEncoder(torch.nn.Module):
    """models/encoders.py:351-406 (SphericalHarmonicsEncoder and its shjax-backed twin): dirs
    [..., 3] unit vectors -> [..., L^2]."""

    def __init__(self, L: int):
        super().__init__()
        self.L = int(L)

    def forward(self, dirs: torch.Tensor) -> torch.Tensor:
        flat = dirs.reshape(-1, 3)
        return spherical_harmonics_encoding(flat, self.L).view(*dirs.shape[:-1], self.L * self.L)
