"""Learned proposal sampler: a small density network places each ray's samples instead of the
occupancy-grid march.  No reference counterpart (the reference marches the occupancy grid,
models/renderers/cuda.py:100-162); the kernels are ngp_proposal_* in include/ngp_gb300.h.

Per training step:
  rays      -> ngp_proposal_rays: coarse-block DDA (occupied interval, or an empty valid ray) and
               samples_per_ray (48 by default) sample slots per fitting ray
  bins      -> ngp_proposal_bin_points, the proposal field (4-level hash grid + MLP) at the bin
               centres, ngp_proposal_sample: inverse-CDF samples in march_rays' layout
  field     -> unchanged (encoder, MLP, fused integrator/loss, backwards, Adam)
  proposal  -> regresses the field's log density at the field's samples and at points drawn in
               occupied cells (ngp_proposal_loss), its own backward and Adam

Every k-th training step (TrainConfig.march_every, 8 by default) marches the occupancy grid instead
-- the sampler's fallback for whole steps: its evenly spread samples train the field's empty
space, which the proposal's concentrated samples rarely visit, and teach the proposal where its
density is wrong.  Without it the field keeps density that the occupancy-grid renderer, against
which the proposal's PSNR is measured, then shows.  Per ray (TrainConfig.proposal_fallback), rays on which the proposal misses more than 1% of
the transmittance the occupancy grid implies are marched within the step (sample()).

Everything stays on the device; the sample count of a step is read by the kernels from `counts`.
"""
from __future__ import annotations

from typing import Callable, Optional

import math

import torch

from . import _lib as L
from .encoders import LevelTable

BINS = 64
SAMPLES = 48
WEIGHTS = 4672
SHAPES = (("P0", (8, 64)), ("P1", (64, 64)), ("P2", (64, 1)))


def proposal_table() -> LevelTable:
    """4 levels of 2^16 rows, resolutions 16, 32, 64, 128."""
    return LevelTable(4, 1 << 16, 2, 16, 128)


class ProposalSampler:
    def __init__(self, n_rays: int, total_samples: int, G: int, bound: float, device="cuda", seed: int = 0,
                 lr: float = 1e-2, distill_points: int = 1 << 14, samples_per_ray: int = SAMPLES, mix: float = 0.1,
                 inference_only: bool = False):
        if G % 8 != 0:
            raise ValueError("the proposal sampler needs an occupancy grid resolution divisible by 8")
        self.R, self.S, self.G, self.bound = n_rays, total_samples, G, float(bound)
        self.spr = int(samples_per_ray)
        if not 1 <= self.spr <= 1024:
            raise ValueError("samples_per_ray must be in [1, 1024]")
        self.slots = total_samples // self.spr
        self.mix = float(mix)
        self.f16 = True   # bins through the FP16 tensor-core MLP
        self.dev = torch.device(device)
        self.table = proposal_table()
        self.lr = lr
        self.M = distill_points
        g = torch.Generator(device=self.dev)
        g.manual_seed(seed + 7919)
        f32 = dict(dtype=torch.float32, device=self.dev)
        i32 = dict(dtype=torch.int32, device=self.dev)
        P = self.table.n_params
        self.latents = torch.empty(P, 2, **f32).uniform_(-1e-4, 1e-4, generator=g)
        ws = []
        for _, (a, b) in SHAPES:
            lim = math.sqrt(6.0 / (a + b))
            ws.append(torch.empty(a * b, **f32).uniform_(-lim, lim, generator=g))
        self.weights = torch.cat(ws).contiguous()
        self.g_lat, self.g_w = torch.zeros_like(self.latents), torch.zeros_like(self.weights)
        self.m_lat, self.v_lat = torch.zeros_like(self.latents), torch.zeros_like(self.latents)
        self.m_w, self.v_w = torch.zeros_like(self.weights), torch.zeros_like(self.weights)
        Gc = G // 8
        self.coarse = torch.zeros(Gc ** 3, dtype=torch.uint8, device=self.dev)
        self.counters = torch.zeros(2, **i32)
        self.counts = torch.zeros(3, **i32)
        # per-ray fallback to the occupancy-grid march: flagged slots, the list of their rays, and
        # the sample counters the marched rays and then the proposal's rays allocate from
        self.slot_flag = torch.zeros(self.slots, dtype=torch.uint8, device=self.dev)
        self.fb_rays = torch.zeros(n_rays, **i32)
        self.fb_count = torch.zeros(1, **i32)
        self.fb_total = torch.zeros(1, **i32)
        self.alloc = torch.zeros(2, **i32)
        self.queue = torch.zeros(1, **i32)
        self.sample_calls = 0
        self.ray_of_slot = torch.zeros(self.slots, **i32)
        self.slot_ta, self.slot_tb = torch.zeros(self.slots, **f32), torch.zeros(self.slots, **f32)
        nb = self.slots * BINS
        self.points = torch.zeros(nb, 3, **f32)
        self.enc_b = torch.zeros(nb, 8, **f32)
        self.x_b = torch.zeros(nb, **f32)
        n_train = 1 if inference_only else max(self.S, self.M)   # sampling only: no training buffers
        self.enc_t = torch.zeros(n_train, 8, **f32)
        self.x_t = torch.zeros(n_train, **f32)
        self.g_x = torch.zeros(n_train, **f32)
        self.g_enc = torch.zeros(n_train, 8, **f32)
        self.loss = torch.zeros(2, **f32)
        self.scratch = torch.empty(L.proposal_backward_scratch_floats(), **f32)
        self.cells = torch.zeros(self.M, **i32)
        self.xyz_d = torch.zeros(self.M, 3, **f32)
        self.sigma_d = torch.zeros(self.M, **f32)
        self.steps = 0

    def _desc(self, n=0, perturb=False, seed=0, count_index=3, sigma_stride=1) -> L.NgpProposalDescriptor:
        return L.NgpProposalDescriptor(n, self.S, self.G, self.bound, int(perturb), seed & 0xFFFFFFFF,
                                       (seed >> 32) & 0xFFFFFFFF, count_index, sigma_stride, self.spr, self.mix)

    # ----------------------------------------------------------------------------- sampling
    def refresh(self, bitfield: torch.Tensor):
        """Coarse occupancy blocks from the (cascade-0) occupancy bitfield."""
        L.call("ngp_proposal_coarse", [bitfield, self.coarse], self._desc())

    def network(self, points: torch.Tensor, enc: torch.Tensor, x: torch.Tensor, count: Optional[torch.Tensor],
                f16: bool = False):
        """Log density at `points`: FP32, or FP16 tensor cores (FP16 operands, FP32 accumulation).
        The sampler's bins and, with `f16` set on the sampler, the training forward use the FP16
        form; the training backward recomputes its own FP32 activations either way, so FP16 only
        rounds the loss's x (relative error ~1e-3 against a regression residual far larger)."""
        n = points.shape[0]
        L.call("ngp_hashgrid_forward", [points, self.latents, count, enc], self.table.descriptor(n, self.bound))
        L.call("ngp_proposal_mlp_forward_f16" if f16 else "ngp_proposal_mlp_forward", [enc, self.weights, count, x],
               L.NgpMlpDescriptor(n, 0))

    def sample(self, rays_o, rays_d, t0, t1, valid, n_samples, startidx, idcs, xyzs, dirs, dss, z_vals,
               perturb: bool, seed: int, fallback=None) -> torch.Tensor:
        """Fills the march_rays-layout sample buffers; returns the device count of samples (u32[1]).

        `fallback` = (occupancy bitfield, density threshold f32[1], noises f32[R], MarchingDescriptor)
        turns on the per-ray fallback: rays on which the proposal misses more than 1% of the
        transmittance the occupancy grid implies (ngp_proposal_judge) are marched instead
        (ngp_march_rays_fallback, first, so they find room in the budget), and the other rays take
        their proposal samples after them (ngp_proposal_sample_alloc)."""
        n = rays_o.shape[0]
        self.sample_calls += 1
        L.call("ngp_proposal_rays", [rays_o, rays_d, t0, t1, self.coarse, self.counters[0:1], self.counters[1:2], valid,
                                     n_samples, startidx, self.ray_of_slot, self.slot_ta, self.slot_tb, self.counts],
               self._desc(n))
        L.call("ngp_proposal_bin_points", [self.counts, rays_o, rays_d, self.ray_of_slot, self.slot_ta, self.slot_tb,
                                           self.points], self._desc())
        self.network(self.points, self.enc_b, self.x_b, self.counts[1:2], f16=self.f16)
        if fallback is None:
            L.call("ngp_proposal_sample", [self.counts, rays_o, rays_d, self.ray_of_slot, self.slot_ta, self.slot_tb,
                                           self.x_b, idcs, xyzs, dirs, dss, z_vals], self._desc(perturb=perturb, seed=seed))
            return self.counts[2:3]
        bits, threshold, noises, d_march = fallback
        L.call("ngp_proposal_judge", [self.counts, rays_o, rays_d, self.ray_of_slot, self.slot_ta, self.slot_tb, self.x_b,
                                      bits, threshold, self.slot_flag, self.fb_rays, self.fb_count, self.fb_total],
               self._desc(n))
        self.alloc.zero_()
        L.call("ngp_march_rays_fallback", [rays_o, rays_d, t0, t1, noises, bits, self.alloc[0:1], self.alloc[1:2], valid,
                                           n_samples, startidx, idcs, xyzs, dirs, dss, z_vals, self.queue, self.fb_rays,
                                           self.fb_count], d_march)
        L.call("ngp_proposal_sample_alloc", [self.counts, rays_o, rays_d, self.ray_of_slot, self.slot_ta, self.slot_tb,
                                             self.x_b, self.slot_flag, self.alloc[0:1], self.alloc[1:2], idcs, xyzs, dirs,
                                             dss, z_vals, valid, n_samples, startidx],
               self._desc(perturb=perturb, seed=seed))
        return self.counts[2:3]

    def for_rendering(self, n_rays: int) -> "ProposalSampler":
        """A sampler for inference that shares this one's proposal field (table, weights) and
        coarse blocks, with a slot for every one of `n_rays` rays per call."""
        r = ProposalSampler(n_rays, n_rays * self.spr, self.G, self.bound, self.dev, samples_per_ray=self.spr,
                            mix=self.mix, inference_only=True)
        r.latents, r.weights, r.coarse, r.f16 = self.latents, self.weights, self.coarse, self.f16
        return r

    def fallback_rate(self) -> float:
        """Mean fallback rays per sampling call so far (reads the device counter)."""
        return float(self.fb_total.item()) / max(self.sample_calls, 1)

    # ----------------------------------------------------------------------------- training
    def train(self, xyzs: torch.Tensor, drgbs: torch.Tensor, distill: Optional[Callable] = None, lr: Optional[float] = None,
              count: Optional[torch.Tensor] = None, max_points: Optional[int] = None):
        """One proposal update from the field's densities at a step's samples (drgbs[:, 0]; the
        first `count` of them, by default this sampler's own, at most `max_points` -- samples sit
        in allocation order, so the first ones are a spread of rays), plus, when
        `distill(xyz, sigma)` is given, at points drawn in occupied cells."""
        S = xyzs.shape[0] if max_points is None else min(xyzs.shape[0], max_points)
        cnt = self.counts[2:3] if count is None else count
        xyzs = xyzs[:S]   # the forward evaluates only the points the update regresses on
        self.loss.zero_()
        self.network(xyzs, self.enc_t[:S], self.x_t[:S], cnt, f16=self.f16)
        L.call("ngp_proposal_loss", [cnt, self.x_t[:S], drgbs, self.g_x[:S], self.loss[0:1]],
               self._desc(S, count_index=0, sigma_stride=4))
        L.call("ngp_proposal_mlp_backward", [self.enc_t[:S], self.weights, self.g_x[:S], cnt, self.scratch,
                                             self.g_enc[:S], self.g_w], L.NgpMlpDescriptor(S, 0))
        L.call("ngp_hashgrid_backward", [xyzs, self.g_enc[:S], cnt, self.g_lat], self.table.descriptor(S, self.bound))
        if distill is not None:
            M = self.M
            distill(self.xyz_d, self.sigma_d)
            self.network(self.xyz_d, self.enc_t[:M], self.x_t[:M], None, f16=self.f16)
            L.call("ngp_proposal_loss", [None, self.x_t[:M], self.sigma_d, self.g_x[:M], self.loss[1:2]],
                   self._desc(M, count_index=3, sigma_stride=1))
            L.call("ngp_proposal_mlp_backward", [self.enc_t[:M], self.weights, self.g_x[:M], None, self.scratch,
                                                 self.g_enc[:M], self.g_w], L.NgpMlpDescriptor(M, 1))
            L.call("ngp_hashgrid_backward", [self.xyz_d, self.g_enc[:M], None, self.g_lat],
                   self.table.descriptor(M, self.bound, accumulate=True))
        self.steps += 1
        lr = self.lr if lr is None else lr
        L.call("ngp_adam", [self.latents, self.g_lat, self.m_lat, self.v_lat],
               L.NgpAdamDescriptor(self.latents.numel(), self.steps, lr, 0.9, 0.99, 1e-15, 1e-15, 0.0, 1))
        L.call("ngp_adam", [self.weights, self.g_w, self.m_w, self.v_w],
               L.NgpAdamDescriptor(self.weights.numel(), self.steps, lr, 0.9, 0.99, 1e-15, 1e-15, 1e-6, 1))
        return self.loss
