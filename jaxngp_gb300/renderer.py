"""Device-resident inference renderer (render_image_inference of models/renderers/cuda.py:244-373).

The reference renders a frame with a host loop over (march_rays_inference -> field ->
integrate_rays_inference) on 8192 rays x 8 steps, reading the number of finished rays back to the
host after every iteration and blocking the stream inside march_rays_inference
(marching.cu:562).  Here the same three stages run with every ray of the frame resident and
hundreds of thousands of slots in flight; slot indices, t_starts, the colour/transmittance
accumulators and a running count of finished rays are updated in place on the device
(ngp_march_rays_inference_inplace, ngp_integrate_rays_inference_inplace), and the host reads the
count only once every `poll_every` iterations.
"""
from __future__ import annotations

from typing import Tuple

import torch

from . import _lib as L
from .encoders import LevelTable, forward_call
from .field import FieldOps


class Renderer:
    def __init__(self, latents: torch.Tensor, weights: torch.Tensor, table: LevelTable, bitfield: torch.Tensor,
                 K: int, G: int, bound: float, stepsize_portion: float, diagonal_n_steps: int = 1024,
                 n_slots: int = 1 << 18, march_steps_cap: int = 8, poll_every: int = 4, precision: str = "fp32",
                 compact: bool = True, activations: torch.dtype = torch.float32):
        self.latents, self.weights, self.table, self.bitfield = latents, weights, table, bitfield
        self.K, self.G, self.bound, self.sp, self.dns = K, G, float(bound), float(stepsize_portion), diagonal_n_steps
        self.n_slots, self.cap, self.poll_every = n_slots, march_steps_cap, poll_every
        self.field = FieldOps(precision)
        self.compact = compact
        if compact and march_steps_cap > 16:
            raise ValueError("the compact renderer supports march_steps_cap <= 16")
        dev = latents.device
        n, c = n_slots, march_steps_cap
        f32 = dict(dtype=torch.float32, device=dev)
        self.xyzs = torch.empty(n * c, 3, **f32)
        self.dirs = torch.empty(n * c, 3, **f32)
        self.dss = torch.empty(n, c, **f32)
        self.zs = torch.empty(n, c, **f32)
        self.enc = torch.empty(n * c, 32, dtype=activations, device=dev)
        self.drgbs = torch.empty(n * c, 4, **f32)
        self.n_samples = torch.empty(n, dtype=torch.int32, device=dev)
        self.indices = torch.empty(n, dtype=torch.int32, device=dev)
        self.terminated = torch.empty(n, dtype=torch.bool, device=dev)
        self.next_ray = torch.empty(1, dtype=torch.int32, device=dev)
        self.sample_start = torch.empty(n, dtype=torch.int32, device=dev)
        self.sample_count = torch.empty(1, dtype=torch.int32, device=dev)
        self.total = torch.empty(1, dtype=torch.int32, device=dev)
        self.total_host = torch.empty(1, dtype=torch.int32).pin_memory()
        self.iterations = 0

    @classmethod
    def from_trainer(cls, tr, **kw) -> "Renderer":
        kw.setdefault("precision", tr.cfg.mlp_precision)
        kw.setdefault("activations", tr.enc.dtype)
        return cls(tr.gather_table, tr.weights, tr.table, tr.bitfield, tr.K, tr.cfg.G, tr.bound, tr.sp,
                   tr.cfg.diagonal_n_steps, **kw)

    @torch.no_grad()
    def render_rays(self, rays_o: torch.Tensor, rays_d: torch.Tensor, t_starts: torch.Tensor, t_ends: torch.Tensor,
                    rays_bg: torch.Tensor, max_iterations: int = 100000) -> Tuple[torch.Tensor, int]:
        """Returns (rays_rgbd [N,4], iterations).  `t_starts` is consumed (advanced in place)."""
        N = rays_o.shape[0]
        n, cap = self.n_slots, self.cap
        rgbd = torch.zeros(N, 4, dtype=torch.float32, device=rays_o.device)
        T = torch.ones(N, dtype=torch.float32, device=rays_o.device)
        self.terminated.fill_(True)   # every slot starts by taking a fresh ray
        self.indices.zero_()
        self.next_ray.zero_()
        self.total.zero_()
        dm = L.MarchingInferenceDescriptor(N, n, self.dns, self.K, self.G, cap, self.bound, self.sp)
        di = L.IntegratingInferenceDescriptor(N, n, cap)
        hg, dh = forward_call(self.table.descriptor(n * cap, self.bound), self.latents, self.enc)
        it = 0
        while it < max_iterations:
            for _ in range(self.poll_every):
                if self.compact:
                    self.sample_count.zero_()
                    L.call("ngp_march_rays_inference_compact",
                           [rays_o, rays_d, t_starts, t_ends, self.bitfield, self.terminated, self.indices,
                            self.next_ray, self.n_samples, self.sample_start, self.sample_count, self.xyzs, self.dirs,
                            self.dss, self.zs], dm)
                    L.call(hg, [self.xyzs, self.latents, self.sample_count, self.enc], dh)
                    self.field.forward(self.enc, self.dirs, self.weights, self.sample_count, self.drgbs)
                    L.call("ngp_integrate_rays_inference_compact",
                           [rays_bg, rgbd, T, self.n_samples, self.indices, self.dss, self.zs, self.drgbs,
                            self.sample_start, self.total, self.terminated], di)
                else:
                    L.call("ngp_march_rays_inference_inplace",
                           [rays_o, rays_d, t_starts, t_ends, self.bitfield, self.terminated, self.indices,
                            self.next_ray, self.n_samples, self.xyzs, self.dirs, self.dss, self.zs], dm)
                    L.call(hg, [self.xyzs, self.latents, None, self.enc], dh)
                    self.field.forward(self.enc, self.dirs, self.weights, None, self.drgbs)
                    L.call("ngp_integrate_rays_inference_inplace",
                           [rays_bg, rgbd, T, self.n_samples, self.indices, self.dss, self.zs, self.drgbs, self.total,
                            self.terminated], di)
                it += 1
            self.total_host.copy_(self.total, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            if int(self.total_host[0]) >= N:
                break
        self.iterations = it
        return rgbd, it

    @torch.no_grad()
    def render_image(self, camera, transform: torch.Tensor, bg=(1.0, 1.0, 1.0)) -> Tuple[torch.Tensor, torch.Tensor]:
        """(rgb u8 [H, W, 3], depth f32 [H, W]) of one pinhole view."""
        from .trainer import camera_rays, near_far
        o, d = camera_rays(camera, transform)
        t0, t1 = near_far(self.bound, o, d)
        bgt = torch.as_tensor(bg, dtype=torch.float32, device=o.device).expand(o.shape[0], 3).contiguous()
        rgbd, _ = self.render_rays(o, d, t0.contiguous(), t1, bgt)
        rgb = (rgbd[:, :3].clamp(0, 1) * 255).round().to(torch.uint8).view(camera.height, camera.width, 3)
        return rgb, rgbd[:, 3].view(camera.height, camera.width)


class ProposalRenderer:
    """Inference with the learned proposal instead of the occupancy-grid march (no reference
    counterpart): rays in chunks; per chunk the proposal places samples_per_ray samples on every
    ray that crosses an occupied coarse block (ngp_proposal_rays, _bin_points, the FP16 proposal
    MLP, ngp_proposal_sample), the field evaluates them (encoder and field MLP at the trainer's
    precision) and integrate_rays composites them; rays that cross no occupied block show the
    background.  The trained proposal and field are shared with the trainer, not copied."""

    def __init__(self, tr, chunk: int = 1 << 16):
        if tr.prop is None:
            raise ValueError("the trainer has no proposal sampler")
        self.tr = tr
        self.chunk = chunk
        self.ps = tr.prop.for_rendering(chunk)
        dev = tr.dev
        S = self.ps.S
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self.valid = torch.zeros(chunk, dtype=torch.bool, device=dev)
        self.n_samples, self.startidx = torch.zeros(chunk, **i32), torch.zeros(chunk, **i32)
        self.idcs = torch.zeros(S, **i32)
        self.xyzs, self.dirs = torch.zeros(S, 3, **f32), torch.zeros(S, 3, **f32)
        self.dss, self.zs = torch.zeros(S, **f32), torch.zeros(S, **f32)
        self.enc = torch.empty(S, 32, dtype=tr.enc.dtype, device=dev)
        self.drgbs = torch.zeros(S, 4, **f32)
        self.measured = torch.zeros(1, **i32)
        self.opacity = torch.zeros(chunk, **f32)
        self.hg = forward_call(tr.table.descriptor(S, tr.bound), tr.gather_table, self.enc)

    @torch.no_grad()
    def render_rays(self, rays_o, rays_d, t_starts, t_ends, rays_bg) -> torch.Tensor:
        """rays_rgbd [N, 4]."""
        tr, ps = self.tr, self.ps
        N = rays_o.shape[0]
        out = torch.empty(N, 4, dtype=torch.float32, device=rays_o.device)
        for s0 in range(0, N, self.chunk):
            n = min(self.chunk, N - s0)
            sl = slice(s0, s0 + n)
            o, d = rays_o[sl].contiguous(), rays_d[sl].contiguous()
            t0, t1 = t_starts[sl].contiguous(), t_ends[sl].contiguous()
            cnt = ps.sample(o, d, t0, t1, self.valid[:n], self.n_samples[:n], self.startidx[:n], self.idcs, self.xyzs,
                            self.dirs, self.dss, self.zs, False, 0)
            L.call(self.hg[0], [self.xyzs, tr.gather_table, cnt, self.enc], self.hg[1])
            tr.field.forward(self.enc, self.dirs, tr.weights, cnt, self.drgbs)
            L.call("integrate_rays", [self.startidx[:n], self.n_samples[:n], rays_bg[sl].contiguous(), self.dss, self.zs,
                                      self.drgbs, self.measured, out[sl], self.opacity[:n]],
                   L.IntegratingDescriptor(n, ps.S))
        return out

    @torch.no_grad()
    def render_image(self, camera, transform: torch.Tensor, bg=(1.0, 1.0, 1.0)) -> Tuple[torch.Tensor, torch.Tensor]:
        """(rgb u8 [H, W, 3], depth f32 [H, W]) of one pinhole view."""
        from .trainer import camera_rays, near_far
        o, d = camera_rays(camera, transform)
        t0, t1 = near_far(self.tr.bound, o, d)
        bgt = torch.as_tensor(bg, dtype=torch.float32, device=o.device).expand(o.shape[0], 3).contiguous()
        rgbd = self.render_rays(o, d, t0, t1, bgt)
        rgb = (rgbd[:, :3].clamp(0, 1) * 255).round().to(torch.uint8).view(camera.height, camera.width, 3)
        return rgb, rgbd[:, 3].view(camera.height, camera.width)
