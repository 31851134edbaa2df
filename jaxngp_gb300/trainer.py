"""The plain NGP training step on libngp_gb300 (the path `train_step` takes in the reference).

One step (app/nerf/_utils.py:80-170 with models/renderers/cuda.py:100-162):
    ray batch (pixel indices -> rays, near/far, jitter, background, target colour)   ngp_train_rays
    march_rays over the occupancy bitfield (training variant)                        ngp_march_rays_train
    hash-grid encoding of the samples                                                ngp_hashgrid_forward
    density/colour MLP                                                               ngp_field_forward
    integrate_rays + masked Huber loss + integrate_rays_backward                     ngp_integrate_loss_backward
    MLP backward (recomputing activations)                                           ngp_field_backward
    table-gradient scatter                                                           ngp_hashgrid_backward
    Adam on the table and on the MLP (+ decayed weights)                             ngp_adam
then, on the reference's cadence (utils/types.py:1378-1392), the occupancy-grid refresh
(decay, sample, density query, max, threshold, packbits).

Everything is enqueued on the current CUDA stream with preallocated buffers; a step never
synchronises with the host (metrics stay on the device until read).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _lib as L
from . import precision as MP
from .encoders import LevelTable, backward_call, forward_call
from .field import SHAPES, FieldOps, glorot_uniform, pack_weights
from .scene import SceneData


@dataclass
class TrainConfig:
    total_samples: int = 1 << 18       # sample budget per step (the reference's batch size)
    n_rays: Optional[int] = None       # rays per step; the reference uses total_samples (train.py:48)
    diagonal_n_steps: int = 1024
    G: int = 128
    perturb: bool = True
    random_bg: bool = True
    lr: float = 1e-2
    L: int = 16
    T: int = 1 << 19
    N_min: int = 16
    N_max: Optional[int] = None        # 2048 * bound (nerfs.py:322-331)
    per_level_scale: Optional[float] = None
    near: float = 0.3
    huber_delta: float = 0.1
    seed: int = 0
    mlp_precision: str = "fp32"        # "fp32" (parity path, FP32 accuracy), "bf16" or "fp16"
    table_precision: str = "fp32"      # "bf16"/"fp16": the encoder gathers from a 16-bit copy of the
                                       # FP32 table, which the table's Adam update rewrites
    half_activations: bool = False     # encodings and their gradient in the MLP's 16-bit type
    loss_scale: Optional[float] = None # initial dynamic loss scale; None: 2^16 with an FP16 MLP, else off
    sampler: str = "march"             # "march" (occupancy grid, the reference's) or "proposal"
    proposal_every: int = 4            # proposal updates every k steps
    proposal_distill: bool = True      # also regress the proposal at points drawn in occupied cells
    proposal_samples: int = 48         # samples on each ray the proposal samples
    proposal_mix: float = 0.1          # share of a uniform pdf mixed into the proposal's
    march_every: int = 8               # proposal sampler: every k-th step marches the occupancy grid (0: never)
    proposal_fallback: bool = False    # proposal sampler: march the rays whose proposal misses > 1% of transmittance
    proposal_train_points: int = 1 << 16   # field samples a proposal update regresses on (at most)
    pipeline: bool = False             # march sampler: march the next step's batch on a second stream while
                                       # this step's field, integrator, backwards and Adam run (same results)
    pipeline_march_blocks: int = 10    # CTAs per SM of that march (measured: 8-10 best; fewer starve it)
    march_coarse_skip: bool = True     # march: skip empty coarse blocks (8^3 cells) in one step and finish
                                       # rays that cross no occupied block at once (exact: the same samples)
    tv_scale: float = 0.0              # the encoder's total-variation term (encoders.py:236-254), added to
                                       # the loss and its gradient to the table's (0: off, the reference's default)
    empty_space_decay: float = 0.0     # proposal sampler: weight of an L1 term on the density at uniform random
                                       # points of the box, added to the step's gradients (0: off).  Space the
                                       # proposal's samples never visit gets no photometric gradient and keeps
                                       # its initial density, which the march renderer then shows as fog.
    empty_space_points: int = 1 << 14  # random points per step of that term


def cascades_for(bound: float) -> int:
    """SceneMeta.cascades (utils/types.py:858-860)."""
    return max(1, int(1 + math.ceil(math.log2(bound))))


def stepsize_portion_for(bound: float) -> float:
    """SceneMeta.stepsize_portion (utils/types.py:874-886)."""
    if bound >= 64:
        return 1 / 128
    if bound >= 16:
        return 6e-3
    if bound >= 4:
        return 5e-3
    if bound > 1:
        return 1 / 256
    return 0.0


def lr_at(lr: float, count: int) -> float:
    """optax.exponential_decay(lr, 10k, 1/3, staircase, begin 10k, end lr/100) (_utils.py:20-27)."""
    p = math.floor(max(count - 10_000, 0) / 10_000)
    return max(lr * (1 / 3) ** p, lr / 100)


class NGPTrainer:
    def __init__(self, data: SceneData, cfg: TrainConfig = TrainConfig(), device="cuda"):
        L.require_cuda()
        self.data, self.cfg = data, cfg
        self.dev = torch.device(device)
        bound = float(data.bound)
        self.bound = bound
        self.K = cascades_for(bound)
        self.sp = stepsize_portion_for(bound)
        self.R = cfg.n_rays or cfg.total_samples
        self.S = cfg.total_samples
        self.field = FieldOps(cfg.mlp_precision)
        MP.check(cfg.table_precision)
        if cfg.half_activations and cfg.mlp_precision == "fp32":
            raise ValueError("half_activations needs a 16-bit MLP (mlp_precision bf16 or fp16)")
        act = MP.TORCH_DTYPE[cfg.mlp_precision] if cfg.half_activations else torch.float32
        self.table = LevelTable(cfg.L, cfg.T, 2, cfg.N_min, cfg.N_max or int(2 ** 11 * bound), cfg.per_level_scale)
        P = self.table.n_params
        g = torch.Generator(device=self.dev)
        g.manual_seed(cfg.seed)
        f32 = dict(dtype=torch.float32, device=self.dev)
        i32 = dict(dtype=torch.int32, device=self.dev)
        # parameters and optimiser state (_utils.py:19-77: one Adam for the field)
        self.latents = torch.empty(P, 2, **f32).uniform_(-1e-4, 1e-4, generator=g)
        self.weights = pack_weights({k: glorot_uniform(s, g, self.dev) for k, s in SHAPES})
        self.g_lat = torch.zeros(P, 2, **f32)
        self.g_w = torch.zeros(L.MLP_WEIGHTS, **f32)
        self.m_lat, self.v_lat = torch.zeros(P, 2, **f32), torch.zeros(P, 2, **f32)
        self.m_w, self.v_w = torch.zeros(L.MLP_WEIGHTS, **f32), torch.zeros(L.MLP_WEIGHTS, **f32)
        # occupancy grid (OccupancyDensityGrid.create, utils/types.py:111-140)
        G3 = cfg.G ** 3
        self.G3 = G3
        self.density = torch.zeros(self.K * G3, **f32)
        self.occ_mask = torch.zeros(self.K * G3, dtype=torch.bool, device=self.dev)
        self.bitfield = torch.full((self.K * G3 // 8,), 255, dtype=torch.uint8, device=self.dev)
        self.threshold = torch.zeros(1, **f32)
        self.thr_scratch = torch.zeros(2, **f32)
        self.thr_step = 0.01 * cfg.diagonal_n_steps / (2 * min(bound, 1) * 3 ** 0.5)
        # batch buffers (rays and their samples): two sets when the next batch is marched ahead
        R, S = self.R, self.S
        self.pipeline = bool(cfg.pipeline) and cfg.sampler == "march"
        self._batches = [self._new_batch(R, S) for _ in range(2 if self.pipeline else 1)]
        self._use_batch(0)
        self._side = torch.cuda.Stream(device=self.dev) if self.pipeline else None
        self._prepared = [None, None]   # events after which a batch prepared on the side stream is ready
        self._ready = None              # the batch prepared for the next step
        self.enc = torch.empty(S, 32, dtype=act, device=self.dev)
        self.drgbs = torch.empty(S, 4, **f32)
        self.g_drgbs = torch.empty(S, 4, **f32)
        self.g_enc = torch.empty(S, 32, dtype=act, device=self.dev)
        self.stats = torch.zeros(4, **f32)
        self.grad_scale = torch.zeros(1, **f32)
        self.loss_scratch = torch.zeros(4 + R, **f32)
        self.mlp_scratch = torch.empty(L.field_backward_scratch_floats(), **f32)
        # mixed precision: the 16-bit working copy of the table and the dynamic loss scale
        self.lat_h = self.latents.to(MP.TORCH_DTYPE[cfg.table_precision]) if cfg.table_precision != "fp32" else None
        ls0 = cfg.loss_scale if cfg.loss_scale is not None else (2.0 ** 16 if cfg.mlp_precision == "fp16" else 0.0)
        self.loss_scale = MP.LossScale(self.dev, init=ls0) if ls0 > 0 else None
        self.step_count = 0
        self._seed = np.random.SeedSequence(cfg.seed)
        # descriptors that do not change between steps
        self._d_march = L.MarchingDescriptor(R, S, cfg.diagonal_n_steps, self.K, cfg.G, bound, self.sp)
        self._hg_fwd = forward_call(self.table.descriptor(S, bound), self.gather_table, self.enc)
        self._hg_bwd = backward_call(self.table.descriptor(S, bound, accumulate=True), self.g_enc)
        # the TV term over the whole sample buffer (the reference evaluates the field on all of it)
        self._d_tv = L.NgpHashGridTVDescriptor(self.table.descriptor(S, bound), float(cfg.tv_scale), 1)
        self.tv = torch.zeros(1, **f32)
        self.tv_acc = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self._d_mlp = L.NgpMlpDescriptor(S, 0)
        self._d_loss = L.NgpIntegrateLossDescriptor(R, S, data.camera.near if hasattr(data.camera, "near") else cfg.near,
                                                    cfg.huber_delta)
        self._n_alive = None
        self.cadence_offset = 0   # added to step_count for the occupancy-grid cadence only
        self.prop = None
        # coarse occupancy blocks for the marcher's shortcut over rays that cannot take a sample
        self.coarse = torch.zeros((cfg.G // 8) ** 3, dtype=torch.uint8, device=self.dev) \
            if (self.K == 1 and cfg.G % 8 == 0) else None
        if cfg.sampler == "proposal":
            from .proposal import ProposalSampler
            if self.K != 1:
                raise ValueError("the proposal sampler supports scenes with one occupancy cascade (bound <= 1)")
            self.prop = ProposalSampler(R, S, cfg.G, bound, self.dev, seed=cfg.seed, samples_per_ray=cfg.proposal_samples,
                                        mix=cfg.proposal_mix)
            self.enc_d = torch.empty(self.prop.M, 32, **f32)
        elif cfg.sampler != "march":
            raise ValueError(f"sampler must be 'march' or 'proposal', got {cfg.sampler!r}")
        self.empty = None
        if cfg.empty_space_decay > 0 and self.prop is not None:
            M = int(cfg.empty_space_points)
            g_rows = torch.zeros(M, 4, **f32)
            g_rows[:, 0] = float(cfg.empty_space_decay) / M   # d(decay * mean density)/d density
            dirs = torch.zeros(M, 3, **f32)
            dirs[:, 2] = 1.0                                   # no colour gradient: any unit direction
            gen = torch.Generator(device=self.dev)
            gen.manual_seed(cfg.seed + 0x9E3779B9)
            genc = torch.empty(M, 32, dtype=act, device=self.dev)
            self.empty = dict(M=M, xyz=torch.empty(M, 3, **f32), enc=torch.empty(M, 32, dtype=act, device=self.dev),
                              genc=genc, dirs=dirs, g=g_rows, gen=gen,
                              bwd=backward_call(self.table.descriptor(M, bound, accumulate=True), genc))
        self.mark_untrained_grid()

    # ---------------------------------------------------------------------------- helpers
    BATCH_FIELDS = ("rays_o", "rays_d", "t0", "t1", "noise", "bgs", "gt", "counters", "queue", "count", "valid",
                    "n_samples", "startidx", "idcs", "xyzs", "dirs", "dss", "z_vals")

    def _new_batch(self, R: int, S: int) -> dict:
        f32 = dict(dtype=torch.float32, device=self.dev)
        i32 = dict(dtype=torch.int32, device=self.dev)
        return dict(rays_o=torch.empty(R, 3, **f32), rays_d=torch.empty(R, 3, **f32), t0=torch.empty(R, **f32),
                    t1=torch.empty(R, **f32), noise=torch.empty(R, **f32), bgs=torch.empty(R, 3, **f32),
                    gt=torch.empty(R, 3, **f32), counters=torch.zeros(2, **i32), queue=torch.zeros(1, **i32),
                    count=torch.zeros(1, **i32), valid=torch.empty(R, dtype=torch.bool, device=self.dev),
                    n_samples=torch.empty(R, **i32), startidx=torch.empty(R, **i32), idcs=torch.empty(S, **i32),
                    xyzs=torch.empty(S, 3, **f32), dirs=torch.empty(S, 3, **f32), dss=torch.empty(S, **f32),
                    z_vals=torch.empty(S, **f32))

    def _use_batch(self, i: int):
        for k in self.BATCH_FIELDS:
            setattr(self, k, self._batches[i][k])

    @property
    def gather_table(self) -> torch.Tensor:
        """The table the encoder forward reads: the 16-bit copy when there is one."""
        return self.lat_h if self.lat_h is not None else self.latents

    def sync_half_table(self):
        """Rewrites the 16-bit table copy from the FP32 table (after the latents were set from
        outside; the Adam update keeps it current otherwise)."""
        if self.lat_h is not None:
            self.lat_h.copy_(self.latents)

    def _encode(self, xyz: torch.Tensor, count, enc: torch.Tensor, n: int):
        name, desc = forward_call(self.table.descriptor(n, self.bound), self.gather_table, enc)
        L.call(name, [xyz, self.gather_table, count, enc], desc)

    def _next_seed(self) -> int:
        return int(self._seed.spawn(1)[0].generate_state(1, np.uint64)[0])

    def _ogrid_desc(self, cascade=0, n_points=0, update_all=False, seed=0) -> L.NgpOgridDescriptor:
        c = self.data.camera
        return L.NgpOgridDescriptor(self.K, self.cfg.G, cascade, n_points, 1 if update_all else 0, self.bound, 0.95,
                                    self.thr_step, seed, self.data.n_views, c.width, c.height, c.fx, c.fy, c.cx, c.cy)

    def mark_untrained_grid(self):
        """utils/types.py:1241-1362 followed by the step-0 packbits with threshold -0.5."""
        L.call("ngp_ogrid_mark_untrained", [self.data.transforms, self.density], self._ogrid_desc())
        thr = torch.full((1,), -0.5, dtype=torch.float32, device=self.dev)
        L.call("ngp_packbits_scalar", [thr, self.density, self.occ_mask, self.bitfield],
               L.PackbitsDescriptor(self.K * self.G3 // 8))
        self._refresh_coarse()
        self._n_alive = [int((self.density[c * self.G3:(c + 1) * self.G3] >= 0).sum().item()) for c in range(self.K)]

    @torch.no_grad()
    def init_occupancy_analytic(self, scene=None, steady_state: bool = True):
        """Fill the density grid from the scene's analytic density at cell centres (a stand-in for
        a converged grid), threshold it as threshold_ogrid does, and, with `steady_state`, run the
        grid refresh on the cadence of a run past its first 256 steps (partial updates every 16
        steps).  Cells marked untrainable keep density -1."""
        from .volrendjax import morton3d_invert
        scene = scene or self.data.scene
        G, G3 = self.cfg.G, self.G3
        xyz = morton3d_invert(torch.arange(G3, dtype=torch.int32, device=self.dev)).float()
        blobs = torch.from_numpy(scene.blobs).to(self.dev).double()
        for c in range(self.K):
            mb = min(2.0 ** c, self.bound)
            centres = (((xyz.double() + 0.5) / G - 0.5) * 2 * mb)
            dens = torch.zeros(G3, dtype=torch.float64, device=self.dev)
            for s0 in range(0, G3, 1 << 18):
                x = centres[s0:s0 + (1 << 18)]
                r2 = ((x[:, None, :] - blobs[None, :, :3]) ** 2).sum(-1)
                dens[s0:s0 + (1 << 18)] = (blobs[None, :, 4] * torch.exp(-r2 / (2 * blobs[None, :, 3] ** 2))).sum(-1)
                if len(scene.shells):   # thin shells: every cell the shell passes through
                    sh = torch.from_numpy(scene.shells).to(self.dev).double()
                    half_diag = 3 ** 0.5 * mb / G
                    dist = ((x[:, None, :] - sh[None, :, :3]) ** 2).sum(-1).sqrt() - sh[None, :, 3]
                    near = dist.abs() <= sh[None, :, 4] + half_diag
                    dens[s0:s0 + (1 << 18)] += (near.double() * sh[None, :, 5]).sum(-1)
            cur = self.density[c * G3:(c + 1) * G3]
            cur.copy_(torch.where(cur < 0, cur, dens.float()))
        live0 = self.density[:G3][self.density[:G3] >= 0]
        self.threshold.fill_(min(self.thr_step, float(live0.mean().item())))
        L.call("ngp_packbits_scalar", [self.threshold, self.density, self.occ_mask, self.bitfield],
               L.PackbitsDescriptor(self.K * self.G3 // 8))
        self._refresh_coarse()
        if steady_state:
            self.cadence_offset = 256

    def ogrid_due(self, step: int) -> bool:
        """NeRFState.should_call_update_ogrid (utils/types.py:1378-1388)."""
        interval = min(16, step // 16 + 1)
        return step > 0 and step % interval == 0

    def update_ogrid(self):
        """update_ogrid_density for every cascade (types.py:1149-1225), then threshold_ogrid
        (types.py:1227-1239)."""
        update_all = self.step_count + self.cadence_offset < 256
        chunk = 1 << 20
        for cas in range(self.K):
            M = self.G3 if update_all else max(1, self._n_alive[cas] // 2)
            d = self._ogrid_desc(cas, M, update_all, self._next_seed())
            L.call("ngp_ogrid_decay", [self.density], d)
            cells = torch.empty(M, dtype=torch.int32, device=self.dev)
            xyz = torch.empty(M, 3, dtype=torch.float32, device=self.dev)
            L.call("ngp_ogrid_sample", [self.density, self.bitfield, cells, xyz], d)
            sigma = torch.empty(M, dtype=torch.float32, device=self.dev)
            for s in range(0, M, chunk):
                n = min(chunk, M - s)
                enc = self.enc[:n] if n <= self.S else torch.empty(n, 32, dtype=self.enc.dtype, device=self.dev)
                self._encode(xyz[s:s + n], None, enc, n)
                self.field.density(enc, self.weights, sigma[s:s + n], n)
            L.call("ngp_ogrid_max", [cells, sigma, self.density], d)
        L.call("ngp_ogrid_threshold", [self.density, self.thr_scratch, self.threshold], self._ogrid_desc())
        L.call("ngp_packbits_scalar", [self.threshold, self.density, self.occ_mask, self.bitfield],
               L.PackbitsDescriptor(self.K * self.G3 // 8))
        self._refresh_coarse()

    def _refresh_coarse(self):
        """Coarse occupancy blocks of the current bitfield, for the marcher's shortcut and the
        proposal sampler (which shares them)."""
        if self.coarse is not None:
            L.call("ngp_proposal_coarse", [self.bitfield, self.coarse],
                   L.NgpProposalDescriptor(0, 48, self.cfg.G, self.bound, 0, 0, 0, 3, 1, 0, 0.1))
        if self.prop is not None:
            if self.coarse is not None:
                self.prop.coarse = self.coarse
            else:
                self.prop.refresh(self.bitfield)

    def _distill(self, xyz: torch.Tensor, sigma: torch.Tensor):
        """The field's density at points drawn in the occupancy grid (half anywhere, half in
        occupied cells), for the proposal's regression."""
        M = xyz.shape[0]
        d = self._ogrid_desc(0, M, False, self._next_seed())
        L.call("ngp_ogrid_sample", [self.density, self.bitfield, self.prop.cells, xyz], d)
        self._encode(xyz, None, self.enc_d, M)
        self.field.density(self.enc_d, self.weights, sigma, M)

    # ------------------------------------------------------------------------------- step
    def _rays(self, b: dict, perm, stream=None) -> int:
        """ngp_train_rays into batch `b`; returns the step seed."""
        cfg, c = self.cfg, self.data.camera
        seed = self._next_seed()
        d_rays = L.NgpTrainRaysDescriptor(self.R, c.width, c.height, self.data.n_views, c.fx, c.fy, c.cx, c.cy,
                                          self.bound, int(cfg.perturb), int(cfg.random_bg), (L.c_f32 * 3)(1, 1, 1), seed)
        L.call("ngp_train_rays", [self.data.transforms, self.data.rgbas, perm, b["rays_o"], b["rays_d"], b["t0"],
                                  b["t1"], b["noise"], b["bgs"], b["gt"]], d_rays, stream=stream)
        return seed

    def _march(self, b: dict, stream=None):
        """The training march of batch `b` and its sample count."""
        L.call("ngp_march_rays_train", [b["rays_o"], b["rays_d"], b["t0"], b["t1"], b["noise"], self.bitfield,
                                        b["counters"][0:1], b["counters"][1:2], b["valid"], b["n_samples"],
                                        b["startidx"], b["idcs"], b["xyzs"], b["dirs"], b["dss"], b["z_vals"],
                                        b["queue"], self.coarse if self.cfg.march_coarse_skip else None],
               self._d_march, stream=stream)
        L.call("ngp_march_count", [b["counters"][0:1], b["counters"][1:2], b["count"]], stream=stream)

    def _prepare_ahead(self, i: int, perm):
        """Rays and march of batch i on the side stream, after everything queued on this stream so
        far (the previous user of batch i, the copy of `perm`), with the march kept to
        pipeline_march_blocks CTAs per SM so that this stream's kernels run beside it."""
        main = torch.cuda.current_stream(self.dev)
        entry = torch.cuda.Event()
        entry.record(main)
        self._side.wait_event(entry)
        side = self._side.cuda_stream
        self._rays(self._batches[i], perm, side)
        prev = L.lib().ngp_set_march_blocks_per_sm(int(self.cfg.pipeline_march_blocks))
        try:
            self._march(self._batches[i], side)
        finally:
            L.lib().ngp_set_march_blocks_per_sm(prev)
        ev = torch.cuda.Event()
        ev.record(self._side)
        self._prepared[i] = ev

    def step(self, perm: Optional[torch.Tensor] = None) -> torch.Tensor:
        """One training step.  `perm`: int32 pixel indices [n_rays] on the device (as the
        reference's `perm`), or None to draw them on the device.  Returns the device tensor
        [loss, n_valid_rays, measured_batch_size, measured_batch_size_before_compaction].

        With TrainConfig.pipeline (march sampler) each call trains on the batch the previous call
        marched and marches the next one on a second stream meanwhile; `perm` then selects the
        pixels of that next batch (the first call draws its own batch on the device).  The
        results are the serial step's: the march reads only the occupancy grid, and a step that
        ends with a grid refresh marches the next batch after the refresh."""
        cfg = self.cfg
        if self.pipeline:
            if self._ready is None:
                b = self._batches[0]
                self._rays(b, None)
                self._march(b)
                self._ready = 0
            cur, nxt = self._ready, 1 - self._ready
            self._use_batch(cur)
            if self._prepared[cur] is not None:
                torch.cuda.current_stream(self.dev).wait_event(self._prepared[cur])
                self._prepared[cur] = None
            refresh = self.ogrid_due(self.step_count + 1 + self.cadence_offset)
            if not refresh:
                self._prepare_ahead(nxt, perm)
            cnt = self.count
            self._train_on(cnt, use_march=True)
            if refresh:
                self._rays(self._batches[nxt], perm)
                self._march(self._batches[nxt])
            self._ready = nxt
            return self.stats
        if self._ready is not None:   # leaving pipelined mode: let a batch still being marched finish
            for i, ev in enumerate(self._prepared):
                if ev is not None:
                    torch.cuda.current_stream(self.dev).wait_event(ev)
                    self._prepared[i] = None
            self._ready = None
            self._use_batch(0)
        seed = self._rays(self._batches[0], perm)
        use_march = self.prop is None or (cfg.march_every > 0 and self.step_count % cfg.march_every == cfg.march_every - 1)
        if use_march:
            self._march(self._batches[0])
            cnt = self.count
        else:
            fb = (self.bitfield, self.threshold, self.noise, self._d_march) if cfg.proposal_fallback else None
            cnt = self.prop.sample(self.rays_o, self.rays_d, self.t0, self.t1, self.valid, self.n_samples,
                                   self.startidx, self.idcs, self.xyzs, self.dirs, self.dss, self.z_vals, cfg.perturb,
                                   seed ^ 0x5BD1E9955BD1E995, fallback=fb)
        self._train_on(cnt, use_march)
        return self.stats

    def _train_on(self, cnt: torch.Tensor, use_march: bool):
        """The rest of the step on the current batch: encoder, field, (proposal update), fused
        integrator + loss, backwards, Adam, and the occupancy-grid refresh when due."""
        cfg = self.cfg
        L.call(self._hg_fwd[0], [self.xyzs, self.gather_table, cnt, self.enc], self._hg_fwd[1])
        self.field.forward(self.enc, self.dirs, self.weights, cnt, self.drgbs)
        if self.prop is not None and (use_march or self.step_count % cfg.proposal_every == 0):
            # march steps teach the proposal at the march's evenly spread samples
            self.prop.train(self.xyzs, self.drgbs, self._distill if cfg.proposal_distill else None, count=cnt,
                            max_points=cfg.proposal_train_points)
        L.call("ngp_integrate_loss_backward", [self.valid, self.startidx, self.n_samples, self.bgs, self.gt, self.dss,
                                               self.z_vals, self.drgbs, cnt, self.loss_scratch, self.g_drgbs,
                                               self.stats, self.grad_scale], self._d_loss)
        self.field.backward(self.enc, self.dirs, self.weights, self.g_drgbs, cnt, self.grad_scale, self.mlp_scratch,
                            self.g_enc, self.g_w, loss_scale=self.loss_scale)
        L.call(self._hg_bwd[0], [self.xyzs, self.g_enc, cnt, self.g_lat], self._hg_bwd[1])
        if cfg.tv_scale > 0:   # loss = rgb + tv (_utils.py:150-158); its gradient in the loss scale's units
            gs = self.loss_scale.state[0:1].view(torch.float32) if self.loss_scale is not None else None
            L.call("ngp_hashgrid_tv", [self.xyzs, self.latents, gs, self.tv, self.g_lat, self.tv_acc], self._d_tv)
            self.stats[0:1] += self.tv
        if self.empty is not None:
            self._empty_space_decay()
        count = self.step_count
        lr = lr_at(cfg.lr, count)
        d_lat = L.NgpAdamDescriptor(self.latents.numel(), count + 1, lr, 0.9, 0.99, 1e-15, 1e-15, 0.0, 1)
        d_w = L.NgpAdamDescriptor(self.weights.numel(), count + 1, lr, 0.9, 0.99, 1e-15, 1e-15, 1e-6, 1)
        if self.loss_scale is None and self.lat_h is None:
            L.call("ngp_adam", [self.latents, self.g_lat, self.m_lat, self.v_lat], d_lat)
            L.call("ngp_adam", [self.weights, self.g_w, self.m_w, self.v_w], d_w)
        else:
            ls = self.loss_scale.state if self.loss_scale is not None else None
            L.call("ngp_adam_mixed", [self.latents, self.g_lat, self.m_lat, self.v_lat, ls, self.lat_h],
                   L.NgpAdamMixedDescriptor(d_lat, MP.CODE[cfg.table_precision]))
            L.call("ngp_adam_mixed", [self.weights, self.g_w, self.m_w, self.v_w, ls, None],
                   L.NgpAdamMixedDescriptor(d_w, L.DTYPE_F32))
            if self.loss_scale is not None:
                self.loss_scale.update()
        self.step_count += 1
        if self.ogrid_due(self.step_count + self.cadence_offset):
            self.update_ogrid()

    def _empty_space_decay(self):
        """Adds the gradient of empty_space_decay * mean(sigma) over uniform random points of the box
        to the field's gradients: the encoder forward at the points, the field backward with a
        density-only upstream gradient (accumulated into dL/dW, under the loss scale when there is
        one), and the encoder's scatter into the table gradient."""
        e = self.empty
        torch.rand(e["xyz"].shape, generator=e["gen"], out=e["xyz"])
        e["xyz"].mul_(2.0 * self.bound).sub_(self.bound)
        self._encode(e["xyz"], None, e["enc"], e["M"])
        self.field.backward(e["enc"], e["dirs"], self.weights, e["g"], None, None, self.mlp_scratch, e["genc"],
                            self.g_w, accumulate=True, loss_scale=self.loss_scale, n=e["M"])
        L.call(e["bwd"][0], [e["xyz"], e["genc"], None, self.g_lat], e["bwd"][1])

    # -------------------------------------------------------------------------- rendering
    @torch.no_grad()
    def render_rays(self, rays_o: torch.Tensor, rays_d: torch.Tensor, bg=(1.0, 1.0, 1.0),
                    chunk: int = 1 << 16, max_samples: int = 1 << 22) -> torch.Tensor:
        """Colours [N, 3] of arbitrary rays (no jitter), marching in chunks."""
        out = torch.empty(rays_o.shape[0], 3, dtype=torch.float32, device=self.dev)
        bgt = torch.tensor(bg, dtype=torch.float32, device=self.dev)
        for s in range(0, rays_o.shape[0], chunk):
            o, d = rays_o[s:s + chunk].contiguous(), rays_d[s:s + chunk].contiguous()
            n = o.shape[0]
            t0, t1 = near_far(self.bound, o, d)
            dm = L.MarchingDescriptor(n, max_samples, self.cfg.diagonal_n_steps, self.K, self.cfg.G, self.bound, self.sp)
            i32 = dict(dtype=torch.int32, device=self.dev)
            cnt, count = torch.zeros(2, **i32), torch.zeros(1, **i32)
            valid = torch.empty(n, dtype=torch.bool, device=self.dev)
            ns, st, idc = torch.empty(n, **i32), torch.empty(n, **i32), torch.empty(max_samples, **i32)
            xyz = torch.empty(max_samples, 3, device=self.dev)
            dirs = torch.empty(max_samples, 3, device=self.dev)
            dss, zs = torch.empty(max_samples, device=self.dev), torch.empty(max_samples, device=self.dev)
            zero = torch.zeros(n, device=self.dev)
            L.call("march_rays", [o, d, t0, t1, zero, self.bitfield, cnt[0:1], cnt[1:2], valid, ns, st, idc, xyz, dirs,
                                  dss, zs], dm)
            L.call("ngp_march_count", [cnt[0:1], cnt[1:2], count])
            enc = torch.empty(max_samples, 32, dtype=self.enc.dtype, device=self.dev)
            self._encode(xyz, count, enc, max_samples)
            drgb = torch.zeros(max_samples, 4, device=self.dev)
            self.field.forward(enc, dirs, self.weights, count, drgb, max_samples)
            m = torch.empty(1, **i32)
            rgbd = torch.empty(n, 4, device=self.dev)
            opac = torch.empty(n, device=self.dev)
            bgs = bgt.expand(n, 3).contiguous()
            L.call("integrate_rays", [st, ns, bgs, dss, zs, drgb, m, rgbd, opac], L.IntegratingDescriptor(n, max_samples))
            out[s:s + n] = rgbd[:, :3]
        return out

    @torch.no_grad()
    def render_view(self, view: int, transforms: Optional[torch.Tensor] = None, bg=(1.0, 1.0, 1.0)) -> torch.Tensor:
        """RGB u8 [H, W, 3] of a view (of the training poses unless `transforms` is given)."""
        tr = self.data.transforms if transforms is None else transforms
        o, d = camera_rays(self.data.camera, tr[view])
        rgb = self.render_rays(o, d, bg)
        return (rgb.clamp(0, 1) * 255).round().to(torch.uint8).view(self.data.camera.height, self.data.camera.width, 3)


def camera_rays(cam, transform: torch.Tensor):
    """Pixel-centre rays of one view (models/renderers/cuda.py:21-53, utils/types.py:400-439)."""
    dev = transform.device
    idx = torch.arange(cam.n_pixels, device=dev)
    x = (idx % cam.width).float()
    y = torch.div(idx, cam.width, rounding_mode="floor").float()
    d = torch.stack([((x + 0.5) - cam.cx) / cam.fx, -(((y + 0.5) - cam.cy) / cam.fy), -torch.ones_like(x)], -1)
    d = d / d.norm(dim=-1, keepdim=True)
    R = transform[:9].view(3, 3)
    d_world = (d @ R.T).contiguous()
    o = transform[9:12].expand_as(d_world).contiguous()
    return o, d_world


def near_far(bound: float, o: torch.Tensor, d: torch.Tensor):
    """make_near_far_from_bound (models/renderers/cuda.py:56-97)."""
    eps = 1e-15
    d = torch.where(torch.signbit(d), torch.clamp(d, max=-eps), torch.clamp(d, min=eps))
    t0 = (-bound - o) / d
    t1 = (bound - o) / d
    ts = torch.maximum(torch.minimum(t0, t1).amax(-1), torch.zeros((), device=o.device))
    te = torch.maximum(t0, t1).amin(-1)
    return ts.contiguous(), te.contiguous()


class HeldOut:
    """Held-out views of a synthetic scene -- poses on the training hemisphere drawn with another
    seed -- with their quadrature ground truth blended over white, rendered once."""

    @torch.no_grad()
    def __init__(self, data: SceneData, n_views: int = 2, seed: int = 12345, n_steps: int = 4096, radius: float = 4.0,
                 device="cuda"):
        from .scene import hemisphere_poses, poses_to_transforms, render_views
        cam = data.camera
        self.cam, self.n_views = cam, n_views
        poses = hemisphere_poses(n_views, radius, np.random.default_rng(seed))
        self.transforms = torch.from_numpy(poses_to_transforms(poses)).to(device)
        gt = render_views(data.scene, cam, self.transforms, n_steps).view(n_views, cam.height, cam.width, 4).float() / 255
        self.gt_rgb = (gt[..., :3] * gt[..., 3:] + (1 - gt[..., 3:])).mul(255).round().to(torch.uint8)

    @torch.no_grad()
    def psnr(self, tr: "NGPTrainer", renderer=None) -> float:
        """Mean PSNR (utils/data.py:407-410) of the trainer's field rendered over a white
        background, by the occupancy-grid inference renderer unless `renderer` is given."""
        from .renderer import Renderer
        from .scene import psnr_u8
        r = renderer if renderer is not None else Renderer.from_trainer(tr, n_slots=1 << 18)
        vals = []
        for v in range(self.n_views):
            rgb, _ = r.render_image(self.cam, self.transforms[v], bg=(1.0, 1.0, 1.0))
            vals.append(psnr_u8(rgb, self.gt_rgb[v]))
        return float(np.mean(vals))


def evaluate_psnr(tr: "NGPTrainer", n_views: int = 2, seed: int = 12345, n_steps: int = 4096,
                  radius: float = 4.0) -> float:
    """Mean PSNR over `n_views` held-out views (HeldOut)."""
    return HeldOut(tr.data, n_views, seed, n_steps, radius, tr.dev).psnr(tr)
