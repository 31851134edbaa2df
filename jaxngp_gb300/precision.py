"""Mixed precision: 16-bit storage types and the dynamic loss scale (no reference counterpart;
the reference trains in FP32 throughout, models/nerfs.py and models/encoders.py).

BF16 has FP32's exponent range, so its gradients need no scaling; FP16's smallest normal value is
6.1e-5, below which the field's per-sample gradients (of order 1/n_rays) would flush, so the FP16
backward runs on gradients multiplied by a loss scale (2^16 to start).  The scale lives on the
device (NgpLossScale, 16 bytes): the field backward multiplies by it and flags values that
overflow their 16-bit type, ngp_adam_mixed skips a flagged step and divides the gradients by the
scale otherwise, and ngp_loss_scale_update halves the scale after an overflow and doubles it after
`growth_interval` clean steps.  No host synchronisation is involved.
"""
from __future__ import annotations

import torch

from . import _lib as L

PRECISIONS = ("fp32", "bf16", "fp16")
TORCH_DTYPE = {"fp32": torch.float32, "bf16": torch.bfloat16, "fp16": torch.float16}
CODE = {"fp32": L.DTYPE_F32, "bf16": L.DTYPE_BF16, "fp16": L.DTYPE_F16}
CODE_OF_DTYPE = {torch.float32: L.DTYPE_F32, torch.bfloat16: L.DTYPE_BF16, torch.float16: L.DTYPE_F16}


def check(precision: str) -> str:
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    return precision


def dtype_code(t: torch.Tensor) -> int:
    try:
        return CODE_OF_DTYPE[t.dtype]
    except KeyError:
        raise ValueError(f"unsupported storage type {t.dtype}") from None


class LossScale:
    """Device-resident dynamic loss scale (NgpLossScale)."""

    def __init__(self, device="cuda", init: float = 2.0 ** 16, growth_factor: float = 2.0, backoff_factor: float = 0.5,
                 growth_interval: int = 2000, max_scale: float = 2.0 ** 24, min_scale: float = 1.0):
        self.state = torch.zeros(4, dtype=torch.int32, device=device)
        self.state[0:1].view(torch.float32).fill_(float(init))
        self.desc = L.NgpLossScaleDescriptor(growth_factor, backoff_factor, int(growth_interval), max_scale, min_scale)

    def update(self):
        L.call("ngp_loss_scale_update", [self.state], self.desc)

    def read(self) -> dict:
        """Host copy of the state (synchronises)."""
        s = self.state.cpu()
        return {"scale": float(s[0:1].view(torch.float32).item()), "overflow": int(s[1]),
                "good_steps": int(s[2]), "skipped_steps": int(s[3])}


def integrate_rays_fp64(rays_sample_startidx: torch.Tensor, rays_n_samples: torch.Tensor, bgs: torch.Tensor,
                        dss: torch.Tensor, z_vals: torch.Tensor, drgbs: torch.Tensor):
    """FP64 checker of integrate_rays on the GPU (ngp_integrate_rays_fp64): the same compositing in
    double on the float inputs.  Returns (rgbd f64[R,4], transmittance f64[R], n_used int32[R]).
    For stating errors only; no training or rendering path calls it."""
    R = rays_sample_startidx.shape[0]
    dev = dss.device
    rgbd = torch.empty(R, 4, dtype=torch.float64, device=dev)
    trans = torch.empty(R, dtype=torch.float64, device=dev)
    used = torch.empty(R, dtype=torch.int32, device=dev)
    bgs = bgs.expand(R, 3).contiguous() if bgs.dim() == 1 else bgs.contiguous()
    L.call("ngp_integrate_rays_fp64", [rays_sample_startidx, rays_n_samples, bgs, dss, z_vals, drgbs.contiguous(),
                                       rgbd, trans, used], L.IntegratingDescriptor(R, dss.shape[0]))
    return rgbd, trans, used
