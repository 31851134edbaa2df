"""The NGP NeRF field on the GPU kernels: hash-grid encoder -> fused density/colour MLP.

Mirrors ``make_nerf_ngp`` (models/nerfs.py:422-454) / ``NeRF.__call__`` (nerfs.py:39-86) for
training: HashGridEncoder(L=16, T=2^19, F=2, N_min=16, N_max=2048*bound), density MLP [64] -> 16
with truncated exponential on channel 0, SH degree 4 on the view direction, colour MLP [64, 64] -> 3
with sigmoid, no biases, glorot-uniform kernels.  The five kernels live packed in one float32
vector (``weights``); ``flax_params()`` / ``load_flax_params()`` convert to and from the reference's
parameter tree (position_encoder / density_mlp / rgb_mlp, Dense_i/kernel [in, out]).
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np
import torch

from . import _lib as L
from . import precision as P
from .encoders import PARAM_NAME, HashGridEncoder, hashgrid_backward, hashgrid_forward

SHAPES = [("W0", (32, 64)), ("W1", (64, 16)), ("W2", (32, 64)), ("W3", (64, 64)), ("W4", (64, 3))]
OFFSETS = {"W0": 0, "W1": 2048, "W2": 3072, "W3": 5120, "W4": 9216}
FLAX_NAMES = {"W0": ("density_mlp", "Dense_0"), "W1": ("density_mlp", "Dense_1"), "W2": ("rgb_mlp", "Dense_0"),
              "W3": ("rgb_mlp", "Dense_1"), "W4": ("rgb_mlp", "Dense_2")}


def glorot_uniform(shape, generator: Optional[torch.Generator] = None, device="cuda") -> torch.Tensor:
    lim = (6.0 / (shape[0] + shape[1])) ** 0.5
    return torch.empty(shape, dtype=torch.float32, device=device).uniform_(-lim, lim, generator=generator)


def pack_weights(w: Dict[str, torch.Tensor]) -> torch.Tensor:
    return torch.cat([torch.as_tensor(w[k], dtype=torch.float32).reshape(-1) for k, _ in SHAPES]).contiguous()


def unpack_weights(flat: torch.Tensor) -> Dict[str, torch.Tensor]:
    return {k: flat[OFFSETS[k]:OFFSETS[k] + s[0] * s[1]].view(*s) for k, s in SHAPES}


# ------------------------------------------------------------------------------ raw entry points

PRECISIONS = ("fp32", "bf16", "fp16")


def entry(name: str, precision: str) -> str:
    """Entry point of a field op for "fp32" (the parity path: tensor cores at FP32 accuracy, three
    BF16 pieces per operand) or "bf16" (tensor cores, BF16 operands with FP32 accumulation, FP32
    encodings).  FP16 and 16-bit encodings go through the
    ``*_mixed`` entries (FieldOps)."""
    if precision not in ("fp32", "bf16"):
        raise ValueError(f"entry() covers fp32 and bf16; use FieldOps for {precision!r}")
    return name if precision == "fp32" else f"{name}_{precision}"


class FieldOps:
    """The field's forward, density and backward at one operand precision.  The encodings'
    storage type is read from the tensor given (FP32, or the operand type for 16-bit
    activations); a loss scale (precision.LossScale) goes to the backward.  FP32, and BF16 with
    FP32 encodings and no loss scale, use the plain entry points; everything else the
    ``ngp_field_*_mixed`` ones."""

    def __init__(self, precision: str = "fp32"):
        self.precision = P.check(precision)
        self.code = P.CODE[precision]
        self._descs = {}

    def _plain(self, enc: torch.Tensor, loss_scale=None) -> bool:
        return self.precision == "fp32" or (self.precision == "bf16" and enc.dtype == torch.float32 and loss_scale is None)

    def _mixed(self, n: int, enc: torch.Tensor, accumulate: bool = False) -> L.NgpFieldMixedDescriptor:
        key = (n, enc.dtype, accumulate)
        d = self._descs.get(key)
        if d is None:
            act = P.dtype_code(enc)
            if self.precision == "fp32" or act not in (L.DTYPE_F32, self.code):
                raise ValueError(f"encodings of type {enc.dtype} do not fit a {self.precision} field")
            d = self._descs[key] = L.NgpFieldMixedDescriptor(n, 1 if accumulate else 0, self.code, act)
        return d

    def forward(self, enc, dirs, weights, count, out, n: Optional[int] = None):
        n = enc.shape[0] if n is None else n
        if self._plain(enc):
            L.call(entry("ngp_field_forward", self.precision), [enc, dirs, weights, count, out], L.NgpMlpDescriptor(n, 0))
        else:
            L.call("ngp_field_forward_mixed", [enc, dirs, weights, count, out], self._mixed(n, enc))
        return out

    def density(self, enc, weights, out, n: Optional[int] = None):
        n = enc.shape[0] if n is None else n
        if self._plain(enc):
            L.call(entry("ngp_field_density", self.precision), [enc, weights, out], L.NgpMlpDescriptor(n, 0))
        else:
            L.call("ngp_field_density_mixed", [enc, weights, out], self._mixed(n, enc))
        return out

    def backward(self, enc, dirs, weights, dL_ddrgb, count, grad_scale, scratch, dL_denc, dL_dw,
                 accumulate: bool = False, loss_scale=None, n: Optional[int] = None):
        n = enc.shape[0] if n is None else n
        if self._plain(enc, loss_scale):
            L.call(entry("ngp_field_backward", self.precision),
                   [enc, dirs, weights, dL_ddrgb, count, grad_scale, scratch, dL_denc, dL_dw],
                   L.NgpMlpDescriptor(n, 1 if accumulate else 0))
        else:
            if dL_denc.dtype != enc.dtype:
                raise ValueError("dL_dencodings must have the encodings' type")
            state = loss_scale.state if loss_scale is not None else None
            L.call("ngp_field_backward_mixed",
                   [enc, dirs, weights, dL_ddrgb, count, grad_scale, state, scratch, dL_denc, dL_dw],
                   self._mixed(n, enc, accumulate))
        return dL_denc, dL_dw


def field_forward(enc: torch.Tensor, dirs: torch.Tensor, weights: torch.Tensor,
                  count: Optional[torch.Tensor] = None, out: Optional[torch.Tensor] = None,
                  precision: str = "fp32") -> torch.Tensor:
    n = enc.shape[0]
    if out is None:
        out = torch.empty(n, 4, dtype=torch.float32, device=enc.device)
    return FieldOps(precision).forward(enc.contiguous(), dirs.contiguous(), weights, count, out, n)


def field_density(enc: torch.Tensor, weights: torch.Tensor, out: Optional[torch.Tensor] = None,
                  precision: str = "fp32") -> torch.Tensor:
    n = enc.shape[0]
    if out is None:
        out = torch.empty(n, dtype=torch.float32, device=enc.device)
    return FieldOps(precision).density(enc.contiguous(), weights, out, n)


_scratch: Dict[int, torch.Tensor] = {}


def backward_scratch(device) -> torch.Tensor:
    dev = torch.device(device)
    key = dev.index if dev.index is not None else torch.cuda.current_device()
    if key not in _scratch:
        _scratch[key] = torch.empty(L.field_backward_scratch_floats(), dtype=torch.float32, device=dev)
    return _scratch[key]


def field_backward(enc: torch.Tensor, dirs: torch.Tensor, weights: torch.Tensor, dL_ddrgb: torch.Tensor,
                   count: Optional[torch.Tensor] = None, grad_scale: Optional[torch.Tensor] = None,
                   dL_denc: Optional[torch.Tensor] = None, dL_dw: Optional[torch.Tensor] = None,
                   accumulate: bool = False, scratch: Optional[torch.Tensor] = None, precision: str = "fp32",
                   loss_scale=None):
    n = enc.shape[0]
    dev = enc.device
    if dL_denc is None:
        dL_denc = torch.empty(n, 32, dtype=enc.dtype, device=dev)
    if dL_dw is None:
        dL_dw = torch.zeros(L.MLP_WEIGHTS, dtype=torch.float32, device=dev)
    if scratch is None:
        scratch = backward_scratch(dev)
    return FieldOps(precision).backward(enc.contiguous(), dirs.contiguous(), weights, dL_ddrgb.contiguous(), count,
                                        grad_scale, scratch, dL_denc, dL_dw, accumulate, loss_scale, n)


class _FieldMlpFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, enc, dirs, weights):
        ctx.save_for_backward(enc, dirs, weights)
        return field_forward(enc, dirs, weights)

    @staticmethod
    def backward(ctx, g):
        enc, dirs, weights = ctx.saved_tensors
        denc, dw = field_backward(enc, dirs, weights, g.contiguous())
        return denc, None, dw


class NGPField(torch.nn.Module):
    """make_nerf_ngp(bound, inference=False) on libngp_gb300."""

    def __init__(self, bound: float, L_levels: int = 16, T: int = 2 ** 19, F: int = 2, N_min: int = 16,
                 N_max: Optional[int] = None, per_level_scale: Optional[float] = None, device="cuda",
                 seed: int = 0):
        super().__init__()
        g = torch.Generator(device=device)
        g.manual_seed(seed)
        self.bound = float(bound)
        self.position_encoder = HashGridEncoder(L_levels, T, F, N_min, N_max if N_max is not None else int(2 ** 11 * bound),
                                                per_level_scale=per_level_scale, device=device, generator=g)
        self.weights = torch.nn.Parameter(pack_weights({k: glorot_uniform(s, g, device) for k, s in SHAPES}))

    def forward(self, xyz: torch.Tensor, dirs: Optional[torch.Tensor]):
        enc, _ = self.position_encoder(xyz, self.bound)
        if dirs is None:
            return field_density(enc, self.weights)
        return _FieldMlpFn.apply(enc, dirs, self.weights)

    # ------------------------------------------------------------------ parameter-tree interchange
    def flax_params(self) -> dict:
        """The reference's parameter tree (nerfs.py names) as NumPy arrays."""
        w = {k: v.detach().cpu().numpy() for k, v in unpack_weights(self.weights.detach()).items()}
        tree = {"position_encoder": {PARAM_NAME: self.position_encoder.latents.detach().cpu().numpy()},
                "density_mlp": {}, "rgb_mlp": {}}
        for k, (mod, dense) in FLAX_NAMES.items():
            tree[mod][dense] = {"kernel": w[k]}
        return tree

    def load_flax_params(self, tree: dict):
        with torch.no_grad():
            lat = torch.as_tensor(np.asarray(tree["position_encoder"][PARAM_NAME]), dtype=torch.float32)
            self.position_encoder.latents.copy_(lat)
            w = {k: torch.as_tensor(np.asarray(tree[mod][dense]["kernel"])) for k, (mod, dense) in FLAX_NAMES.items()}
            self.weights.copy_(pack_weights(w).to(self.weights.device))
