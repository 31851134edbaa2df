"""ctypes binding of libngp_gb300.so and the descriptor structs of include/ngp_gb300.h.

The library is the only compute path: if it is missing, or no CUDA device is present, calls raise
instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os
from typing import Sequence

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libngp_gb300.so")

c_u32 = ctypes.c_uint32
c_u64 = ctypes.c_uint64
c_f32 = ctypes.c_float
MAX_LEVELS = 32
MLP_WEIGHTS = 9408


class NgpError(RuntimeError):
    """A libngp_gb300 entry point returned a non-zero status."""

    def __init__(self, name: str, status: int, message: str):
        super().__init__(f"{name} failed with status {status}: {message}")
        self.status = status


# ----------------------------------------------------------------------------- descriptors

class _Desc(ctypes.Structure):
    def to_bytes(self) -> bytes:
        return ctypes.string_at(ctypes.addressof(self), ctypes.sizeof(self))


class IntegratingDescriptor(_Desc):
    _fields_ = [("n_rays", c_u32), ("total_samples", c_u32)]


class IntegratingBackwardDescriptor(_Desc):
    _fields_ = [("n_rays", c_u32), ("total_samples", c_u32), ("near_distance", c_f32)]


class IntegratingInferenceDescriptor(_Desc):
    _fields_ = [("n_total_rays", c_u32), ("n_rays", c_u32), ("march_steps_cap", c_u32)]


class MarchingDescriptor(_Desc):
    _fields_ = [("n_rays", c_u32), ("total_samples", c_u32), ("diagonal_n_steps", c_u32), ("K", c_u32),
                ("G", c_u32), ("bound", c_f32), ("stepsize_portion", c_f32)]


class MarchingInferenceDescriptor(_Desc):
    _fields_ = [("n_total_rays", c_u32), ("n_rays", c_u32), ("diagonal_n_steps", c_u32), ("K", c_u32),
                ("G", c_u32), ("march_steps_cap", c_u32), ("bound", c_f32), ("stepsize_portion", c_f32)]


class Morton3DDescriptor(_Desc):
    _fields_ = [("length", c_u32)]


class PackbitsDescriptor(_Desc):
    _fields_ = [("n_bytes", c_u32)]


class SphericalHarmonicsEncodingDescriptor(_Desc):
    _fields_ = [("n", c_u32), ("degree", c_u32)]


class NgpHashGridDescriptor(_Desc):
    _fields_ = [("n_coords", c_u32), ("L", c_u32), ("F", c_u32), ("T", c_u32), ("first_hash_level", c_u32),
                ("n_params", c_u32), ("bound", c_f32), ("two_bound", c_f32), ("accumulate", c_u32),
                ("scales", c_f32 * MAX_LEVELS),
                ("resolutions", c_u32 * MAX_LEVELS), ("offsets", c_u32 * (MAX_LEVELS + 1))]


class NgpMlpDescriptor(_Desc):
    _fields_ = [("n_samples", c_u32), ("accumulate", c_u32)]


class NgpTrainRaysDescriptor(_Desc):
    _fields_ = [("n_rays", c_u32), ("width", c_u32), ("height", c_u32), ("n_views", c_u32), ("fx", c_f32),
                ("fy", c_f32), ("cx", c_f32), ("cy", c_f32), ("bound", c_f32), ("perturb", c_u32),
                ("random_bg", c_u32), ("bg", c_f32 * 3), ("seed", c_u64)]


class NgpIntegrateLossDescriptor(_Desc):
    _fields_ = [("n_rays", c_u32), ("total_samples", c_u32), ("near_distance", c_f32), ("huber_delta", c_f32)]


class NgpAdamDescriptor(_Desc):
    _fields_ = [("n", c_u32), ("step", c_u32), ("lr", c_f32), ("beta1", c_f32), ("beta2", c_f32), ("eps", c_f32),
                ("eps_root", c_f32), ("weight_decay", c_f32), ("zero_grad", c_u32)]


class NgpProposalDescriptor(_Desc):
    _fields_ = [("n", c_u32), ("total_samples", c_u32), ("G", c_u32), ("bound", c_f32), ("perturb", c_u32),
                ("seed_lo", c_u32), ("seed_hi", c_u32), ("count_index", c_u32), ("sigma_stride", c_u32),
                ("samples_per_ray", c_u32), ("mix", c_f32)]


class NgpOgridDescriptor(_Desc):
    _fields_ = [("K", c_u32), ("G", c_u32), ("cascade", c_u32), ("n_points", c_u32), ("update_all", c_u32),
                ("bound", c_f32), ("decay", c_f32), ("threshold_step", c_f32), ("seed", c_u64),
                ("n_views", c_u32), ("width", c_u32), ("height", c_u32), ("fx", c_f32), ("fy", c_f32),
                ("cx", c_f32), ("cy", c_f32)]


class NgpRenderBlobsDescriptor(_Desc):
    _fields_ = [("n_rays", c_u32), ("n_blobs", c_u32), ("n_steps", c_u32), ("width", c_u32), ("height", c_u32),
                ("n_views", c_u32), ("view0", c_u32), ("n_shells", c_u32), ("fx", c_f32), ("fy", c_f32),
                ("cx", c_f32), ("cy", c_f32), ("bound", c_f32)]


DTYPE_F32, DTYPE_BF16, DTYPE_F16 = 0, 1, 2


class NgpLossScaleDescriptor(_Desc):
    _fields_ = [("growth_factor", c_f32), ("backoff_factor", c_f32), ("growth_interval", c_u32), ("max_scale", c_f32),
                ("min_scale", c_f32)]


class NgpFieldMixedDescriptor(_Desc):
    _fields_ = [("n_samples", c_u32), ("accumulate", c_u32), ("operand", c_u32), ("activations", c_u32)]


class NgpHashGridMixedDescriptor(_Desc):
    _fields_ = [("grid", NgpHashGridDescriptor), ("table", c_u32), ("encodings", c_u32)]


class NgpHashGridTVDescriptor(_Desc):
    _fields_ = [("grid", NgpHashGridDescriptor), ("tv_scale", c_f32), ("with_grad", c_u32)]


class NgpAdamMixedDescriptor(_Desc):
    _fields_ = [("adam", NgpAdamDescriptor), ("half_copy", c_u32)]


# ------------------------------------------------------------------------------------ loading

_lib = None


def lib() -> ctypes.CDLL:
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: build it with `python -m jaxngp_gb300.build`")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.ngp_last_status_message.restype = ctypes.c_char_p
        _lib.ngp_field_backward_scratch_floats.restype = ctypes.c_size_t
    return _lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("libngp_gb300 needs a CUDA device; there is no CPU fallback")


def _ptr(t) -> int:
    if t is None:
        return 0
    if isinstance(t, int):
        return t
    if not t.is_cuda:
        raise ValueError("all buffers must be CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("all buffers must be contiguous")
    return t.data_ptr()


def call(name: str, buffers: Sequence, desc: _Desc | None = None, stream=None) -> None:
    """Invoke `name_status(stream, buffers, opaque, len)`; raise NgpError on a non-zero status."""
    require_cuda()
    L = lib()
    arr = (ctypes.c_void_p * max(1, len(buffers)))(*[_ptr(b) for b in buffers])
    opaque = desc.to_bytes() if desc is not None else b""
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    fn = getattr(L, name + "_status")
    st = fn(ctypes.c_void_p(stream), arr, ctypes.c_char_p(opaque), ctypes.c_size_t(len(opaque)))
    if st != 0:
        raise NgpError(name, st, L.ngp_last_status_message().decode())


def proposal_backward_scratch_floats() -> int:
    lib().ngp_proposal_backward_scratch_floats.restype = ctypes.c_size_t
    return int(lib().ngp_proposal_backward_scratch_floats())


def field_backward_scratch_floats() -> int:
    require_cuda()
    return int(lib().ngp_field_backward_scratch_floats())
