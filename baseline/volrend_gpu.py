"""ctypes loader of baseline/_ref/libvolrend_ref_gpu.so: the reference's own volume-rendering
kernels (deps/volume-rendering-jax/lib/impl/*.cu) and spherical-harmonics kernel
(deps/spherical-harmonics-encoding-jax/lib/impl/*.cu) built unmodified for sm_103a by
baseline/volrend_gpu.sh.  The GPU tests use it as an oracle and bench.py as the per-kernel bar;
the product (jaxngp_gb300/) never loads it.

The entry points take the reference's XLA custom-call arguments: the buffers in the order of its
lowering rules (deps/volume-rendering-jax/src/volrendjax/*/lowering.py) and the raw bytes of its
descriptor structs (lib/impl/volrend.h:23-118), which are byte-identical to the ones
jaxngp_gb300._lib defines for the drop-in library.
"""
from __future__ import annotations

import ctypes
import os
from typing import Sequence

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libvolrend_ref_gpu.so")
NAMES = ("pack_density_into_bits", "march_rays", "march_rays_inference", "morton3d", "morton3d_invert",
         "integrate_rays", "integrate_rays_backward", "integrate_rays_inference",
         "spherical_harmonics_encoding_cuda_f32")
# the reference's integrators return before a __syncthreads() in a partial last block
# (integrating.cu:45/:100, :263/:318); callers keep n_rays a multiple of their 512-thread block
INTEGRATOR_BLOCK = 512

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError(f"{LIB_PATH} is missing: stage and build it with baseline/volrend_gpu.sh")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.ref_last_error.restype = ctypes.c_char_p
    return _lib


def _ptr(t) -> int:
    if t is None:
        return 0
    if not (t.is_cuda and t.is_contiguous()):
        raise ValueError("buffers must be contiguous CUDA tensors")
    return t.data_ptr()


def call(name: str, buffers: Sequence, desc, stream=None) -> None:
    """volrendjax::<name>(stream, buffers, opaque, opaque_len) of the reference; raises on the
    exception the reference throws."""
    if name not in NAMES:
        raise KeyError(name)
    if name in ("integrate_rays", "integrate_rays_inference"):
        n = desc.n_rays
        if n % INTEGRATOR_BLOCK != 0:
            raise ValueError(f"{name}: n_rays must be a multiple of {INTEGRATOR_BLOCK} for the reference's kernel")
    L = lib()
    if not hasattr(L, "ref_" + name):
        raise RuntimeError(f"the reference's GPU build has no {name}")
    arr = (ctypes.c_void_p * max(1, len(buffers)))(*[_ptr(b) for b in buffers])
    opaque = desc.to_bytes()
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    st = getattr(L, "ref_" + name)(ctypes.c_void_p(stream), arr, ctypes.c_char_p(opaque), ctypes.c_size_t(len(opaque)))
    if st != 0:
        raise RuntimeError(f"reference {name} failed: {L.ref_last_error().decode()}")
