"""NumPy front end of the CPU oracle for the volume-rendering ops.  TEST INFRASTRUCTURE ONLY.

Two CPU back ends sit behind the same functions:

* ``backend="oracle"``: ``oracle/volrend_oracle.c``, a plain-C restatement of the reference's
  kernels (built by ``oracle/Makefile``);
* ``backend="ref"``: the reference's own ``marching.cu``, ``integrating.cu`` and ``packbits.cu``
  compiled for the CPU by ``oracle/build_ref.sh`` (only where the reference checkout exists).

The functions mirror the public API of ``volrendjax`` (deps/volume-rendering-jax/src/volrendjax/
``marching/__init__.py:8-157``, ``integrating/__init__.py:11-110``, ``morton3d/__init__.py:6-10``,
``packbits/__init__.py:8-28``) on NumPy arrays, including the broadcasting those wrappers do.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "liboracle_volrend.so")
_REF_SO = os.path.join(_HERE, "_ref", "libvolrend_ref_cpu.so")

_libs = {}

_P = ctypes.c_void_p
_U = ctypes.c_uint32
_F = ctypes.c_float


def build_oracle() -> str:
    """Compile oracle/volrend_oracle.c (seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _ORACLE_SO


def build_ref(reference_root: str | None = None) -> str:
    """Compile the reference's kernels for the CPU into oracle/_ref/ (oracle/build_ref.sh finds
    the checkout itself unless `reference_root` is given, and builds nothing without one)."""
    subprocess.run([os.path.join(_HERE, "build_ref.sh")] + ([reference_root] if reference_root else []), check=True,
                   stdout=subprocess.DEVNULL)
    return _REF_SO


def ref_available() -> bool:
    return os.path.exists(_REF_SO)


def _lib(backend: str):
    if backend in _libs:
        return _libs[backend]
    if backend == "oracle":
        if not os.path.exists(_ORACLE_SO):
            build_oracle()
        lib = ctypes.CDLL(_ORACLE_SO)
        prefix = "oracle_"
    elif backend == "ref":
        if not os.path.exists(_REF_SO):
            raise FileNotFoundError(f"{_REF_SO} missing; run oracle/build_ref.sh")
        lib = ctypes.CDLL(_REF_SO)
        prefix = "ref_"
    else:
        raise ValueError(backend)
    sigs = {
        "packbits": [_U, _P, _P, _P, _P],
        "morton3d": [_U, _P, _P],
        "morton3d_invert": [_U, _P, _P],
        "march_rays": [_U, _U, _U, _U, _U, _F, _F] + [_P] * 6 + ([_P] * 2 if backend == "ref" else [_P]) + [_P] * 8,
        "march_rays_ex": [_U, _U, _U, _U, _U, _F, _F] + [_P] * 6 + [_P] + [_P] * 8 + [ctypes.c_int],
        "march_rays_inference": [_U, _U, _U, _U, _U, _U, _F, _F] + [_P] * 14,
        "integrate_rays": [_U] + [_P] * 9,
        "integrate_rays_backward": [_U, _F] + [_P] * 12,
        "integrate_rays_inference": [_U, _U, _U] + [_P] * 12,
    }
    fns = {}
    for name, argt in sigs.items():
        if not hasattr(lib, prefix + name):
            continue
        f = getattr(lib, prefix + name)
        f.argtypes = argt
        f.restype = None
        fns[name] = f
    _libs[backend] = fns
    return fns


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


# ------------------------------------------------------------------------------------ packbits

def packbits(density_threshold, density_grid, backend: str = "oracle") -> Tuple[np.ndarray, np.ndarray]:
    """packbits/__init__.py:8-28 + packbits.cu:9-34."""
    grid = _f32(density_grid)
    thr = _f32(np.broadcast_to(np.asarray(density_threshold, np.float32), grid.shape))
    n_bits = grid.shape[0]
    if n_bits % 8:
        raise ValueError("packbits expects a density grid whose size is divisible by 8")
    mask = np.zeros(n_bits, np.uint8)
    bits = np.zeros(n_bits // 8, np.uint8)
    _lib(backend)["packbits"](n_bits // 8, _p(thr), _p(grid), _p(mask), _p(bits))
    return mask.astype(bool), bits


def morton3d(xyzs, backend: str = "oracle") -> np.ndarray:
    """morton3d/__init__.py:6-7 + marching.cu:399-414."""
    xyzs = _u32(xyzs)
    out = np.zeros(xyzs.shape[0], np.uint32)
    _lib(backend)["morton3d"](xyzs.shape[0], _p(xyzs), _p(out))
    return out


def morton3d_invert(idcs, backend: str = "oracle") -> np.ndarray:
    """morton3d/__init__.py:9-10 + marching.cu:416-433."""
    idcs = _u32(idcs)
    out = np.zeros((idcs.shape[0], 3), np.uint32)
    _lib(backend)["morton3d_invert"](idcs.shape[0], _p(idcs), _p(out))
    return out


# ---------------------------------------------------------------------------------- marching

def march_rays(total_samples, diagonal_n_steps, K, G, bound, stepsize_portion, rays_o, rays_d,
               t_starts, t_ends, noises, occupancy_bitfield, backend: str = "oracle",
               return_counters: bool = False, early_exit: bool = True):
    """marching/__init__.py:8-93 + marching.cu:101-268 (ray-order atomics).

    early_exit=True is the reference run one thread at a time (a ray starting after the buffer
    filled is dropped, marching.cu:135); early_exit=False counts every ray before any slot is taken
    (the reference with its whole grid resident; oracle backend only)."""
    rays_o, rays_d = _f32(rays_o), _f32(rays_d)
    n = rays_o.shape[0]
    t_starts, t_ends = _f32(t_starts), _f32(t_ends)
    noises = _f32(np.broadcast_to(np.asarray(noises, np.float32), (n,)))
    bits = np.ascontiguousarray(occupancy_bitfield, dtype=np.uint8)
    assert bits.shape == (K * G * G * G // 8,)
    counters = np.zeros(2, np.uint32)
    valid = np.zeros(n, np.uint8)
    n_samples = np.zeros(n, np.uint32)
    startidx = np.zeros(n, np.uint32)
    idcs = np.zeros(total_samples, np.uint32)
    xyzs = np.zeros((total_samples, 3), np.float32)
    dirs = np.zeros((total_samples, 3), np.float32)
    dss = np.zeros(total_samples, np.float32)
    zs = np.zeros(total_samples, np.float32)
    args = [n, total_samples, diagonal_n_steps, K, G, bound, stepsize_portion, _p(rays_o),
            _p(rays_d), _p(t_starts), _p(t_ends), _p(noises), _p(bits)]
    if backend == "ref":
        if not early_exit:
            raise ValueError("the reference build runs threads one at a time (early_exit=True)")
        args += [_p(counters[0:1]), ctypes.c_void_p(counters.ctypes.data + 4)]
    else:
        args += [_p(counters)]
    args += [_p(valid), _p(n_samples), _p(startidx), _p(idcs), _p(xyzs), _p(dirs), _p(dss), _p(zs)]
    if backend == "oracle" and not early_exit:
        _lib(backend)["march_rays_ex"](*args, 0)
    else:
        _lib(backend)["march_rays"](*args)
    measured = np.uint32(counters[0] - counters[1])
    out = (measured, valid.astype(bool), n_samples, startidx, idcs, xyzs, dirs, dss, zs)
    if return_counters:
        return out, counters
    return out


def march_rays_inference(diagonal_n_steps, K, G, march_steps_cap, bound, stepsize_portion, rays_o,
                         rays_d, t_starts, t_ends, occupancy_bitfield, next_ray_index_in,
                         terminated, indices, backend: str = "oracle"):
    """marching/__init__.py:96-157 + marching.cu:271-397 (slot-order refill).

    Returns (next_ray_index, indices, n_samples, t_starts, xyzs, dss, z_vals) where t_starts is the
    input array with the advanced values scattered back (marching/__init__.py:156)."""
    rays_o, rays_d = _f32(rays_o), _f32(rays_d)
    n_total = rays_o.shape[0]
    t_starts, t_ends = _f32(t_starts), _f32(t_ends)
    bits = np.ascontiguousarray(occupancy_bitfield, dtype=np.uint8)
    term = np.ascontiguousarray(terminated, dtype=np.uint8)
    idx_in = _u32(indices)
    n_rays = term.shape[0]
    cap = march_steps_cap
    nri = np.array([np.asarray(next_ray_index_in).reshape(-1)[0]], np.uint32)
    idx_out = np.zeros(n_rays, np.uint32)
    n_samples = np.zeros(n_rays, np.uint32)
    t_out = np.zeros(n_rays, np.float32)
    xyzs = np.zeros((n_rays, cap, 3), np.float32)
    dss = np.zeros((n_rays, cap), np.float32)
    zs = np.zeros((n_rays, cap), np.float32)
    _lib(backend)["march_rays_inference"](
        n_total, n_rays, diagonal_n_steps, K, G, cap, bound, stepsize_portion, _p(rays_o),
        _p(rays_d), _p(t_starts), _p(t_ends), _p(bits), _p(term), _p(idx_in), _p(nri),
        _p(idx_out), _p(n_samples), _p(t_out), _p(xyzs), _p(dss), _p(zs))
    t_new = t_starts.copy()
    ok = idx_out < n_total
    t_new[idx_out[ok]] = t_out[ok]
    return nri, idx_out, n_samples, t_new, xyzs, dss, zs


# ------------------------------------------------------------------------------- integrating

def integrate_rays(near_distance, rays_sample_startidx, rays_n_samples, bgs, dss, z_vals, drgbs,
                   backend: str = "oracle"):
    """integrating/__init__.py:11-59 + integrating.cu:24-104 (forward only)."""
    startidx, n_samples = _u32(rays_sample_startidx), _u32(rays_n_samples)
    n = startidx.shape[0]
    bgs = _f32(np.broadcast_to(np.asarray(bgs, np.float32), (n, 3)))
    dss, z_vals, drgbs = _f32(dss), _f32(z_vals), _f32(drgbs)
    measured = np.zeros(1, np.uint32)
    rgbds = np.zeros((n, 4), np.float32)
    opac = np.zeros(n, np.float32)
    _lib(backend)["integrate_rays"](n, _p(startidx), _p(n_samples), _p(bgs), _p(dss), _p(z_vals),
                                    _p(drgbs), _p(measured), _p(rgbds), _p(opac))
    return measured[0], rgbds, opac


def integrate_rays_backward(near_distance, rays_sample_startidx, rays_n_samples, bgs, dss, z_vals,
                            drgbs, final_rgbds, final_opacities, dL_dfinal_rgbds,
                            backend: str = "oracle"):
    """integrating/impl.py:109-141 + integrating.cu:106-240.

    Returns (dL_dbgs, dL_dz_vals, dL_ddrgbs)."""
    startidx, n_samples = _u32(rays_sample_startidx), _u32(rays_n_samples)
    n = startidx.shape[0]
    s = np.asarray(dss).shape[0]
    bgs = _f32(np.broadcast_to(np.asarray(bgs, np.float32), (n, 3)))
    dss, z_vals, drgbs = _f32(dss), _f32(z_vals), _f32(drgbs)
    rgbds, opac, g = _f32(final_rgbds), _f32(final_opacities), _f32(dL_dfinal_rgbds)
    g_bgs = np.zeros((n, 3), np.float32)
    g_z = np.zeros(s, np.float32)
    g_c = np.zeros((s, 4), np.float32)
    _lib(backend)["integrate_rays_backward"](
        n, near_distance, _p(startidx), _p(n_samples), _p(bgs), _p(dss), _p(z_vals), _p(drgbs),
        _p(rgbds), _p(opac), _p(g), _p(g_bgs), _p(g_z), _p(g_c))
    return g_bgs, g_z, g_c


def integrate_rays_inference(rays_bg, rays_rgbd, rays_T, n_samples, indices, dss, z_vals, drgbs,
                             backend: str = "oracle"):
    """integrating/__init__.py:62-110 + integrating.cu:242-322.

    Returns (terminate_cnt, terminated, rays_rgbd, rays_T) with the per-slot outputs scattered
    back into the full-size arrays (integrating/__init__.py:108-109)."""
    rays_bg, rays_rgbd, rays_T = _f32(rays_bg), _f32(rays_rgbd), _f32(rays_T)
    n_samples, indices = _u32(n_samples), _u32(indices)
    dss, z_vals, drgbs = _f32(dss), _f32(z_vals), _f32(drgbs)
    n_total = rays_rgbd.shape[0]
    n_rays, cap = dss.shape
    cnt = np.zeros(1, np.uint32)
    term = np.zeros(n_rays, np.uint8)
    rgbd_out = np.zeros((n_rays, 4), np.float32)
    T_out = np.zeros(n_rays, np.float32)
    _lib(backend)["integrate_rays_inference"](
        n_total, n_rays, cap, _p(rays_bg), _p(rays_rgbd), _p(rays_T), _p(n_samples), _p(indices),
        _p(dss), _p(z_vals), _p(drgbs), _p(cnt), _p(term), _p(rgbd_out), _p(T_out))
    new_rgbd, new_T = rays_rgbd.copy(), rays_T.copy()
    ok = indices < n_total
    new_rgbd[indices[ok]] = rgbd_out[ok]
    new_T[indices[ok]] = T_out[ok]
    return cnt[0], term.astype(bool), new_rgbd, new_T
