"""The FP64 integrator checker on the GPU (ngp_integrate_rays_fp64): against the CPU FP64
restatement of integrating.cu:24-104 (oracle/adjoint.py), then used to state the float
integrator's error at the training batch size (2^14 rays x 16 samples = 2^18 samples)."""
import numpy as np
import pytest
import torch

from oracle.adjoint import integrate_forward64

pytestmark = pytest.mark.gpu


def ray_batch(rng, R, n):
    """R rays of n samples each, laid out ray after ray: densities spanning transparent to opaque
    (so some rays stop early and some reach the background), the march's step size."""
    sigma = np.exp(rng.normal(2.0, 2.5, size=(R, n))).astype(np.float32)
    rgb = rng.uniform(size=(R, n, 3)).astype(np.float32)
    dt = (2 * np.sqrt(3) / 1024 * rng.uniform(0.5, 1.5, size=(R, n))).astype(np.float32)
    z = (1.0 + np.cumsum(dt, axis=1)).astype(np.float32)
    bg = rng.uniform(size=(R, 3)).astype(np.float32)
    return sigma, rgb, dt, z, bg


def device_inputs(sigma, rgb, dt, z, bg):
    R, n = sigma.shape
    startidx = torch.arange(R, dtype=torch.int32, device="cuda") * n
    ns = torch.full((R,), n, dtype=torch.int32, device="cuda")
    drgbs = torch.from_numpy(np.concatenate([sigma[..., None], rgb], -1).reshape(R * n, 4)).cuda()
    return (startidx, ns, torch.from_numpy(bg).cuda(), torch.from_numpy(dt.reshape(-1)).cuda(),
            torch.from_numpy(z.reshape(-1)).cuda(), drgbs)


def test_fp64_checker_matches_the_cpu_fp64_restatement():
    from jaxngp_gb300.precision import integrate_rays_fp64
    rng = np.random.default_rng(0)
    sigma, rgb, dt, z, bg = ray_batch(rng, 4096, 16)
    out, op, used = integrate_forward64(sigma, rgb, dt, z, bg)
    rgbd, T, n_used = integrate_rays_fp64(*device_inputs(sigma, rgb, dt, z, bg))
    assert np.allclose(rgbd.cpu().numpy(), out, rtol=1e-12, atol=1e-12)
    assert np.allclose(T.cpu().numpy(), 1.0 - op, rtol=1e-12, atol=1e-15)
    assert np.array_equal(n_used.cpu().numpy(), used)
    assert 0.1 < (used < 16).mean() < 0.9   # both early-stopped rays and rays reaching the background


def test_float_integrator_error_at_batch_size():
    """integrate_rays (FP32) against the FP64 checker on 2^18 samples: colour, depth and opacity
    within 1e-6 norm-relative, 1e-5 column-wise, on every ray whose transmittance never passes
    within a factor of two of the 1e-4 stopping threshold (where float and double may stop one
    sample apart, as any two float evaluations may)."""
    from jaxngp_gb300 import volrendjax as vr
    from jaxngp_gb300.precision import integrate_rays_fp64
    rng = np.random.default_rng(1)
    R, n = 1 << 14, 16
    sigma, rgb, dt, z, bg = ray_batch(rng, R, n)
    startidx, ns, bgs, dss, zs, drgbs = device_inputs(sigma, rgb, dt, z, bg)
    _, rgbd32, op32 = vr.integrate_rays(0.0, startidx, ns, bgs, dss, zs, drgbs)
    rgbd64, T64, _ = integrate_rays_fp64(startidx, ns, bgs, dss, zs, drgbs)
    Tk = np.exp(-np.cumsum(sigma.astype(np.float64) * dt.astype(np.float64), axis=1))
    near = (np.abs(np.log(np.maximum(Tk, 1e-300) / 1e-4)) < np.log(2.0)).any(axis=1)
    keep = ~near
    assert keep.mean() > 0.8
    a = rgbd32.cpu().numpy().astype(np.float64)[keep]
    b = rgbd64.cpu().numpy()[keep]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-6
    assert (np.abs(a - b).max(0) / np.abs(b).max(0)).max() <= 1e-5
    o32 = op32.cpu().numpy().astype(np.float64)[keep]
    assert np.abs(o32 - (1.0 - T64.cpu().numpy()[keep])).max() <= 1e-6
