"""The device-resident inference renderer against the reference's host render loop
(models/renderers/cuda.py:318-361) composed from the drop-in ops, whose march and integrate
kernels are themselves checked against the oracle in test_gpu_volrend.py."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    from jaxngp_gb300.scene import make_scene_data
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    data = make_scene_data(n_blobs=16, n_views=8, width=96, height=72, n_steps=1024, seed=5)
    tr = NGPTrainer(data, TrainConfig(total_samples=1 << 16, T=1 << 16, seed=4))
    tr.init_occupancy_analytic(steady_state=False)
    for _ in range(150):
        tr.step()
    torch.cuda.synchronize()
    return tr


def host_loop(tr, o, d, t0, t1, bg, n_slots, cap):
    """The reference's render loop: march_rays_inference -> field on every slot ->
    integrate_rays_inference, with the scatters done by the drop-in wrappers."""
    from jaxngp_gb300 import volrendjax as vr
    from jaxngp_gb300.encoders import hashgrid_forward
    from jaxngp_gb300.field import field_forward
    N = o.shape[0]
    dev = o.device
    rgbd = torch.zeros(N, 4, device=dev)
    T = torch.ones(N, device=dev)
    t_starts = t0.clone()
    nri = torch.zeros(1, dtype=torch.int32, device=dev)
    term = torch.ones(n_slots, dtype=torch.bool, device=dev)
    idx = torch.zeros(n_slots, dtype=torch.int32, device=dev)
    done, it = 0, 0
    while done < N:
        nri, idx, ns, t_starts, xyzs, dss, zs = vr.march_rays_inference(
            tr.cfg.diagonal_n_steps, tr.K, tr.cfg.G, cap, tr.bound, tr.sp, o, d, t_starts, t1, tr.bitfield,
            nri, term, idx)
        ii = idx.long().clamp(max=N - 1)
        dirs = d[ii][:, None, :].expand(n_slots, cap, 3).reshape(-1, 3)
        enc = hashgrid_forward(tr.table, xyzs.view(-1, 3), tr.latents, tr.bound)
        drgbs = field_forward(enc, dirs, tr.weights).view(n_slots, cap, 4)
        cnt, term, rgbd, T = vr.integrate_rays_inference(bg, rgbd, T, ns, idx, dss, zs, drgbs)
        done += int(cnt)
        it += 1
        assert it < 100000
    return rgbd, it


@pytest.mark.parametrize("compact", [False, True])
@pytest.mark.parametrize("n_slots,cap", [(512, 8), (4096, 8), (1000, 3)])
def test_renderer_matches_host_loop(trained, n_slots, cap, compact):
    from jaxngp_gb300.renderer import Renderer
    from jaxngp_gb300.trainer import camera_rays, near_far
    tr = trained
    o, d = camera_rays(tr.data.camera, tr.data.transforms[3])
    t0, t1 = near_far(tr.bound, o, d)
    bg = torch.rand(o.shape[0], 3, device=o.device, generator=torch.Generator(o.device).manual_seed(7))
    want, _ = host_loop(tr, o, d, t0, t1, bg, n_slots, cap)
    r = Renderer.from_trainer(tr, n_slots=n_slots, march_steps_cap=cap, poll_every=3, compact=compact)
    got, iters = r.render_rays(o, d, t0.clone(), t1, bg)
    torch.cuda.synchronize()
    assert iters > 0
    # every ray's march and compositing is independent of which slot, iteration and (compact)
    # sample position carry it
    assert torch.equal(got, want), (got - want).abs().max()
    assert torch.isfinite(got).all()
    # some rays terminate on opacity, some reach the far plane and show the background
    assert 0.0 < float((got[:, 3] > 0).float().mean()) < 1.0


def test_render_image_close_to_training_renderer(trained):
    """The in-place renderer and the training-style renderer (march_rays without jitter, no
    early termination) draw the same image up to the transmittance cut-off."""
    from jaxngp_gb300.renderer import Renderer
    tr = trained
    cam = tr.data.camera
    r = Renderer.from_trainer(tr, n_slots=1 << 14)
    rgb, depth = r.render_image(cam, tr.data.transforms[1])
    ref = tr.render_view(1)
    torch.cuda.synchronize()
    assert rgb.shape == (cam.height, cam.width, 3) and depth.shape == (cam.height, cam.width)
    diff = (rgb.int() - ref.int()).abs().float()
    # the training march has no far-plane sample and composites the background under T <= 1e-4
    assert float((diff <= 2).float().mean()) > 0.99 and float(diff.mean()) < 0.5, (diff.max(), diff.mean())
    assert torch.isfinite(depth).all()


def test_renderer_empty_grid(trained):
    """With an empty occupancy grid every ray terminates on its first iteration and shows its
    background."""
    from jaxngp_gb300.renderer import Renderer
    from jaxngp_gb300.trainer import camera_rays, near_far
    tr = trained
    o, d = camera_rays(tr.data.camera, tr.data.transforms[0])
    t0, t1 = near_far(tr.bound, o, d)
    bg = torch.rand(o.shape[0], 3, device=o.device)
    empty = torch.zeros_like(tr.bitfield)
    r = Renderer(tr.latents, tr.weights, tr.table, empty, tr.K, tr.cfg.G, tr.bound, tr.sp,
                 tr.cfg.diagonal_n_steps, n_slots=o.shape[0], poll_every=1)
    got, iters = r.render_rays(o, d, t0.clone(), t1, bg)
    assert iters == 1
    assert torch.equal(got[:, :3], bg) and torch.equal(got[:, 3], torch.zeros_like(got[:, 3]))


def test_compact_march_packs_samples(trained):
    """The compact march writes each slot's samples contiguously from sample_start, the ranges
    tile [0, sample_count) without gaps, and positions equal the strided march's."""
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.trainer import camera_rays, near_far
    tr = trained
    o, d = camera_rays(tr.data.camera, tr.data.transforms[2])
    t0, t1 = near_far(tr.bound, o, d)
    N, n, cap = o.shape[0], 3000, 8
    i32 = dict(dtype=torch.int32, device="cuda")
    dm = L.MarchingInferenceDescriptor(N, n, tr.cfg.diagonal_n_steps, tr.K, tr.cfg.G, cap, tr.bound, tr.sp)

    def run(compact):
        ts = t0.clone()
        term = torch.ones(n, dtype=torch.bool, device="cuda")
        idx, nri, ns = torch.zeros(n, **i32), torch.zeros(1, **i32), torch.zeros(n, **i32)
        xyz, dirs = torch.zeros(n * cap, 3, device="cuda"), torch.zeros(n * cap, 3, device="cuda")
        dss, zs = torch.zeros(n, cap, device="cuda"), torch.zeros(n, cap, device="cuda")
        if compact:
            start, cnt = torch.zeros(n, **i32), torch.zeros(1, **i32)
            L.call("ngp_march_rays_inference_compact",
                   [o, d, ts, t1, tr.bitfield, term, idx, nri, ns, start, cnt, xyz, dirs, dss, zs], dm)
            return ts, idx, ns, xyz, dirs, dss, zs, start, cnt
        L.call("ngp_march_rays_inference_inplace", [o, d, ts, t1, tr.bitfield, term, idx, nri, ns, xyz, dirs, dss, zs],
               dm)
        return ts, idx, ns, xyz, dirs, dss, zs

    a, b = run(False), run(True)
    # which slot takes which ray follows the order of the warps' atomics: compare per ray
    assert torch.equal(a[0], b[0])  # advanced t of every ray
    ia, ib = a[1].long().cpu(), b[1].long().cpu()
    assert torch.equal(torch.sort(ia).values, torch.sort(ib).values)
    pa, pb = torch.empty(N, dtype=torch.long), torch.empty(N, dtype=torch.long)
    pa[ia], pb[ib] = torch.arange(n), torch.arange(n)   # ray -> slot
    rays = ia
    for k in (2, 5, 6):  # n_samples, dss, z_vals
        assert torch.equal(a[k].cpu()[pa[rays]], b[k].cpu()[pb[rays]])
    ns, start, cnt = b[2].long().cpu(), b[7].long().cpu(), int(b[8])
    assert cnt == int(ns.sum()) and cnt > 0
    cover = torch.zeros(cnt, dtype=torch.int32)
    for i in torch.nonzero(ns).flatten().tolist():
        cover[start[i]:start[i] + ns[i]] += 1
    assert (cover == 1).all()
    xa, da = a[3].view(n, cap, 3).cpu(), a[4].view(n, cap, 3).cpu()
    xb, db = b[3].cpu(), b[4].cpu()
    for r in rays[::97].tolist():
        i, j = int(pa[r]), int(pb[r])
        k = int(ns[j])
        assert torch.equal(xb[start[j]:start[j] + k], xa[i, :k])
        assert torch.equal(db[start[j]:start[j] + k], da[i, :k])
