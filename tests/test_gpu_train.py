"""The composed training step (ray batch -> march -> field -> integrate/loss -> backward -> Adam ->
occupancy-grid refresh) on a small blob scene."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_scene():
    from jaxngp_gb300.scene import make_scene_data
    return make_scene_data(n_blobs=16, n_views=12, width=64, height=64, n_steps=1024, seed=3)


def test_scene_ground_truth(small_scene):
    """Ground-truth alpha is high where blobs are and zero in empty corners."""
    rgba = small_scene.rgbas.view(12, 64, 64, 4).float() / 255
    assert rgba[..., 3].max() > 0.9 and rgba[..., 3].min() == 0.0
    assert torch.isfinite(rgba).all()


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_train_loss_decreases(small_scene, precision):
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    tr = NGPTrainer(small_scene, TrainConfig(total_samples=1 << 14, T=1 << 16, seed=1, mlp_precision=precision))
    before = L.lib().ngp_kernel_launches
    before.restype = __import__("ctypes").c_ulonglong
    n0 = before()
    losses, valid = [], []
    for it in range(300):
        st = tr.step()
        if it % 20 == 0 or it >= 280:
            s = st.cpu().numpy()
            losses.append(s[0])
            valid.append(s[1])
    assert np.isfinite(losses).all() and min(valid) > 0
    assert np.mean(losses[-5:]) < 0.5 * losses[0], losses
    assert before() > n0 + 300 * 10
    # occupancy bitfield equals packbits of the density grid at the current threshold
    thr = tr.threshold.item()
    dens = tr.density.cpu().numpy()
    bits = np.packbits(dens > thr, bitorder="little")
    assert np.array_equal(bits, tr.bitfield.cpu().numpy())
    assert 0 < (dens > thr).mean() < 1


@pytest.mark.parametrize("form", ["bf16-mixed", "fp16-mixed"])
def test_train_mixed_precision(small_scene, form):
    """BF16/FP16 MLP with a 16-bit table copy and 16-bit encodings (FP16 under the dynamic loss
    scale): the loss falls as in FP32, the 16-bit copy tracks the FP32 master table exactly, and
    the loss scale rarely has to back off."""
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    prec = form.split("-")[0]
    cfg = TrainConfig(total_samples=1 << 14, T=1 << 16, seed=1, mlp_precision=prec, table_precision=prec,
                      half_activations=True)
    tr = NGPTrainer(small_scene, cfg)
    dt = torch.bfloat16 if prec == "bf16" else torch.float16
    assert tr.enc.dtype == dt and tr.g_enc.dtype == dt and tr.lat_h.dtype == dt
    assert (tr.loss_scale is not None) == (prec == "fp16")
    losses = []
    for it in range(300):
        st = tr.step()
        if it % 20 == 0 or it >= 280:
            losses.append(st.cpu().numpy()[0])
    assert np.isfinite(losses).all()
    # the first step's loss can be small (few rays carry samples before the grid is refreshed):
    # compare with the largest of the early losses
    assert np.mean(losses[-5:]) < 0.5 * max(losses[:3]), losses
    assert torch.equal(tr.lat_h, tr.latents.to(dt))
    if tr.loss_scale is not None:
        s = tr.loss_scale.read()
        assert s["skipped_steps"] <= 3 and s["scale"] >= 2.0 ** 12, s


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_train_with_total_variation(small_scene, prec):
    """TrainConfig.tv_scale > 0 (encoders.py:236-254): the step's loss is the TV-free step's plus the
    TV term of the initial table at the step's whole sample buffer (the oracle's value), and
    training with it stays finite -- under FP16 the TV gradient joins the table's in the loss
    scale's units."""
    from oracle import hashgrid as H
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    # a budget no ray overflows, no jitter, the same pixels: both trainers see the same batch (the
    # table starts at +-1e-4, so a large tv_scale lifts the term far above the loss's float noise)
    kw = dict(total_samples=1 << 18, n_rays=512, T=1 << 16, seed=2, perturb=False, random_bg=False,
              mlp_precision=prec, table_precision=prec, half_activations=prec != "fp32")
    s = 10.0
    perm = torch.randint(0, small_scene.n_pixels, (512,), dtype=torch.int32, device="cuda")
    a, b = NGPTrainer(small_scene, TrainConfig(**kw)), NGPTrainer(small_scene, TrainConfig(tv_scale=s, **kw))
    lat0 = b.latents.detach().cpu().numpy().copy()
    la, lb = a.step(perm).cpu().numpy(), b.step(perm).cpu().numpy()
    tab = H.LevelTable(b.table.L, b.table.T, b.table.F, b.table.N_min, b.table.N_max)
    want = H.total_variation(b.xyzs.cpu().numpy(), lat0, b.bound, tab, s, dtype=np.float64)
    assert abs(float(b.tv) - want) <= 1e-5 * want
    assert abs((float(lb[0]) - float(la[0])) - want) <= 1e-5 * want + 8 * float(np.spacing(la[0]))
    losses = [float(b.step().cpu().numpy()[0]) for _ in range(40)]
    assert np.isfinite(losses).all()


def test_train_step_with_host_perm(small_scene):
    """The step accepts the reference's `perm` (pixel indices); with a sample budget no ray
    overflows, two runs agree up to the order of float atomics (which rays fit an overflowing
    budget depends on the order of the warps' slot atomics, as in the reference)."""
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    cfg = TrainConfig(total_samples=1 << 18, n_rays=512, T=1 << 14, seed=2, perturb=False, random_bg=False)
    perm = torch.randint(0, small_scene.n_pixels, (512,), dtype=torch.int32, device="cuda")
    a = NGPTrainer(small_scene, cfg)
    b = NGPTrainer(small_scene, cfg)
    sa, sb = a.step(perm).clone(), b.step(perm).clone()
    assert torch.allclose(sa, sb, rtol=1e-5, atol=0)
    assert torch.allclose(a.weights, b.weights, rtol=1e-4, atol=1e-7)


def test_render_view(small_scene):
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    tr = NGPTrainer(small_scene, TrainConfig(total_samples=1 << 14, T=1 << 16, seed=1))
    img = tr.render_view(0)
    assert img.shape == (64, 64, 3) and img.dtype == torch.uint8


def test_pipelined_march_matches_serial(small_scene):
    """TrainConfig.pipeline marches the next batch on a second stream while the current step
    trains; the batches are the serial trainer's, ray for ray (the march reads only the
    occupancy grid, which no step between refreshes changes), and the step across a grid refresh
    marches after it.  Losses agree to float-atomics order."""
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    # 64 rays cannot fill a 2^16-sample budget (at most 1024 samples each), so which rays fit does
    # not depend on the order in which concurrent warps allocate (near a full budget it does, in
    # the reference too)
    cfgs = [TrainConfig(total_samples=1 << 16, n_rays=64, T=1 << 16, seed=4, pipeline=p) for p in (False, True)]
    a, b = NGPTrainer(small_scene, cfgs[0]), NGPTrainer(small_scene, cfgs[1])
    assert b.pipeline and not a.pipeline
    for tr in (a, b):
        tr.init_occupancy_analytic()
        tr.cadence_offset = 1009   # refreshes every 16 steps, the first after step 15
    for it in range(24):
        sa, sb = a.step().cpu().numpy(), b.step().cpu().numpy()
        assert sa[3] <= 64 * 1024   # nothing overflowed
        if it < 15:   # before the first refresh both grids are the analytic one
            assert torch.equal(a.valid, b.valid) and torch.equal(a.n_samples, b.n_samples), it
            assert sa[1] == sb[1] and sa[2] == sb[2] and sa[3] == sb[3], (it, sa, sb)
        assert abs(sa[0] - sb[0]) <= 1e-3 * abs(sa[0]) + 1e-7, (it, sa[0], sb[0])
    torch.cuda.synchronize()


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_empty_space_decay_gradient(small_scene, precision):
    """The learned-proposal forms' empty-space term (TrainConfig.empty_space_decay) adds to the
    step's gradients exactly the field backward of decay / M on the density channel at its M
    uniform random points of the box, and that backward's scatter into the table gradient."""
    from jaxngp_gb300.encoders import hashgrid_backward, hashgrid_forward
    from jaxngp_gb300.field import field_backward
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    M, decay = 4096, 1e-3
    cfg = TrainConfig(total_samples=1 << 14, T=1 << 16, seed=1, mlp_precision=precision, sampler="proposal",
                      empty_space_decay=decay, empty_space_points=M)
    tr = NGPTrainer(small_scene, cfg)
    tr.g_w.zero_()
    tr.g_lat.zero_()
    tr._empty_space_decay()
    xyz = tr.empty["xyz"].clone()
    assert bool((xyz.abs() <= tr.bound).all()) and float(xyz.std()) > 0.4 * tr.bound
    enc = hashgrid_forward(tr.table, xyz, tr.gather_table, tr.bound)
    g = torch.zeros(M, 4, device="cuda")
    g[:, 0] = decay / M
    dirs = torch.zeros(M, 3, device="cuda")
    dirs[:, 2] = 1.0
    denc, dw = field_backward(enc, dirs, tr.weights, g, precision=precision)
    glat = hashgrid_backward(tr.table, xyz, denc, tr.bound)
    assert torch.equal(tr.g_w, dw)                       # fixed-order reductions: bit-identical
    torch.testing.assert_close(tr.g_lat, glat, rtol=1e-5, atol=1e-12)   # table atomics reorder sums
    assert float(dw.abs().max()) > 0 and float(glat.abs().max()) > 0
    # a step with the term trains and stays finite
    for _ in range(5):
        st = tr.step()
    assert bool(torch.isfinite(st).all())
