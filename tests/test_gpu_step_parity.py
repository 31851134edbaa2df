"""One composed training step on the GPU (NGPTrainer.step) against the CPU restatement of the
reference's step, from identical state, and the step's occupancy-grid refresh and optimiser
against restatements of the reference's.

The reference's step (app/nerf/_utils.py:80-170, models/renderers/cuda.py:100-162): rays from the
pixel indices `perm` (_utils.py:93-115, utils/types.py:417-439), near/far from the AABB
(renderers/cuda.py:56-97), jittered starts, a random background per ray, the target blended over
it (utils/data.py:443-465), march_rays -> field -> integrate_rays, the Huber loss (delta 0.1)
averaged over the colour channels and over the valid rays, value_and_grad, and the optax chain of
_utils.py:19-77.  The GPU draws the jitter and the background with its own counter-based RNG (the
reference draws them with jax.random); the CPU side takes the values the GPU drew and everything
else from the restatements in oracle/.

Bars:
* rays, near/far, target blend: within 1e-6 (unit directions absolutely, distances relatively);
* ray validity, per-ray sample counts and per-ray sample sequences: bit-exact;
* encodings: bit-exact; field outputs: 1e-5 of each column's scale against FP64;
* loss: 1e-5 relative; dL/ddrgbs: 1e-5 of each column's scale, plus the float32 uncertainty of
  the loss residual (pred - gt) propagated to each sample, on rays away from the T = 1e-4 stopping
  threshold;
* dL/dW and dL/dlatents: 1e-5 of each matrix's scale against FP64 sums with FP64 ReLU decisions,
  plus, per element, what the decisions within float32-accurate rounding of a kink can move (every
  pre-activation within 1e-6 of its terms' absolute sum, flipped one at a time in FP64: the field
  kernels evaluate each layer to FP32 accuracy on the tensor cores, whose pre-activations no
  float32 restatement reproduces to the bit);
* the parameter update: the optax chain on the step's own gradients, 1e-6 relative.
"""
import numpy as np
import pytest
import torch

from oracle import field as Fd
from oracle import hashgrid as H
from oracle import ogrid as OG
from oracle import optim as OP
from oracle import train_step as TS
from oracle import volrend as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    from jaxngp_gb300.scene import make_scene_data
    return make_scene_data(n_blobs=16, n_views=12, width=64, height=64, n_steps=1024, seed=3)


def cpu_scene(data):
    c = data.camera
    return TS.CpuScene(c.width, c.height, c.fx, c.fy, c.cx, c.cy, data.transforms.cpu().numpy(), data.bound, c.near)


def h(t):
    a = t.detach().cpu().numpy()
    return a.view(np.uint32) if a.dtype == np.int32 else a


def col_err(a, b, mask=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    if a.size == 0:
        return 0.0
    scale = np.abs(b).max(axis=0) if b.ndim > 1 else np.abs(b).max()
    return float((np.abs(a - b).max(axis=0) / np.maximum(scale, 1e-30)).max())


def mat_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


class Spy:
    """Wraps jaxngp_gb300._lib.call for the duration of a step and keeps copies of what the
    optimiser reads and writes (Adam zeroes the gradients it consumes)."""

    def __init__(self, tr):
        from jaxngp_gb300 import _lib as L
        self.L, self.tr, self.rec, self.names = L, tr, {}, []

    def __enter__(self):
        self.orig = self.L.call

        def spy(name, buffers, desc=None, stream=None):
            self.names.append(name)
            key = None
            if name == "ngp_adam":
                key = "lat" if buffers[0].data_ptr() == self.tr.latents.data_ptr() else "w"
                self.rec[key + "_in"] = [b.clone() for b in buffers]
                self.rec[key + "_desc"] = desc
            self.orig(name, buffers, desc, stream)
            if key is not None:
                self.rec[key + "_out"] = [b.clone() for b in buffers]
        self.L.call = spy
        return self

    def __exit__(self, *a):
        self.L.call = self.orig


def test_train_step_matches_cpu_restatement(scene):
    from jaxngp_gb300.field import unpack_weights
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig, lr_at
    # a budget no ray overflows (1024 rays x at most 1024 samples), jitter and random background on
    cfg = TrainConfig(total_samples=1 << 20, n_rays=1024, T=1 << 16, seed=5)
    tr = NGPTrainer(scene, cfg)
    tr.init_occupancy_analytic()
    # a trained field: densities of a fresh one are all near 1, where alpha = 1 - exp(-sigma ds) of
    # float32 carries a relative error of ulp(1) / (sigma ds) ~ 2e-5 in any float32 evaluation (the
    # reference's included); trained densities put the gradient's scale on samples where it is small
    for _ in range(300):
        tr.step()
    while tr.ogrid_due(tr.step_count + 1 + tr.cadence_offset):   # no grid refresh inside the step
        tr.step()
    torch.cuda.synchronize()
    lat0 = h(tr.latents).copy()
    w0 = {k: v.detach().cpu().numpy().copy() for k, v in unpack_weights(tr.weights).items()}
    bits = h(tr.bitfield).copy()
    count0 = tr.step_count
    perm = torch.randint(0, scene.n_pixels, (cfg.n_rays,), dtype=torch.int32, device="cuda",
                         generator=torch.Generator(device="cuda").manual_seed(9))
    with Spy(tr) as spy:
        stats = h(tr.step(perm)).copy()
    torch.cuda.synchronize()
    assert spy.names[:2] == ["ngp_train_rays", "ngp_march_rays_train"]

    # ---- ray batch (_utils.py:93-115, renderers/cuda.py:56-97, data.py:443-465)
    sc = cpu_scene(scene)
    pm = h(perm).astype(np.int64)
    o, d = TS.rays_from_pixels(sc, pm)
    t0, t1 = TS.near_far(sc.bound, o, d)
    o_g, d_g, t0_g, t1_g = h(tr.rays_o), h(tr.rays_d), h(tr.t0), h(tr.t1)
    noise, bgs, gt_g = h(tr.noise), h(tr.bgs), h(tr.gt)
    assert np.array_equal(o_g, o)
    assert np.abs(d_g - d).max() <= 1e-6
    # near/far of rays that cross the box (a ray that misses it has t_start >= t_end either way; its
    # distances to the planes of faces it runs almost parallel to are ill-conditioned)
    hit = t1 > t0
    assert np.array_equal(t1_g > t0_g, hit) and hit.mean() > 0.5
    assert np.abs(t0_g - t0)[hit].max() <= 1e-6 * np.abs(t0[hit]).max()
    assert np.abs(t1_g - t1)[hit].max() <= 1e-6 * np.abs(t1[hit]).max()
    assert noise.min() >= 0 and noise.max() < 1 and bgs.min() >= 0 and bgs.max() < 1
    assert noise.std() > 0.2 and bgs.std() > 0.2   # drawn, not constant
    rgba = h(scene.rgbas)[pm].astype(np.float32) / np.float32(255)
    gt = rgba[:, :3] * rgba[:, 3:] + bgs * (np.float32(1) - rgba[:, 3:])
    assert np.abs(gt_g - gt).max() <= 1e-6

    # ---- march (bit-exact, per ray) on the GPU's rays
    G = cfg.G
    m, valid, ns, st, idcs, xyzs, dirs, dss, zs = V.march_rays(tr.S, cfg.diagonal_n_steps, 1, G, tr.bound, 0.0, o_g, d_g,
                                                                t0_g, t1_g, noise, bits, early_exit=True)
    valid_g, ns_g, st_g = h(tr.valid), h(tr.n_samples), h(tr.startidx)
    nv = int(valid.sum())
    assert np.array_equal(valid_g, valid) and np.array_equal(ns_g, ns)
    used = int(m)
    assert int(stats[3]) == used and int(ns.sum()) == used and 0 < used < tr.S
    xyz_g, dirs_g, dss_g, zs_g = h(tr.xyzs), h(tr.dirs), h(tr.dss), h(tr.z_vals)
    order_g = np.concatenate([np.arange(st_g[r], st_g[r] + ns_g[r]) for r in np.nonzero(ns_g)[0]])
    order_c = np.concatenate([np.arange(st[r], st[r] + ns[r]) for r in np.nonzero(ns)[0]])
    for a, b in ((xyz_g, xyzs), (dirs_g, dirs), (dss_g, dss), (zs_g, zs)):
        assert np.array_equal(a[order_g], b[order_c])

    # ---- encoder (bit-exact) and field forward
    tab = H.LevelTable(tr.table.L, tr.table.T, tr.table.F, tr.table.N_min, tr.table.N_max)
    enc = H.encode(xyz_g[:used], lat0, tr.bound, tab)
    assert np.array_equal(h(tr.enc)[:used], enc)
    drgb_g = h(tr.drgbs)[:used]
    drgb64, _ = Fd.forward(enc, dirs_g[:used], w0, dtype=np.float64)
    assert col_err(drgb_g, drgb64) <= 1e-5
    # a float32 evaluation of the field (explicit FMA chains): the forward kernel (three BF16 pieces
    # per operand on the tensor cores, FP32 accumulation) is another float32 evaluation of the
    # same layers, a few ulps away in each layer's sum
    drgb32, cache = Fd.forward_fma32(enc, dirs_g[:used], w0)
    e32 = col_err(drgb_g, drgb32)
    assert e32 <= 5e-6
    print(f"\nstep parity: {cfg.n_rays} rays, {used} samples, {nv} valid rays; field outputs {col_err(drgb_g, drgb64):.2e} "
          f"from FP64 and {e32:.2e} from the float32 FMA-chain evaluation (column scale)")

    # ---- integrate + masked Huber loss + integrate backward (on the GPU's field values)
    drgbs_full = np.zeros((tr.S, 4), np.float32)
    drgbs_full[:used] = drgb_g
    meas, rgbd, opac = V.integrate_rays(sc.near, st_g, ns_g, bgs, dss_g, zs_g, drgbs_full)
    e = rgbd[:, :3].astype(np.float64) - gt
    ae = np.abs(e)
    delta = 0.1
    huber = np.where(ae <= delta, 0.5 * e * e, delta * (ae - 0.5 * delta)).mean(-1)
    loss = float(np.where(valid, huber, 0.0).sum() / nv)
    assert int(stats[1]) == nv and int(stats[2]) == int(meas)
    assert abs(float(stats[0]) - loss) <= 1e-5 * loss
    g = (np.where(ae <= delta, e, delta * np.sign(e)) / 3.0 / nv) * valid[:, None]
    gs = float(h(tr.grad_scale)[0])
    assert abs(gs - 1.0 / nv) <= 1e-6 / nv
    g_drgbs_g = h(tr.g_drgbs)[:used].astype(np.float64) * gs
    # The per-ray loss gradient (pred - gt) / (3 n_valid) (Huber's quadratic zone) is ill-conditioned
    # once the field fits: the prediction's float32 summation error (two orders of summation of at
    # most n + 4 terms of total size <= 2 differ by up to 4 (n + 4) ulps) is large against a small
    # residual.  That uncertainty is propagated to each sample's gradient -- dL/dc_k = w_k g_c and
    # |d(dL/dsigma_k) / dg_c| <= 3 ds_k -- and added to the 1e-5 bar; rays within 1e-5 of Huber's
    # kink are left out.
    g4 = np.concatenate([g, np.zeros((len(g), 1))], -1).astype(np.float32)
    kink = (np.abs(ae - delta) <= 1e-5).any(-1)
    dg = np.where(ae <= delta, 4.0 * (ns_g[:, None].astype(np.float64) + 4) * 2.0 ** -24 *
                  np.maximum(np.abs(rgbd[:, :3]), 1.0) / (3.0 * nv), 0.0)
    _, _, g_drgbs = V.integrate_rays_backward(sc.near, st_g, ns_g, bgs, dss_g, zs_g, drgbs_full, rgbd, opac, g4)
    # both sides are in the GPU's slot layout (the oracle integrated the GPU's buffers); rays whose
    # transmittance before some sample lies within rounding of the 1e-4 stopping threshold are left
    # out (the two evaluations may disagree on whether that sample counts)
    T = 1.0 - opac.astype(np.float64)
    ok_ray = (np.abs(T / 1e-4 - 1.0) > 1e-2) & ~near_stop(st_g, ns_g, dss_g, drgbs_full) & ~kink
    assert ok_ray.mean() > 0.95
    msk = ok_s_mask(st_g, ns_g, ok_ray, used)
    ray_of = np.zeros(used, np.int64)
    for r in np.nonzero(ns_g)[0]:
        ray_of[st_g[r]:st_g[r] + ns_g[r]] = r
    w64 = sample_weights(st_g, ns_g, dss_g, drgbs_full)[:used]
    b64 = g_drgbs[:used].astype(np.float64)
    scale = np.abs(b64[msk]).max(0)
    tol = 1e-5 * scale[None, :] + np.concatenate(
        [(3.0 * dss_g[:used] * dg[ray_of].sum(-1))[:, None], w64[:, None] * dg[ray_of]], -1)
    over = (np.abs(g_drgbs_g - b64) > tol) & msk[:, None]
    print(f"dL/ddrgbs vs oracle: {col_err(g_drgbs_g, b64, mask=msk):.2e} of the column scale "
          f"(bar 1e-5 plus the residual's propagated float32 uncertainty); samples over the bar {int(over.sum())}")
    assert not over.any()

    # ---- field backward (FP64, FP64 ReLU decisions, plus what decisions at a kink can move) and
    # table scatter
    _, cache64 = Fd.forward(enc, dirs_g[:used], w0, dtype=np.float64)
    denc64, gw64 = Fd.backward(g_drgbs_g, cache64, w0, dtype=np.float64)
    tol_w, tol_enc, n_near = Fd.kink_flip_tolerance(g_drgbs_g, cache64, w0)
    gw_g = {k: v.cpu().numpy() for k, v in unpack_weights(spy.rec["w_in"][1]).items()}
    print(f"dL/dW vs FP64: {max(mat_err(gw_g[k], gw64[k]) for k in gw64):.2e} of the matrix scale; "
          f"{n_near} pre-activations within 1e-6 of a kink")
    for k in gw64:
        over = np.abs(gw_g[k] - gw64[k]) > 1e-5 * np.abs(gw64[k]).max() + tol_w[k]
        assert not over.any(), (k, mat_err(gw_g[k], gw64[k]), int(over.sum()))
    glat64 = H.encode_backward(xyz_g[:used], denc64, tr.bound, tab, dtype=np.float64)
    tol_lat = H.encode_backward(xyz_g[:used], tol_enc, tr.bound, tab, dtype=np.float64)   # weights >= 0
    glat_g = h(spy.rec["lat_in"][1])
    over = np.abs(glat_g - glat64) > 1e-5 * np.abs(glat64).max() + tol_lat
    assert not over.any(), (mat_err(glat_g, glat64), int(over.sum()))

    # ---- optimiser: the optax chain on the step's own gradients
    lr = OP.reference_lr(count0, cfg.lr)
    assert abs(lr_at(cfg.lr, count0) - lr) <= 1e-7 * lr
    for key, wd in (("lat", 0.0), ("w", 1e-6)):
        p, gg, mm, vv = (h(x) for x in spy.rec[key + "_in"])
        desc = spy.rec[key + "_desc"]
        assert desc.step == count0 + 1 and abs(desc.weight_decay - wd) <= 1e-12
        p1, m1, v1 = OP.adam_update(p, gg, mm, vv, count0, lr, weight_decay=wd)
        po, go, mo, vo = (h(x) for x in spy.rec[key + "_out"])
        assert not go.any()   # the step zeroes the gradient it consumed
        assert np.all(np.abs(po - p1) <= 1e-6 * (np.abs(p1) + lr)), key
        assert np.all(np.abs(mo - m1) <= 1e-6 * np.abs(m1) + 1e-30), key
        assert np.all(np.abs(vo - v1) <= 1e-6 * np.abs(v1) + 1e-30), key


def sample_weights(st, ns, dss, drgbs):
    """Per sample (buffer layout), the compositing weight T_k alpha_k in FP64."""
    w = np.zeros(len(dss))
    for r in np.nonzero(ns)[0]:
        a, b = int(st[r]), int(st[r]) + int(ns[r])
        x = drgbs[a:b, 0].astype(np.float64) * dss[a:b]
        T = np.exp(-np.concatenate([[0.0], np.cumsum(x)[:-1]]))
        w[a:b] = T * -np.expm1(-x)
    return w


def near_stop(st, ns, dss, drgbs, rel=1e-3):
    """Rays whose transmittance before one of their samples is within `rel` of 1e-4 (FP64)."""
    out = np.zeros(len(ns), bool)
    for r in np.nonzero(ns)[0]:
        a, b = int(st[r]), int(st[r]) + int(ns[r])
        x = drgbs[a:b, 0].astype(np.float64) * dss[a:b]
        T = np.exp(-np.concatenate([[0.0], np.cumsum(x)[:-1]]))
        out[r] = bool(np.any(np.abs(T / 1e-4 - 1.0) <= rel))
    return out


def ok_s_mask(st, ns, ok_ray, used):
    """Samples [0, used) of the GPU's buffer that belong to rays away from the stopping threshold."""
    m = np.zeros(used, bool)
    for r in np.nonzero(ok_ray & (ns > 0))[0]:
        m[st[r]:st[r] + ns[r]] = True
    return m


def test_ogrid_refresh_matches_reference_restatement(scene):
    """update_ogrid_density + threshold_ogrid (utils/types.py:1149-1239) step by step on the
    trainer's own grid: decay and max bit-exact, the sampled cells and jittered points where the
    reference puts them, the density query within 1e-5 of FP64, the threshold min(0.01 * diag /
    (2 min(bound,1) sqrt3), mean live density) within 1e-5, and the bitfield bit-exact."""
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.field import unpack_weights
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    cfg = TrainConfig(total_samples=1 << 16, n_rays=1024, T=1 << 16, seed=6)
    tr = NGPTrainer(scene, cfg)
    tr.init_occupancy_analytic()
    for _ in range(5):
        tr.step()
    torch.cuda.synchronize()
    G, G3, bound = cfg.G, cfg.G ** 3, tr.bound
    tab = H.LevelTable(tr.table.L, tr.table.T, tr.table.F, tr.table.N_min, tr.table.N_max)
    lat = h(tr.latents)
    w = {k: v.detach().cpu().numpy() for k, v in unpack_weights(tr.weights).items()}
    for update_all in (False, True):
        dens0, bits0 = h(tr.density).copy(), h(tr.bitfield).copy()
        alive = dens0 >= 0
        occ = np.unpackbits(bits0, bitorder="little").astype(bool)
        assert 0 < alive.mean() and 0 < (occ & alive).mean() < alive.mean()
        M = G3 if update_all else max(1, int(alive.sum()) // 2)
        d = tr._ogrid_desc(0, M, update_all, 1234 + int(update_all))
        L.call("ngp_ogrid_decay", [tr.density], d)
        dens1 = h(tr.density).copy()
        assert np.array_equal(dens1, OG.decay(dens0, 0, G))
        cells = torch.empty(M, dtype=torch.int32, device="cuda")
        xyz = torch.empty(M, 3, device="cuda")
        L.call("ngp_ogrid_sample", [tr.density, tr.bitfield, cells, xyz], d)
        c, x = h(cells), h(xyz)
        if update_all:   # every cell once; cells marked untrainable are skipped
            assert np.array_equal(c[alive], np.nonzero(alive)[0]) and (c[~alive] == 0xFFFFFFFF).all()
            live = alive
        else:            # M/2 cells uniform among the live ones, M/2 among the live occupied ones
            assert (c < G3).all() and alive[c].all()
            assert occ[c[M // 2:]].mean() > 0.99
            share = (occ & alive).sum() / alive.sum()
            assert abs(occ[c[:M // 2]].mean() - share) < 0.02
            live = np.ones(M, bool)
        base, hcw = OG.cell_points_base(c[live], 0, G, bound)
        assert np.all(np.abs(x[live] - base) <= hcw * (1 + 1e-5))
        sigma = torch.empty(M, device="cuda")
        for s in range(0, M, tr.S):
            n = min(tr.S, M - s)
            tr._encode(xyz[s:s + n], None, tr.enc[:n], n)
            tr.field.density(tr.enc[:n], tr.weights, sigma[s:s + n], n)
        sg = h(sigma)
        pick = np.nonzero(live)[0][:: max(1, int(live.sum()) // 20000)]
        sig64 = Fd.density_only(H.encode(x[pick], lat, bound, tab), w, dtype=np.float64)
        assert col_err(sg[pick], sig64) <= 1e-5
        L.call("ngp_ogrid_max", [cells, sigma, tr.density], d)
        dens2 = h(tr.density).copy()
        assert np.array_equal(dens2, OG.max_update(dens1, 0, G, c[live], sg[live]))
        L.call("ngp_ogrid_threshold", [tr.density, tr.thr_scratch, tr.threshold], tr._ogrid_desc())
        thr = float(h(tr.threshold)[0])
        want = OG.threshold(dens2, G, cfg.diagonal_n_steps, bound)
        assert abs(thr - want) <= 1e-5 * want
        L.call("ngp_packbits_scalar", [tr.threshold, tr.density, tr.occ_mask, tr.bitfield], L.PackbitsDescriptor(G3 // 8))
        _, bits_ref = V.packbits(np.float32(thr), dens2)
        assert np.array_equal(h(tr.bitfield), bits_ref)


@pytest.mark.parametrize("K,G,bound,views", [(1, 32, 1.0, 3), (2, 32, 2.0, 2), (1, 64, 1.0, 12)])
def test_mark_untrained_matches_reference_restatement(scene, K, G, bound, views):
    """mark_untrained_density_grid (utils/types.py:1241-1362): the cells no training camera sees
    (no corner in front of it and inside its image) are marked untrainable -- bit-exact."""
    from jaxngp_gb300 import _lib as L
    c = scene.camera
    tf = scene.transforms[:views].contiguous()
    dens = torch.zeros(K * G ** 3, device="cuda")
    desc = L.NgpOgridDescriptor(K, G, 0, 0, 0, bound, 0.95, 0.0, 0, views, c.width, c.height, c.fx, c.fy, c.cx, c.cy)
    L.call("ngp_ogrid_mark_untrained", [tf, dens], desc)
    alive_g = h(dens) >= 0
    alive = OG.mark_untrained(K, G, bound, h(tf), c.width, c.height, c.fx, c.fy, c.cx, c.cy)
    assert np.array_equal(alive_g, alive), (alive_g != alive).sum()
    if views < 12:
        assert 0 < alive.mean() < 1


@pytest.mark.parametrize("wd", [0.0, 1e-6])
@pytest.mark.parametrize("count", [0, 1, 9999, 10000, 19999, 20000, 39999, 250000])
def test_adam_matches_optax_chain(count, wd):
    """ngp_adam against the optax chain of _utils.py:19-77 (adam b1 .9, b2 .99, eps 1e-15,
    eps_root 1e-15; decayed weights after the lr scaling; the staircase schedule) on parameters,
    both moments and the zeroed gradient, at counts on both sides of the schedule's steps; n is not
    a multiple of 4 (the kernel's scalar tail)."""
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.trainer import lr_at
    rng = np.random.default_rng(count + int(wd * 1e7))
    n = 10007
    p = rng.uniform(-0.1, 0.1, n).astype(np.float32)
    g = (rng.normal(size=n) * 10.0 ** rng.uniform(-9, -1, n)).astype(np.float32)
    g[::97] = 0.0
    m = (rng.normal(size=n) * 1e-3).astype(np.float32)
    v = (rng.uniform(size=n) * 1e-6).astype(np.float32)
    lr = OP.reference_lr(count, 1e-2)
    assert abs(lr_at(1e-2, count) - lr) <= 1e-7 * lr
    T = [torch.from_numpy(a.copy()).cuda() for a in (p, g, m, v)]
    L.call("ngp_adam", T, L.NgpAdamDescriptor(n, count + 1, lr_at(1e-2, count), 0.9, 0.99, 1e-15, 1e-15, wd, 1))
    p1, m1, v1 = OP.adam_update(p, g, m, v, count, lr, weight_decay=wd)
    po, go, mo, vo = (h(t) for t in T)
    assert not go.any()
    assert np.all(np.abs(po - p1) <= 1e-6 * (np.abs(p1) + lr))
    assert np.all(np.abs(mo - m1) <= 1e-6 * np.abs(m1))
    assert np.all(np.abs(vo - v1) <= 1e-6 * np.abs(v1))
