"""GPU checks of the learned proposal sampler (ngp_proposal_*, through the C ABI) against the CPU
oracle (oracle/proposal.py), and of what the trained proposal gains over sampling without it.

Bars: coarse blocks, intervals, slot allocation and bin points bit-exact (integer work and float
operations in the oracle's order, built without FMA contraction); the proposal MLP within 1e-5 of
FP64 (gradients on samples away from ReLU kinks); samples within 1e-5 of the oracle's (exp
differs by an ulp between CUDA and the host); the loss kernel within 1e-6 relative.
"""
import numpy as np
import pytest
import torch

from golden_inputs import make_rays
from oracle import hashgrid as Hh
from oracle import proposal as P
from tests.test_oracle_proposal import CENTRES, blob_bitfield

pytestmark = pytest.mark.gpu


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def desc(n=0, S=48 * 64, G=128, bound=1.0, perturb=0, seed=0, count_index=3, stride=1, spr=0, mix=0.1):
    from jaxngp_gb300 import _lib as L
    return L.NgpProposalDescriptor(n, S, G, bound, perturb, seed & 0xFFFFFFFF, seed >> 32, count_index, stride, spr, mix)


@pytest.fixture(scope="module")
def grid():
    G = 128
    bits = blob_bitfield(G, CENTRES, 0.2)
    return G, bits, P.coarse_grid(bits, G)


def test_coarse_grid_bitexact(grid):
    from jaxngp_gb300 import _lib as L
    G, bits, want = grid
    out = torch.zeros((G // 8) ** 3, dtype=torch.uint8, device="cuda")
    L.call("ngp_proposal_coarse", [cu(bits), out], desc(G=G))
    assert np.array_equal(out.cpu().numpy(), want)


def run_rays(o, d, t0, t1, coarse, S, G=128):
    from jaxngp_gb300 import _lib as L
    R = o.shape[0]
    i32 = dict(dtype=torch.int32, device="cuda")
    ctr, counts = torch.zeros(2, **i32), torch.zeros(3, **i32)
    valid = torch.zeros(R, dtype=torch.bool, device="cuda")
    ns, st = torch.zeros(R, **i32), torch.zeros(R, **i32)
    slots = S // 48
    ros, ta, tb = torch.zeros(slots, **i32), torch.zeros(slots, device="cuda"), torch.zeros(slots, device="cuda")
    L.call("ngp_proposal_rays", [o, d, t0, t1, coarse, ctr[0:1], ctr[1:2], valid, ns, st, ros, ta, tb, counts],
           desc(R, S=S, G=G))
    return ctr, counts, valid, ns, st, ros, ta, tb


def test_intervals_and_allocation(grid):
    G, bits, coarse = grid
    rng = np.random.default_rng(3)
    o, d, t0, t1 = make_rays(rng, 5000, 1.0)
    S = 48 * 1000   # fewer slots than hitting rays: some rays do not fit
    ctr, counts, valid, ns, st, ros, ta, tb = [x.cpu().numpy() for x in run_rays(cu(o), cu(d), cu(t0), cu(t1), cu(coarse), S)]
    ref = [P.ray_interval(o[i], d[i], t0[i], t1[i], coarse, G // 8, 1.0) for i in range(len(o))]
    hit = np.array([h for h, _, _ in ref])
    assert 0 < hit.sum() and hit.sum() > 1000
    # a ray without an interval is valid unless its warp took up the counter after the budget
    # filled (marching.cu:135's drop): some are, some are not with 1000 slots for > 1000 rays
    assert (ns[~hit] == 0).all() and 0 < valid[~hit].sum() < (~hit).sum()
    fits = valid & hit
    assert fits.sum() == 1000 and (ns[fits] == 48).all()
    assert ctr[0] == 48 * hit.sum() and ctr[1] == 48 * (hit.sum() - 1000)
    assert list(counts) == [1000, 64000, 48000]
    assert np.array_equal(np.sort(st[fits]), 48 * np.arange(1000))
    for r in np.nonzero(fits)[0]:
        j = st[r] // 48
        assert ros[j] == r
        assert ta[j] == ref[r][1] and tb[j] == ref[r][2]


@pytest.mark.parametrize("spr", [48, 20])
def test_bins_network_and_samples(grid, spr):
    """Bin points bit-exact; proposal MLP against FP64; samples against the oracle."""
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.proposal import ProposalSampler
    G, bits, coarse = grid
    rng = np.random.default_rng(4)
    o, d, t0, t1 = make_rays(rng, 3000, 1.0)
    S = spr * 512
    ps = ProposalSampler(3000, S, G, 1.0, seed=5, samples_per_ray=spr)
    ps.f16 = False   # FP32 bins: checked against FP64 below (the FP16 path has its own test)
    with torch.no_grad():
        ps.latents.uniform_(-1, 1)
    ps.refresh(cu(bits))
    R = 3000
    i32 = dict(dtype=torch.int32, device="cuda")
    valid = torch.zeros(R, dtype=torch.bool, device="cuda")
    ns, st = torch.zeros(R, **i32), torch.zeros(R, **i32)
    idcs = torch.zeros(S, **i32)
    xyzs, dirs = torch.zeros(S, 3, device="cuda"), torch.zeros(S, 3, device="cuda")
    dss, zs = torch.zeros(S, device="cuda"), torch.zeros(S, device="cuda")
    cnt = ps.sample(cu(o), cu(d), cu(t0), cu(t1), valid, ns, st, idcs, xyzs, dirs, dss, zs, False, 0)
    n_slots = int(ps.counts[0])
    assert int(cnt) == spr * n_slots and n_slots == 512
    ros, ta, tb = ps.ray_of_slot.cpu().numpy(), ps.slot_ta.cpu().numpy(), ps.slot_tb.cpu().numpy()
    pts = ps.points.cpu().numpy()
    for j in range(0, n_slots, 37):
        r = ros[j]
        want, _ = P.bin_points(o[r], d[r], ta[j], tb[j])
        assert np.array_equal(pts[j * 64:(j + 1) * 64], want)
    # network at the bin points against FP64
    lat = ps.latents.cpu().numpy()
    w = P.unpack(ps.weights.cpu().numpy())
    tab = P.table()
    npts = n_slots * 64
    enc64 = Hh.encode(pts[:npts], lat, 1.0, tab, dtype=np.float64)
    x64, _ = P.mlp_forward(enc64, w, dtype=np.float64)
    xg = ps.x_b.cpu().numpy()[:npts]
    assert np.abs(xg - x64).max() <= 1e-5 * max(1.0, np.abs(x64).max())
    # samples against the oracle from the GPU's own bin values
    X, Ds, Zs, Dr = xyzs.cpu().numpy(), dss.cpu().numpy(), zs.cpu().numpy(), dirs.cpu().numpy()
    for j in range(0, n_slots, 29):
        r = ros[j]
        t, ds = P.sample_ray(xg[j * 64:(j + 1) * 64], ta[j], tb[j], np.full(spr, 0.5, np.float32), spr)
        s = slice(j * spr, (j + 1) * spr)
        scale = max(1.0, abs(float(tb[j])))
        assert np.abs(Zs[s] - t).max() <= 1e-5 * scale
        assert np.abs(Ds[s] - ds).max() <= 2e-5 * scale
        assert np.allclose(X[s], o[r][None] + Zs[s][:, None] * d[r][None], rtol=0, atol=1e-6)
        assert np.array_equal(Dr[s], np.repeat(d[r][None], spr, 0))
        assert (np.diff(Zs[s]) >= 0).all() and Zs[s][0] >= ta[j] and Zs[s][-1] <= tb[j]
        assert (idcs.cpu().numpy()[s] == r).all()


def test_perturbed_samples_stay_sorted(grid):
    from jaxngp_gb300.proposal import ProposalSampler
    G, bits, coarse = grid
    rng = np.random.default_rng(6)
    o, d, t0, t1 = make_rays(rng, 2000, 1.0)
    S = 48 * 256
    ps = ProposalSampler(2000, S, G, 1.0, seed=7)
    ps.refresh(cu(bits))
    R = 2000
    i32 = dict(dtype=torch.int32, device="cuda")
    bufs = [torch.zeros(R, dtype=torch.bool, device="cuda"), torch.zeros(R, **i32), torch.zeros(R, **i32),
            torch.zeros(S, **i32), torch.zeros(S, 3, device="cuda"), torch.zeros(S, 3, device="cuda"),
            torch.zeros(S, device="cuda"), torch.zeros(S, device="cuda")]
    ps.sample(cu(o), cu(d), cu(t0), cu(t1), *bufs, True, 1234)
    z = bufs[7].cpu().numpy().reshape(-1, 48)
    ta, tb = ps.slot_ta.cpu().numpy(), ps.slot_tb.cpu().numpy()
    assert (np.diff(z, axis=1) >= 0).all()
    assert (z[:, 0] >= ta[:, None][:, 0]).all() and (z[:, -1] <= tb).all()
    a = z.copy()
    ps.sample(cu(o), cu(d), cu(t0), cu(t1), *bufs, True, 1235)
    assert not np.array_equal(a, bufs[7].cpu().numpy().reshape(-1, 48))


def test_mlp_backward_vs_fp64():
    from jaxngp_gb300 import _lib as L
    rng = np.random.default_rng(8)
    n = 20000
    enc = rng.normal(size=(n, 8)).astype(np.float32)
    g = rng.normal(size=n).astype(np.float32)
    w = P.init_weights(9)
    _, c64 = P.mlp_forward(enc, w, dtype=np.float64)
    kink = np.minimum(np.abs(c64["a1"]).min(1) / np.abs(c64["a1"]).max(), np.abs(c64["a2"]).min(1) / np.abs(c64["a2"]).max())
    keep = kink > 1e-4
    enc, g = enc[keep], g[keep]
    n = enc.shape[0]
    _, c64 = P.mlp_forward(enc, w, dtype=np.float64)
    de64, gw64 = P.mlp_backward(g, c64, w)
    wt = cu(P.pack(w))
    denc = torch.zeros(n, 8, device="cuda")
    dw = torch.zeros(P.N_WEIGHTS, device="cuda")
    scratch = torch.zeros(L.proposal_backward_scratch_floats(), device="cuda")
    L.call("ngp_proposal_mlp_backward", [cu(enc), wt, cu(g), None, scratch, denc, dw], L.NgpMlpDescriptor(n, 0))
    de = denc.cpu().numpy()
    assert (np.abs(de - de64) / np.abs(de64).max(0, keepdims=True)).max() <= 1e-5
    gw = P.unpack(dw.cpu().numpy())
    for k in gw:
        assert np.abs(gw[k] - gw64[k]).max() / np.abs(gw64[k]).max() <= 1e-5, k


def test_loss_kernel():
    from jaxngp_gb300 import _lib as L
    rng = np.random.default_rng(10)
    n = 5000
    x = rng.normal(size=n).astype(np.float32)
    drgb = np.abs(rng.normal(size=(n, 4))).astype(np.float32) * 3
    counts = torch.tensor([0, 0, 4000], dtype=torch.int32, device="cuda")
    gx = torch.full((n,), 9.0, device="cuda")
    loss = torch.zeros(1, device="cuda")
    L.call("ngp_proposal_loss", [counts, cu(x), cu(drgb), gx, loss], desc(n, count_index=2, stride=4))
    want, lsum = P.loss_grad(x[:4000], drgb[:4000, 0], 4000)
    got = gx.cpu().numpy()
    assert np.allclose(got[:4000], want, rtol=1e-6, atol=1e-9) and (got[4000:] == 0).all()
    assert abs(float(loss) - lsum) <= 1e-5 * lsum


@pytest.fixture(scope="module")
def trained_pair():
    """The same scene (blobs and two thin shells) trained for the same steps with the
    occupancy-grid march and with the proposal sampler (BF16 field MLP)."""
    from jaxngp_gb300.scene import make_scene_data
    from jaxngp_gb300.trainer import NGPTrainer, TrainConfig
    data = make_scene_data(n_blobs=16, n_shells=2, n_views=16, width=96, height=96, n_steps=1024, seed=11)
    out = {}
    for sampler in ("march", "proposal"):
        cfg = TrainConfig(total_samples=1 << 16, T=1 << 16, seed=3, mlp_precision="bf16", sampler=sampler,
                          proposal_fallback=True)
        tr = NGPTrainer(data, cfg)
        tr.init_occupancy_analytic(steady_state=False)
        losses, hit_samples, rays_with_samples = [], [], []
        for it in range(500):
            st = tr.step()
            if it % 50 == 0 or it >= 490:
                losses.append(float(st[0]))
                ns = tr.n_samples[tr.valid & (tr.n_samples > 0)]
                hit_samples.append(float((ns == 48).float().mean()) if ns.numel() else 0.0)
                rays_with_samples.append(int(ns.numel()))
        out[sampler] = (tr, losses, hit_samples, rays_with_samples)
    return data, out


def test_proposal_and_march_training_quality(trained_pair):
    """Both samplers train on the same sample budget (2^16 samples, 2^16 rays per step) and are
    judged by the same occupancy-grid renderer.  On this scene the march spends ~170 samples on
    each ray it fits (its rays fit in ray order until the budget is full), the proposal 48 on
    more rays, which resolve the thin shells less well: at equal steps the proposal's held-out
    PSNR (29-31 dB over runs) is 2-4 dB below the march's (33.6 dB); the test asks for 27 dB
    and 32 dB.  The proposal runs with both fallbacks: a march step every 8th step, whose evenly
    spread samples also teach the proposal, and the per-ray march of the rays on which the
    proposal misses transmittance.  The fallback rays come first in the budget and take ~150
    samples each, so the share of rays with samples that carry the proposal's 48 varies over
    runs and steps (0.24 to above 0.5 at step 499); the test asks that every proposal step among
    the last ten gives the proposal's samples to some rays and that fewer than half the slots fall
    back."""
    from jaxngp_gb300.trainer import evaluate_psnr
    data, out = trained_pair
    psnr = {}
    for sampler, (tr, losses, hit, nrays) in out.items():
        assert np.isfinite(losses).all()
        # the median: a march step among the last ones (every 8th of the proposal sampler) has the
        # loss of its own, fewer, valid rays
        assert np.median(losses[-5:]) < 0.5 * losses[0], (sampler, losses)
        psnr[sampler] = evaluate_psnr(tr, n_views=8)
        print(f"{sampler}: PSNR {psnr[sampler]:.2f} dB over 8 views; rays with samples per step "
              f"(median of the last 10 steps) {np.median(nrays[-10:]):.0f}")
    assert psnr["proposal"] >= 27.0 and psnr["march"] >= 32.0, psnr
    tr = out["proposal"][0]
    assert tr.cfg.march_every == 8
    # the last ten records are steps 490-499; step 495 (495 % 8 == 7) is the march step
    shares = [h for it, h in zip(range(490, 500), out["proposal"][2][-10:]) if it % 8 != 7]
    print("proposal steps 490-499: share of rays with samples that carry 48:", np.round(shares, 2))
    assert min(shares) > 0, shares
    assert 0 < tr.prop.fallback_rate() < 0.5 * tr.prop.slots


def test_proposal_samples_place_like_dense(trained_pair):
    """The trained proposal's 48 samples per ray composite the field about as close to a dense
    (1024-sample) rendering as 48 stratified uniform samples over the same interval, or closer."""
    from jaxngp_gb300 import volrendjax as vr
    from jaxngp_gb300.encoders import hashgrid_forward
    from jaxngp_gb300.field import field_forward
    from jaxngp_gb300.trainer import camera_rays, near_far
    data, out = trained_pair
    tr = out["proposal"][0]
    precision = tr.cfg.mlp_precision
    o, d = camera_rays(data.camera, data.transforms[5])
    t0, t1 = near_far(tr.bound, o, d)
    R = o.shape[0]
    S = tr.prop.S
    i32 = dict(dtype=torch.int32, device="cuda")
    valid = torch.zeros(R, dtype=torch.bool, device="cuda")
    ns, st_ = torch.zeros(R, **i32), torch.zeros(R, **i32)
    idcs = torch.zeros(S, **i32)
    xyzs, dirs = torch.zeros(S, 3, device="cuda"), torch.zeros(S, 3, device="cuda")
    dss, zs = torch.zeros(S, device="cuda"), torch.zeros(S, device="cuda")
    tr.prop.sample(o, d, t0, t1, valid, ns, st_, idcs, xyzs, dirs, dss, zs, False, 0)
    n_slots = int(tr.prop.counts[0])
    assert n_slots > 50
    rays = tr.prop.ray_of_slot[:n_slots].long()
    ta, tb = tr.prop.slot_ta[:n_slots], tr.prop.slot_tb[:n_slots]

    def composite(t, dt):
        """colour of each slot's ray from samples at distances t [n, k] with widths dt."""
        n, k = t.shape
        p = (o[rays][:, None, :] + t[..., None] * d[rays][:, None, :]).reshape(-1, 3).contiguous()
        dr = d[rays][:, None, :].expand(n, k, 3).reshape(-1, 3).contiguous()
        enc = hashgrid_forward(tr.table, p, tr.latents, tr.bound)
        drgb = field_forward(enc, dr, tr.weights, precision=precision)
        start = (torch.arange(n, device="cuda", dtype=torch.int32) * k)
        nsamp = torch.full((n,), k, dtype=torch.int32, device="cuda")
        bg = torch.ones(n, 3, device="cuda")
        _, rgbd, _ = vr.integrate_rays(0.0, start, nsamp, bg, dt.reshape(-1).contiguous(), t.reshape(-1).contiguous(), drgb)
        return rgbd[:, :3]

    K = 1024
    u = (torch.arange(K, device="cuda").float() + 0.5) / K
    t_dense = ta[:, None] + u[None] * (tb - ta)[:, None]
    dense = composite(t_dense, ((tb - ta) / K)[:, None].expand(-1, K))
    tp = zs[:n_slots * 48].view(n_slots, 48)
    prop = composite(tp, dss[:n_slots * 48].view(n_slots, 48))
    uu = (torch.arange(48, device="cuda").float() + 0.5) / 48
    tu = ta[:, None] + uu[None] * (tb - ta)[:, None]
    unif = composite(tu, ((tb - ta) / 48)[:, None].expand(-1, 48))
    e_prop = float((prop - dense).abs().mean())
    e_unif = float((unif - dense).abs().mean())
    assert e_prop < 1.5 * e_unif, (e_prop, e_unif)


def test_proposal_mlp_f16_forward():
    """The FP16 tensor-core forward against FP64: within 2e-2 of the output scale (FP16 operands),
    and its active count respected."""
    from jaxngp_gb300 import _lib as L
    rng = np.random.default_rng(12)
    n = 70000
    enc = rng.normal(scale=0.5, size=(n, 8)).astype(np.float32)
    w = P.init_weights(13)
    x64, _ = P.mlp_forward(enc, w, dtype=np.float64)
    out = torch.full((n,), -9.0, device="cuda")
    count = torch.tensor([n - 123], dtype=torch.int32, device="cuda")
    L.call("ngp_proposal_mlp_forward_f16", [cu(enc), cu(P.pack(w)), count, out], L.NgpMlpDescriptor(n, 0))
    got = out.cpu().numpy()
    assert np.abs(got[:n - 123] - x64[:n - 123]).max() <= 2e-2 * np.abs(x64).max()
    assert (got[n - 123:] == -9.0).all()
    assert L.lib().ngp_device_status() == 0


def test_fallback_flow(grid):
    """Per-ray fallback: ngp_proposal_judge flags the rays the oracle's missed-transmittance test
    flags (away from the 1% limit); the flagged rays carry exactly the occupancy-grid march's
    samples, the others exactly the proposal's samples, the ranges tile [0, count) and the rest of
    the buffers is zeroed."""
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.proposal import ProposalSampler
    G, bits, coarse = grid
    rng = np.random.default_rng(12)
    R = 3000
    o, d, t0, t1 = make_rays(rng, R, 1.0)
    S = 48 * 1400
    ps = ProposalSampler(R, S, G, 1.0, seed=13)
    with torch.no_grad():
        ps.latents.uniform_(-1, 1)
    ps.refresh(cu(bits))
    thr = torch.tensor([3.0], device="cuda")
    noises = torch.zeros(R, device="cuda")
    dm = L.MarchingDescriptor(R, S, 1024, 1, G, 1.0, 0.0)
    i32 = dict(dtype=torch.int32, device="cuda")

    def bufs():
        return [torch.zeros(R, dtype=torch.bool, device="cuda"), torch.zeros(R, **i32), torch.zeros(R, **i32),
                torch.zeros(S, **i32), torch.full((S, 3), 5.0, device="cuda"), torch.zeros(S, 3, device="cuda"),
                torch.full((S,), 5.0, device="cuda"), torch.zeros(S, device="cuda")]
    fb = bufs()
    cnt = int(ps.sample(cu(o), cu(d), cu(t0), cu(t1), *fb, False, 0, fallback=(cu(bits), thr, noises, dm)))
    valid, ns, st, idcs, X, Dr, Ds, Z = [b.cpu().numpy() for b in fb]
    n_slots = int(ps.counts[0])
    flags = ps.slot_flag.cpu().numpy()[:n_slots].astype(bool)
    ros, ta, tb = ps.ray_of_slot.cpu().numpy(), ps.slot_ta.cpu().numpy(), ps.slot_tb.cpu().numpy()
    xb = ps.x_b.cpu().numpy()
    n_fb = int(ps.fb_count)
    assert n_fb == flags.sum() and 0 < n_fb < n_slots
    assert sorted(ps.fb_rays.cpu().numpy()[:n_fb]) == sorted(ros[:n_slots][flags])
    for j in range(n_slots):
        m = P.missed_transmittance(xb[j * 64:(j + 1) * 64], ta[j], tb[j], o[ros[j]], d[ros[j]], bits, G, 1.0, 3.0)
        if abs(m - P.MISS_LIMIT) > 1e-4:
            assert flags[j] == (m > P.MISS_LIMIT), (j, m)
    # the flagged rays' samples are the march's (march_rays on every ray, with room for all)
    big = 1 << 22
    mv = [torch.zeros(R, dtype=torch.bool, device="cuda"), torch.zeros(R, **i32), torch.zeros(R, **i32),
          torch.zeros(big, **i32), torch.zeros(big, 3, device="cuda"), torch.zeros(big, 3, device="cuda"),
          torch.zeros(big, device="cuda"), torch.zeros(big, device="cuda")]
    ctr = torch.zeros(2, **i32)
    L.call("march_rays", [cu(o), cu(d), cu(t0), cu(t1), noises, cu(bits), ctr[0:1], ctr[1:2]] + mv,
           L.MarchingDescriptor(R, big, 1024, 1, G, 1.0, 0.0))
    m_ns, m_st, m_X, m_Ds, m_Z = mv[1].cpu().numpy(), mv[2].cpu().numpy(), mv[4].cpu().numpy(), mv[6].cpu().numpy(), mv[7].cpu().numpy()
    for r in ros[:n_slots][flags]:
        assert valid[r]
        assert ns[r] == m_ns[r], (r, ns[r], m_ns[r])
        a, b = slice(st[r], st[r] + ns[r]), slice(m_st[r], m_st[r] + m_ns[r])
        assert np.array_equal(Z[a], m_Z[b]) and np.array_equal(Ds[a], m_Ds[b]) and np.array_equal(X[a], m_X[b])
    # the other slots' rays carry the proposal's samples (the same as without the fallback)
    pl = bufs()
    ps.sample(cu(o), cu(d), cu(t0), cu(t1), *pl, False, 0)
    p_valid, p_ns, p_st, _, _, _, p_Ds, p_Z = [b.cpu().numpy() for b in pl]
    for r in ros[:n_slots][~flags]:
        if not valid[r]:
            continue   # past the budget
        assert ns[r] == 48 and p_ns[r] == 48
        a, b = slice(st[r], st[r] + 48), slice(p_st[r], p_st[r] + 48)
        assert np.array_equal(Z[a], p_Z[b]) and np.array_equal(Ds[a], p_Ds[b])
    # ranges tile [0, count); the tail is zeroed
    owned = np.zeros(S, int)
    for r in np.nonzero(valid & (ns > 0))[0]:
        owned[st[r]:st[r] + ns[r]] += 1
    assert cnt == int(ns[valid].sum()) and (owned[:cnt] == 1).all() and (owned[cnt:] == 0).all()
    assert (Ds[cnt:] == 0).all() and (Z[cnt:] == 0).all() and (X[cnt:] == 0).all()


def test_proposal_renderer(trained_pair):
    """The learned proposal's renderer: a ray that misses the scene box shows the background
    exactly; its held-out PSNR on the proposal-trained field is within 1 dB of the occupancy-grid
    march renderer's (both judged against the quadrature ground truth)."""
    from jaxngp_gb300.renderer import ProposalRenderer
    from jaxngp_gb300.trainer import HeldOut, camera_rays, near_far
    data, out = trained_pair
    tr = out["proposal"][0]
    rnd = ProposalRenderer(tr, chunk=1 << 12)
    held = HeldOut(data, n_views=2)
    p_march, p_prop = held.psnr(tr), held.psnr(tr, rnd)
    assert p_prop >= p_march - 1.0, (p_prop, p_march)
    o, d = camera_rays(data.camera, data.transforms[3])
    t0, t1 = near_far(tr.bound, o, d)
    bg = torch.rand(o.shape[0], 3, device="cuda")
    rgbd = rnd.render_rays(o, d, t0, t1, bg)
    assert torch.isfinite(rgbd).all()
    miss = t1 <= t0   # rays that miss the scene box take no samples
    assert bool(miss.any()) and torch.equal(rgbd[miss, :3], bg[miss])
