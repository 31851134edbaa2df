"""The fused integrate + Huber loss + backward entry point (ngp_integrate_loss_backward) against
its parts: the drop-in integrate_rays / integrate_rays_backward (checked against the oracle in
test_gpu_volrend.py) and the masked Huber loss of app/nerf/_utils.py:151-156 restated here.

Bar: colours, loss and per-sample gradients within 1e-5 of the column's scale (the fused kernel
composites in the drop-in kernels' order), on rays away from the T = 1e-4 threshold."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def layout(rng, R, S, empty_frac, max_n, clustered):
    """A march_rays-like sample layout: per-ray counts, contiguous starts, some rays empty, some
    invalid (past the budget)."""
    n = rng.integers(1, max_n + 1, size=R)
    n[rng.uniform(size=R) < empty_frac] = 0
    order = np.arange(R) if clustered else rng.permutation(R)
    start = np.zeros(R, np.int64)
    valid = np.ones(R, bool)
    pos = 0
    for r in order:
        if n[r] == 0:
            continue
        if pos + n[r] > S:
            valid[r] = False
            n[r] = 0
            continue
        start[r] = pos
        pos += n[r]
    return valid, n.astype(np.int32), start.astype(np.int32), pos


@pytest.mark.parametrize("clustered", [False, True])
def test_fused_loss_matches_parts(clustered):
    from jaxngp_gb300 import _lib as L
    rng = np.random.default_rng(5 if clustered else 6)
    R, S = 20000, 1 << 17
    valid, ns, st, used = layout(rng, R, S, 0.6, 48, clustered)
    dss = rng.uniform(0.001, 0.02, size=S).astype(np.float32)
    zs = np.zeros(S, np.float32)
    for r in range(R):
        if ns[r]:
            zs[st[r]:st[r] + ns[r]] = 0.5 + np.cumsum(dss[st[r]:st[r] + ns[r]])
    drgbs = np.concatenate([rng.exponential(20.0, size=(S, 1)), rng.uniform(size=(S, 3))], 1).astype(np.float32)
    bgs = rng.uniform(size=(R, 3)).astype(np.float32)
    gt = rng.uniform(size=(R, 3)).astype(np.float32)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    count = torch.tensor([used], dtype=torch.int32, device="cuda")
    g_drgbs = torch.full((S, 4), 7.0, device="cuda")
    stats = torch.zeros(4, device="cuda")
    gs = torch.zeros(1, device="cuda")
    scratch = torch.zeros(4 + R, device="cuda")
    near, delta = 0.3, 0.1
    L.call("ngp_integrate_loss_backward", [cu(valid), cu(st), cu(ns), cu(bgs), cu(gt), cu(dss), cu(zs), cu(drgbs), count,
                                           scratch, g_drgbs, stats, gs], L.NgpIntegrateLossDescriptor(R, S, near, delta))

    # the parts: integrate_rays, Huber, integrate_rays_backward
    i32 = dict(dtype=torch.int32, device="cuda")
    measured = torch.zeros(1, **i32)
    rgbd = torch.zeros(R, 4, device="cuda")
    opac = torch.zeros(R, device="cuda")
    L.call("integrate_rays", [cu(st), cu(ns), cu(bgs), cu(dss), cu(zs), cu(drgbs), measured, rgbd, opac],
           L.IntegratingDescriptor(R, S))
    pred = rgbd[:, :3].cpu().numpy().astype(np.float64)
    e = pred - gt
    ae = np.abs(e)
    hub = np.where(ae <= delta, 0.5 * e * e, delta * (ae - 0.5 * delta)).mean(1)
    nv = valid.sum()
    loss = (hub * valid).sum() / nv
    go = np.where(ae <= delta, e, delta * np.sign(e)) / 3.0 * valid[:, None]
    dL_dfinal = np.concatenate([go, np.zeros((R, 1))], 1).astype(np.float32)
    dbg, dz, dd = torch.zeros(R, 3, device="cuda"), torch.zeros(S, device="cuda"), torch.zeros(S, 4, device="cuda")
    L.call("integrate_rays_backward", [cu(st), cu(ns), cu(bgs), cu(dss), cu(zs), cu(drgbs), rgbd, opac, cu(dL_dfinal),
                                       dbg, dz, dd], L.IntegratingBackwardDescriptor(R, S, near))
    st_ = stats.cpu().numpy()
    assert st_[1] == nv
    assert abs(st_[0] - loss) <= 1e-5 * abs(loss)
    assert st_[2] == float(measured.item()) and st_[3] == used
    assert abs(float(gs) - 1.0 / nv) <= 1e-7
    # rays away from the termination threshold (a rounding can flip which side they fall)
    T = 1.0 - opac.cpu().numpy()
    keep_ray = (np.abs(T - 1e-4) > 1e-3 * 1e-4) | (ns == 0)
    keep = np.zeros(S, bool)
    for r in np.nonzero(keep_ray & (ns > 0))[0]:
        keep[st[r]:st[r] + ns[r]] = True
    a, b = g_drgbs.cpu().numpy(), dd.cpu().numpy()
    scale = np.abs(b[keep]).max(0)
    assert (np.abs(a[keep] - b[keep]) / scale).max() <= 1e-5
    assert (a[used:] == 0).all()
