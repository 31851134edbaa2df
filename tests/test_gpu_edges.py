"""Edge cases through the C ABI: the size limits the descriptors allow (G = 1024, the Morton code's
10 bits per axis and the marcher's shared expansion table; K = 16 cascades; L = 32 levels, the
encoder's shared tile) against the oracle, and empty inputs (no points, no rays, no samples)
through every entry point that takes a count."""
import numpy as np
import pytest
import torch

from golden_inputs import make_rays, random_bitfield
from oracle import hashgrid as H
from oracle import volrend as V

pytestmark = pytest.mark.gpu


def cu(a):
    a = np.asarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    a = t.detach().cpu().numpy()
    return a.view(np.uint32) if a.dtype == np.int32 else a


@pytest.mark.parametrize("K,G,bound,sp,n", [(1, 1024, 1.0, 0.0, 1500), (16, 64, 16.0, 1 / 256, 3000)])
def test_march_at_the_size_limits(K, G, bound, sp, n):
    """G = 1024 (a 128 MB bitfield per cascade) and K = 16 cascades: per-ray counts, validity and
    sample sequences bit-exact against the oracle."""
    from jaxngp_gb300 import volrendjax as vr
    rng = np.random.default_rng(K * 7 + G)
    o, d, t0, t1 = make_rays(rng, n, bound)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, K, G, 0.02 if G == 1024 else 0.25)
    total = 1 << 22
    a = V.march_rays(total, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits)
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), _ = vr.march_rays(
        total, 1024, K, G, bound, sp, cu(o), cu(d), cu(t0), cu(t1), cu(noise), cu(bits), return_counters=True)
    ns, st, valid = host(ns), host(st), host(valid)
    assert int(host(m)) == a[0] and a[0] > 0
    assert np.array_equal(valid, a[1]) and np.array_equal(ns, a[2])
    X, Z = host(xyzs), host(zs)
    for r in np.nonzero(ns)[0][:: max(1, len(np.nonzero(ns)[0]) // 300)]:
        x0, y0, k = st[r], a[3][r], ns[r]
        assert np.array_equal(X[x0:x0 + k], a[5][y0:y0 + k]) and np.array_equal(Z[x0:x0 + k], a[8][y0:y0 + k])


def test_hashgrid_at_32_levels():
    """L = 32 (the most the descriptor holds; the forward's shared tile is exactly full): encodings
    bit-exact, table gradient and TV term within 1e-5 of FP64."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward, hashgrid_forward, hashgrid_tv
    rng = np.random.default_rng(32)
    n = 4096 + 17
    pos = rng.uniform(-1.05, 1.05, size=(n, 3)).astype(np.float32)
    tab = H.LevelTable(32, 2 ** 16, 2, 16, 4096)
    t = LevelTable(32, 2 ** 16, 2, 16, 4096)
    lat = rng.uniform(-1, 1, size=(tab.n_params, 2)).astype(np.float32)
    assert np.array_equal(hashgrid_forward(t, cu(pos), cu(lat), 1.0).cpu().numpy(), H.encode(pos, lat, 1.0, tab))
    g = rng.normal(size=(n, 64)).astype(np.float32)
    got = hashgrid_backward(t, cu(pos), cu(g), 1.0).cpu().numpy()
    want = H.encode_backward(pos, g, 1.0, tab)
    assert (np.abs(got - want).max(0) / np.abs(want).max(0)).max() <= 1e-5
    tv = float(hashgrid_tv(t, cu(pos), cu(lat), 1.0, 0.1))
    want_tv = H.total_variation(pos, lat, 1.0, tab, 0.1, dtype=np.float64)
    assert abs(tv - want_tv) <= 1e-5 * want_tv


def test_empty_inputs_everywhere():
    """No points, rays or samples: every entry point returns without touching memory it was not
    given, outputs that depend on nothing are zero (the table gradient is zero-filled, the MLP's
    weight gradient is zero), and the TV term is the mean of nothing, NaN, as in the reference."""
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300 import volrendjax as vr
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward, hashgrid_forward, hashgrid_tv
    from jaxngp_gb300.field import field_backward, field_forward, pack_weights
    from jaxngp_gb300.precision import integrate_rays_fp64
    from oracle import field as Fd
    e3 = torch.zeros(0, 3, device="cuda")
    t = LevelTable(16, 2 ** 14, 2, 16, 2048)
    lat = torch.rand(t.n_params, 2, device="cuda")
    assert hashgrid_forward(t, e3, lat, 1.0).shape == (0, 32)
    assert hashgrid_forward(t, e3, lat.to(torch.bfloat16), 1.0, enc_dtype=torch.bfloat16).shape == (0, 32)
    gl = hashgrid_backward(t, e3, torch.zeros(0, 32, device="cuda"), 1.0)
    assert gl.shape == (t.n_params, 2) and not gl.any()
    assert np.isnan(float(hashgrid_tv(t, e3, lat, 1.0, 0.5)))
    assert float(hashgrid_tv(t, e3, lat, 1.0, 0.0)) == 0.0
    w = pack_weights({k: torch.from_numpy(v) for k, v in Fd.init_weights(1).items()}).cuda()
    e32 = torch.zeros(0, 32, device="cuda")
    assert field_forward(e32, e3, w).shape == (0, 4)
    denc, dw = field_backward(e32, e3, w, torch.zeros(0, 4, device="cuda"))
    assert denc.shape == (0, 32) and dw.shape == (L.MLP_WEIGHTS,) and not dw.any()
    ei = torch.zeros(0, dtype=torch.int32, device="cuda")
    assert vr.morton3d(torch.zeros(0, 3, dtype=torch.int32, device="cuda")).shape == (0,)
    assert vr.morton3d_invert(ei).shape == (0, 3)
    rgbd, T, used = integrate_rays_fp64(ei, ei, torch.zeros(0, 3, device="cuda"), torch.zeros(0, device="cuda"),
                                        torch.zeros(0, device="cuda"), torch.zeros(0, 4, device="cuda"))
    assert rgbd.shape == (0, 4) and T.shape == (0,) and used.shape == (0,)
    assert L.lib().ngp_device_status() == 0
