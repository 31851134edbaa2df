"""Edge cases of the drop-in march and integrators on the GPU, against the oracle: cascades with a
t-dependent step under overflow (the ray-order schedule's every buffer, bit for bit), budgets too
small for the ray-order passes' borrowed words (the finish-order form's invariants), ragged and
empty batches, and rays of the largest sample count through the warp-per-ray integrators."""
import numpy as np
import pytest
import torch

from golden_inputs import make_rays, random_bitfield
from oracle import volrend as V
from tests.test_gpu_volrend import assert_close, away_from_threshold, dev, host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vr():
    from jaxngp_gb300 import volrendjax
    return volrendjax


def _march(vr, total, K, G, bound, sp, o, d, t0, t1, noise, bits):
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), counters = vr.march_rays(
        total, 1024, K, G, bound, sp, dev(o), dev(d), dev(t0), dev(t1), dev(noise), dev(bits), return_counters=True)
    return [host(x) for x in (valid, ns, st, idcs, xyzs, dirs, dss, zs)], host(counters), int(host(m))


@pytest.mark.parametrize("seed,K,G,bound,sp,n,frac", [(4, 3, 64, 4.0, 1 / 256, 3000, 0.25),
                                                      (5, 2, 32, 2.0, 6e-3, 777, 0.5),
                                                      (6, 1, 128, 1.0, 0.0, 257, 0.1)])
def test_march_overflow_cascades_ragged(vr, seed, K, G, bound, sp, n, frac):
    """Overflowing budgets with cascades and a t-dependent step, ragged ray counts: every buffer
    and both counters equal the oracle's one-at-a-time ray-order march."""
    rng = np.random.default_rng(seed)
    o, d, t0, t1 = make_rays(rng, n, bound)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, K, G, 0.3)
    full = V.march_rays(1 << 24, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits)[2]
    total = max(4 * ((n + 255) // 256) + 8, int(full.sum() * frac))
    got, counters, m = _march(vr, total, K, G, bound, sp, o, d, t0, t1, noise, bits)
    ref, cref = V.march_rays(total, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits, return_counters=True,
                             early_exit=True)
    assert np.array_equal(counters, cref) and m == int(cref[0]) - int(cref[1])
    for name, x, y in zip(("valid", "n_samples", "startidx", "idcs", "xyzs", "dirs", "dss", "z_vals"), got, ref[1:]):
        assert np.array_equal(x, y), name


def test_march_budget_below_borrowed_words(vr):
    """A budget smaller than the ray-order passes borrow (2 ceil(R / 256) + 3 words): the rays take
    slots in the order their warps finish, as in the reference; every ray that fits carries its full
    sample run, the written samples tile [0, measured) and the tail is zero."""
    rng = np.random.default_rng(7)
    n = 4096
    o, d, t0, t1 = make_rays(rng, n, 1.0)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, 1, 64, 0.5)
    full = V.march_rays(1 << 24, 1024, 1, 64, 1.0, 0.0, o, d, t0, t1, noise, bits)[2]
    total = 2 * ((n + 255) // 256) + 2   # 34 slots: one word short
    (valid, ns, st, idcs, xyzs, dirs, dss, zs), counters, m = _march(vr, total, 1, 64, 1.0, 0.0, o, d, t0, t1, noise,
                                                                     bits)
    assert m == int(counters[0]) - int(counters[1]) and m <= total and int(ns.sum()) == m
    fit = ns > 0
    assert np.array_equal(ns[fit], full[fit])
    owned = np.zeros(total, int)
    for r in np.nonzero(fit)[0]:
        owned[st[r]:st[r] + ns[r]] += 1
        assert (idcs[st[r]:st[r] + ns[r]] == r).all()
    assert (owned[:m] == 1).all() and (owned[m:] == 0).all()
    assert not zs[m:].any() and not dss[m:].any()


def test_march_empty_batch_and_budget(vr):
    """No rays: nothing marched, counters zero, the sample buffers zeroed."""
    bits = random_bitfield(np.random.default_rng(8), 1, 64, 0.5)
    z3 = np.zeros((0, 3), np.float32)
    z1 = np.zeros(0, np.float32)
    got, counters, m = _march(vr, 64, 1, 64, 1.0, 0.0, z3, z3, z1, z1, z1, bits)
    assert m == 0 and not counters.any()
    assert not got[3].any() and not got[7].any()


@pytest.mark.parametrize("n", [1, 31, 33, 1000])
def test_integrate_ragged_and_longest_rays(vr, n):
    """Ragged ray counts, rays without samples beside rays of 1024 samples (the largest count a
    march gives): forward and backward against the oracle; `measured` exact."""
    rng = np.random.default_rng(100 + n)
    ns = rng.choice([0, 1, 5, 200, 1024], size=n).astype(np.uint32)
    st = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.uint32)
    S = max(int(ns.sum()), 1)
    dss = rng.uniform(0.001, 0.004, S).astype(np.float32)
    zs = (np.cumsum(dss) % 4.0).astype(np.float32)
    drgbs = np.concatenate([rng.exponential(2.0, (S, 1)), rng.uniform(size=(S, 3))], -1).astype(np.float32)
    bgs = rng.uniform(size=(n, 3)).astype(np.float32)
    a = V.integrate_rays(0.3, st, ns, bgs, dss, zs, drgbs)
    drgbs_d = dev(drgbs).requires_grad_(True)
    bgs_d = dev(bgs).requires_grad_(True)
    zs_d = dev(zs).requires_grad_(True)
    m, rgbd, opac = vr.integrate_rays(0.3, dev(st), dev(ns), bgs_d, dev(dss), zs_d, drgbs_d)
    assert int(host(m)) == int(a[0])
    ok = away_from_threshold(a[2])
    assert_close(host(rgbd), a[1], mask=ok)
    assert_close(host(opac), a[2])
    g = rng.normal(size=(n, 4)).astype(np.float32)
    torch.autograd.backward(rgbd, dev(g))
    b = V.integrate_rays_backward(0.3, st, ns, bgs, dss, zs, drgbs, a[1], a[2], g)
    ok_s = np.repeat(ok, ns.astype(np.int64))
    assert_close(host(bgs_d.grad), b[0], mask=ok)
    assert_close(host(zs_d.grad)[:ok_s.size], b[1][:ok_s.size], mask=ok_s)
    assert_close(host(drgbs_d.grad)[:ok_s.size], b[2][:ok_s.size], mask=ok_s)
