"""GPU parity of the volume-rendering ops (through the C ABI) against the reference's own outputs
(golden fixtures) and the CPU oracle.

Bar: bit-exact for integer outputs (sample counts, start indices, ray indices, Morton codes,
bitfields, masks, counters) and for the marcher's float outputs (same operation sequence, one
rounding each); integrator outputs within 1e-5 relative to each output channel's magnitude,
max|gpu - ref| <= 1e-5 * max over rays of |ref| (column-wise max norm).  Both sides evaluate the
reference's arithmetic with one rounding per operation, but CUDA's expf and the C library's may
differ in the last ulp, and in alpha = 1 - exp(-sigma*ds) that ulp is a relative error of up to
~1e-4 when sigma*ds is small; elementwise relative errors on nearly transparent rays are therefore
not a meaningful bar, errors relative to the quantity's scale are.
"""
import numpy as np
import pytest
import torch

from golden_inputs import make_rays, random_bitfield
from oracle import volrend as V
from tests.golden_util import load

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def dev(a, dtype=None):
    a = np.asarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


def host(t):
    a = t.detach().cpu().numpy()
    return a.view(np.uint32) if a.dtype == np.int32 else a


def assert_close(a, b, rtol=RTOL, mask=None):
    """max|a - b| <= rtol * max|b|, per column (the last axis of a 2-D array)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape
    if mask is not None:
        a, b = a[mask], b[mask]
    if a.size == 0:
        return
    scale = np.abs(b).max(axis=0) if b.ndim > 1 else np.abs(b).max()
    err = np.abs(a - b).max(axis=0) / np.maximum(scale, 1e-30)
    assert np.max(err) <= rtol, f"max rel err {np.max(err)}"


def away_from_threshold(opacity, rtol=1e-3):
    """Rays whose final transmittance is not within `rtol` of the 1e-4 early-stop threshold.  On
    a ray that ends right at the threshold the output formula switches (normalised by opacity vs.
    blended over the background), so a last-ulp difference anywhere on the ray moves the result by
    ~1e-4; any two float32 evaluations can disagree there."""
    T = 1.0 - np.asarray(opacity, np.float64)
    return np.abs(T / 1e-4 - 1.0) > rtol


@pytest.fixture(scope="module")
def vr():
    from jaxngp_gb300 import volrendjax
    return volrendjax


def run_march(vr, z, total):
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), counters = vr.march_rays(
        total, int(z["diagonal_n_steps"]), int(z["K"]), int(z["G"]), float(z["bound"]),
        float(z["stepsize_portion"]), dev(z["rays_o"]), dev(z["rays_d"]), dev(z["t_starts"]), dev(z["t_ends"]),
        dev(z["noises"]), dev(z["bitfield"]), return_counters=True)
    return [host(x) for x in (m, valid, ns, st, idcs, xyzs, dirs, dss, zs)], host(counters)


def test_packbits_morton_golden(vr):
    z = load("volrend_packbits_morton")
    mask, bits = vr.packbits(float(z["threshold"]), dev(z["density"]))
    assert np.array_equal(host(mask), z["mask"]) and np.array_equal(host(bits), z["bits"])
    thr_arr = np.full_like(z["density"], z["threshold"])
    mask, bits = vr.packbits(dev(thr_arr), dev(z["density"]))
    assert np.array_equal(host(mask), z["mask"]) and np.array_equal(host(bits), z["bits"])
    assert np.array_equal(host(vr.morton3d(dev(z["xyz"]))), z["codes"])
    assert np.array_equal(host(vr.morton3d_invert(dev(z["codes_in"]))), z["inv"])


@pytest.mark.parametrize("tag", ["k1", "k2", "empty", "full"])
def test_march_rays_golden(vr, tag):
    """Per-ray results bit-exact against the reference's kernel.  The GPU's slot order follows
    its warps' atomics, so samples are compared ray by ray, not by flat position."""
    z = load(f"volrend_march_{tag}")
    total = 1 << 18
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), counters = run_march(vr, z, total)
    assert np.array_equal(counters, z["counters"]) and m == z["counters"][0] - z["counters"][1]
    assert np.array_equal(valid, z["ray_is_valid"]) and np.array_equal(ns, z["rays_n_samples"])
    used = int(z["counters"][0])
    for r in np.nonzero(ns)[0]:
        a, b = st[r], z["rays_sample_startidx"][r]
        n = ns[r]
        assert np.all(idcs[a:a + n] == r) and np.all(z["idcs"][b:b + n] == r)
        for name, x in [("xyzs", xyzs), ("dirs", dirs), ("dss", dss), ("z_vals", zs)]:
            assert np.array_equal(x[a:a + n], z[name][b:b + n]), (r, name)
    # slots are a permutation of [0, used) and the tail is zero
    covered = np.zeros(total, bool)
    for r in np.nonzero(ns)[0]:
        assert not covered[st[r]:st[r] + ns[r]].any()
        covered[st[r]:st[r] + ns[r]] = True
    assert covered[:used].all() and not covered[used:].any()
    assert not idcs[used:].any() and not xyzs[used:].any() and not dss[used:].any() and not zs[used:].any()


@pytest.mark.parametrize("seed,K,G,bound,sp,n", [(0, 1, 128, 1.0, 0.0, 20000), (1, 3, 64, 4.0, 1 / 256, 8000),
                                                 (2, 5, 32, 16.0, 6e-3, 4000)])
def test_march_rays_vs_oracle(vr, seed, K, G, bound, sp, n):
    rng = np.random.default_rng(seed)
    o, d, t0, t1 = make_rays(rng, n, bound)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, K, G, 0.25)
    total = 1 << 23
    a = V.march_rays(total, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits)
    z = dict(diagonal_n_steps=1024, K=K, G=G, bound=bound, stepsize_portion=sp, rays_o=o, rays_d=d, t_starts=t0,
             t_ends=t1, noises=noise, bitfield=bits)
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), _ = run_march(vr, z, total)
    assert m == a[0]
    assert np.array_equal(valid, a[1]) and np.array_equal(ns, a[2])
    for r in np.nonzero(ns)[0][:: max(1, len(np.nonzero(ns)[0]) // 500)]:
        x0, y0, k = st[r], a[3][r], ns[r]
        assert np.array_equal(xyzs[x0:x0 + k], a[5][y0:y0 + k])
        assert np.array_equal(zs[x0:x0 + k], a[8][y0:y0 + k])
        assert np.array_equal(dss[x0:x0 + k], a[7][y0:y0 + k])


def test_march_rays_overflow(vr):
    """A sample budget below demand: the drop-in march gives the reference kernel's result under
    its one-at-a-time ray-order schedule (every buffer and both counters), so nothing past
    `measured` is written and the counters obey measured = next - exceeded."""
    rng = np.random.default_rng(3)
    n = 4096
    o, d, t0, t1 = make_rays(rng, n, 1.0)
    bits = random_bitfield(rng, 1, 64, 0.5)
    full = V.march_rays(1 << 24, 1024, 1, 64, 1.0, 0.0, o, d, t0, t1, 0.5, bits)
    total = int(full[2].sum() // 3)
    z = dict(diagonal_n_steps=1024, K=1, G=64, bound=1.0, stepsize_portion=0.0, rays_o=o, rays_d=d, t_starts=t0,
             t_ends=t1, noises=np.full(n, 0.5, np.float32), bitfield=bits)
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), counters = run_march(vr, z, total)
    assert counters[1] > 0 and m == counters[0] - counters[1] and m <= total
    assert ns.sum() == m
    fit = ns > 0
    assert np.array_equal(ns[fit], full[2][fit])  # rays that fit carry their full sample run
    assert not idcs[m:].any() and not zs[m:].any()
    a, ca = V.march_rays(total, 1024, 1, 64, 1.0, 0.0, o, d, t0, t1, np.full(n, 0.5, np.float32), bits,
                         return_counters=True, early_exit=True)
    assert np.array_equal(counters, ca)
    for x, y in zip((valid, ns, st, idcs, xyzs, dirs, dss, zs), a[1:]):
        assert np.array_equal(x, y)


def test_march_rays_inference_golden(vr):
    z = load("volrend_march_inference")
    for k in range(2):
        r = vr.march_rays_inference(int(z["diagonal_n_steps"]), int(z["K"]), int(z["G"]), int(z["cap"]),
                                    float(z["bound"]), float(z["stepsize_portion"]), dev(z["rays_o"]),
                                    dev(z["rays_d"]), dev(z[f"it{k}_t_starts_in"]), dev(z["t_ends"]),
                                    dev(z["bitfield"]), dev(z[f"it{k}_next_ray_index_in"]),
                                    dev(z[f"it{k}_terminated_in"]), dev(z[f"it{k}_indices_in"]))
        nri, idx, ns, t_new, xyzs, dss, zs = [host(x) for x in r]
        assert np.array_equal(nri, z[f"it{k}_next_ray_index"])
        assert np.array_equal(t_new, z[f"it{k}_t_starts"])
        # refilled slots may receive their rays in a different order: compare per ray index
        ref_slot = {int(r_): s for s, r_ in enumerate(z[f"it{k}_indices"])}
        assert sorted(ref_slot) == sorted(int(x) for x in idx)
        for s, r_ in enumerate(idx):
            q = ref_slot[int(r_)]
            assert ns[s] == z[f"it{k}_n_samples"][q]
            for name, x in [("xyzs", xyzs), ("dss", dss), ("z_vals", zs)]:
                assert np.array_equal(x[s], z[f"it{k}_{name}"][q]), (k, s, name)


def test_integrate_golden(vr):
    z = load("volrend_integrate")
    st, ns = dev(z["rays_sample_startidx"]), dev(z["rays_n_samples"])
    bgs, dss, zs = dev(z["bgs"]), dev(z["dss"]), dev(z["z_vals"])
    drgbs = dev(z["drgbs"]).requires_grad_(True)
    zs.requires_grad_(True)
    bgs.requires_grad_(True)
    m, rgbd, opac = vr.integrate_rays(float(z["near_distance"]), st, ns, bgs, dss, zs, drgbs)
    assert int(host(m)) == int(z["measured_batch_size"])
    ok = away_from_threshold(z["final_opacities"])
    assert ok.mean() > 0.99
    assert_close(host(rgbd), z["final_rgbds"], mask=ok)
    assert_close(host(opac), z["final_opacities"])
    torch.autograd.backward(rgbd, dev(z["dL_dfinal_rgbds"]))
    assert_close(host(bgs.grad), z["dL_dbgs"], mask=ok)
    ok_s = np.repeat(ok, z["rays_n_samples"].astype(np.int64))
    assert_close(host(zs.grad), z["dL_dz_vals"], mask=ok_s)
    assert_close(host(drgbs.grad), z["dL_ddrgbs"], mask=ok_s)


def test_integrate_inference_golden(vr):
    z = load("volrend_integrate_inference")
    cnt, term, rgbd, T = vr.integrate_rays_inference(dev(z["rays_bg"]), dev(z["rays_rgbd"]), dev(z["rays_T"]),
                                                     dev(z["n_samples"]), dev(z["indices"]), dev(z["dss"]),
                                                     dev(z["z_vals"]), dev(z["drgbs"]))
    assert int(host(cnt)) == int(z["terminate_cnt"])
    assert np.array_equal(host(term), z["terminated"])
    assert_close(host(rgbd), z["rays_rgbd_out"])
    assert_close(host(T), z["rays_T_out"])


def test_integrate_vs_oracle_large(vr):
    rng = np.random.default_rng(9)
    n = 1 << 16
    ns = rng.integers(0, 160, size=n).astype(np.uint32)
    st = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.uint32)
    S = int(ns.sum())
    dss = rng.uniform(0.001, 0.02, S).astype(np.float32)
    zs = (np.cumsum(dss) % 4.0).astype(np.float32)
    drgbs = np.concatenate([rng.exponential(10, (S, 1)), rng.uniform(size=(S, 3))], -1).astype(np.float32)
    bgs = rng.uniform(size=(n, 3)).astype(np.float32)
    a = V.integrate_rays(0.3, st, ns, bgs, dss, zs, drgbs)
    m, rgbd, opac = vr.integrate_rays(0.3, dev(st), dev(ns), dev(bgs), dev(dss), dev(zs), dev(drgbs))
    assert abs(int(host(m)) - int(a[0])) <= 2  # an early-stop step may move on a threshold ray
    ok = away_from_threshold(a[2])
    assert ok.mean() > 0.99
    assert_close(host(rgbd), a[1], mask=ok)
    assert_close(host(opac), a[2])


def test_error_statuses(vr):
    """Bad descriptors and shapes are reported as errors before any kernel runs."""
    from jaxngp_gb300 import _lib as L
    with pytest.raises(L.NgpError) as e:
        L.call("march_rays", [None] * 16, L.Morton3DDescriptor(4))  # wrong opaque length
    assert e.value.status == 1
    x = torch.zeros(7, dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        vr.packbits(0.5, x)  # not divisible by 8
    z = load("volrend_march_k1")
    with pytest.raises(ValueError):
        vr.march_rays(1024, 1024, 2, int(z["G"]), 1.0, 0.0, dev(z["rays_o"]), dev(z["rays_d"]), dev(z["t_starts"]),
                      dev(z["t_ends"]), 0.0, dev(z["bitfield"]))  # bitfield size mismatch for K=2
    desc = L.MarchingDescriptor(4, 16, 1024, 0, 16, 1.0, 0.0)  # K = 0 (ffi.cc:78-80)
    with pytest.raises(L.NgpError) as e:
        L.call("march_rays", [None] * 16, desc)
    assert e.value.status == 2
    # the legacy signature reports through ngp_last_status
    import ctypes
    lib = L.lib()
    arr = (ctypes.c_void_p * 16)()
    lib.march_rays(ctypes.c_void_p(0), arr, ctypes.c_char_p(b"xx"), ctypes.c_size_t(2))
    assert lib.ngp_last_status() == 1


def test_empty_inputs(vr):
    z = load("volrend_march_k1")
    e3 = torch.zeros(0, 3, dtype=torch.float32, device="cuda")
    e1 = torch.zeros(0, dtype=torch.float32, device="cuda")
    m, valid, ns, st, idcs, xyzs, dirs, dss, zs = vr.march_rays(64, 1024, 1, int(z["G"]), 1.0, 0.0, e3, e3, e1, e1,
                                                                0.0, dev(z["bitfield"]))
    assert int(host(m)) == 0 and valid.numel() == 0 and not host(idcs).any()
    ei = torch.zeros(0, dtype=torch.int32, device="cuda")
    m, rgbd, opac = vr.integrate_rays(0.3, ei, ei, torch.zeros(0, 3, device="cuda"), e1, e1,
                                      torch.zeros(0, 4, device="cuda"))
    assert int(host(m)) == 0 and rgbd.shape == (0, 4)


def test_march_rays_inference_multiwarp_vs_oracle(vr):
    """Many warps, a mix of finished and running slots, several refill rounds: the set of rays in
    flight and each ray's samples and advanced t match the oracle ray by ray."""
    rng = np.random.default_rng(11)
    n_total, n_slots, cap, G = 6000, 1024, 8, 64
    o, d, t0, t1 = make_rays(rng, n_total, 1.0)
    bits = random_bitfield(rng, 1, G, 0.15)
    term_h = np.ones(n_slots, bool)
    idx_h = np.zeros(n_slots, np.uint32)
    nri_h = np.zeros(1, np.uint32)
    t_h = t0.copy()
    for it in range(4):
        ref = V.march_rays_inference(1024, 1, G, cap, 1.0, 0.0, o, d, t_h, t1, bits, nri_h, term_h, idx_h)
        r = vr.march_rays_inference(1024, 1, G, cap, 1.0, 0.0, dev(o), dev(d), dev(t_h), dev(t1), dev(bits),
                                    dev(nri_h), dev(term_h), dev(idx_h))
        nri, idx, ns, t_new, xyzs, dss, zs = [host(x) for x in r]
        assert np.array_equal(nri, ref[0])
        assert np.array_equal(t_new, ref[3])
        assert sorted(idx.tolist()) == sorted(ref[1].tolist())
        pos = {int(v): s for s, v in enumerate(ref[1])}
        for s, v in enumerate(idx):
            q = pos[int(v)]
            assert ns[s] == ref[2][q]
            assert np.array_equal(xyzs[s], ref[4][q]) and np.array_equal(zs[s], ref[6][q])
        # follow the oracle's state into the next round
        term_h = ref[2] < cap
        term_h[rng.uniform(size=n_slots) < 0.2] = True
        idx_h, nri_h, t_h = ref[1], ref[0], ref[3]


def _march_train(z, total, coarse=None, queue=None):
    from jaxngp_gb300 import _lib as L
    n = z["rays_o"].shape[0]
    i32 = dict(dtype=torch.int32, device="cuda")
    out = [torch.zeros(1, **i32), torch.zeros(1, **i32), torch.empty(n, dtype=torch.bool, device="cuda"),
           torch.empty(n, **i32), torch.empty(n, **i32), torch.empty(total, **i32),
           torch.empty(total, 3, device="cuda"), torch.empty(total, 3, device="cuda"), torch.empty(total, device="cuda"),
           torch.empty(total, device="cuda")]
    queue = torch.zeros(1, **i32) if queue is None else queue
    d = L.MarchingDescriptor(n, total, int(z["diagonal_n_steps"]), int(z["K"]), int(z["G"]), float(z["bound"]),
                             float(z["stepsize_portion"]))
    L.call("ngp_march_rays_train", [dev(z["rays_o"]), dev(z["rays_d"]), dev(z["t_starts"]), dev(z["t_ends"]),
                                    dev(z["noises"]), dev(z["bitfield"])] + out + [queue, coarse], d)
    return [host(x) for x in out]


def _assert_sequential(z, total, got):
    """ngp_march_rays_train's buffers and counters equal, bit for bit, the reference kernel's run
    one thread at a time in ray order (the oracle's march with early_exit: a ray that starts
    after the buffer filled is dropped, marching.cu:135)."""
    (m, valid, ns, st, idcs, xyzs, dirs, dss, zs), cnt = V.march_rays(
        total, z["diagonal_n_steps"], z["K"], z["G"], z["bound"], z["stepsize_portion"], z["rays_o"], z["rays_d"],
        z["t_starts"], z["t_ends"], z["noises"], z["bitfield"], return_counters=True, early_exit=True)
    c0, c1 = int(got[0][0]), int(got[1][0])
    assert (c0, c1) == (int(cnt[0]), int(cnt[1]))
    for name, x, y in zip(("valid", "n_samples", "startidx", "idcs", "xyzs", "dirs", "dss", "z_vals"), got[2:],
                          (valid, ns, st, idcs, xyzs, dirs, dss, zs)):
        assert np.array_equal(x, y), name
    return ns, valid


def _first_cut(full_n, live, total):
    """The first ray the one-at-a-time schedule drops or cannot fit, or None."""
    prefix = np.concatenate([[0], np.cumsum(full_n.astype(np.int64))[:-1]])
    cut = (prefix >= total) | ((full_n > 0) & (prefix + full_n > total))
    idx = np.nonzero(cut)[0]
    return int(idx[0]) if idx.size else None


@pytest.mark.parametrize("budget_frac", [None, 0.3, 0.02])
def test_march_rays_train_variant(vr, budget_frac):
    """The training marcher is the reference kernel under the one-at-a-time ray-order schedule:
    without overflow it is the plain march, with overflow the rays before the budget filled keep
    their results, the one that does not fit is invalid with its samples left out, and every later
    ray is dropped.  Every buffer and both counters equal the oracle's, and two runs agree."""
    rng = np.random.default_rng(21)
    n = 6000
    o, d, t0, t1 = make_rays(rng, n, 1.0)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, 1, 64, 0.3)
    full_n = V.march_rays(1 << 24, 1024, 1, 64, 1.0, 0.0, o, d, t0, t1, noise, bits)[2]
    total = (1 << 24) if budget_frac is None else max(1, int(full_n.sum() * budget_frac))
    z = dict(diagonal_n_steps=1024, K=1, G=64, bound=1.0, stepsize_portion=0.0, rays_o=o, rays_d=d, t_starts=t0,
             t_ends=t1, noises=noise, bitfield=bits)
    got = _march_train(z, total)
    ns, valid = _assert_sequential(z, total, got)
    if budget_frac is None:
        assert np.array_equal(ns, full_n)
    else:
        q = _first_cut(full_n, t1 > t0, total)
        assert q is not None and not valid[q:].any() and (ns[:q] == full_n[:q]).all()
    again = _march_train(z, total)
    for x, y in zip(again, got):
        assert np.array_equal(x, y)


def test_march_rays_train_many_chunks(vr):
    """A batch of many more rays than fit (2^17 rays, a budget of 1% of their samples), with the
    leading rays' launch covering the fit, short of it, or sized by a first call: the result is
    the one-at-a-time schedule's, bit for bit, and the call leaves its first dropped or unfit ray
    in the queue word."""
    rng = np.random.default_rng(23)
    n = 1 << 17
    o, d, t0, t1 = make_rays(rng, n, 1.0)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, 1, 64, 0.3)
    full_n = V.march_rays(1 << 26, 1024, 1, 64, 1.0, 0.0, o, d, t0, t1, noise, bits, early_exit=False)[2]
    total = int(full_n.astype(np.int64).sum() // 100)
    z = dict(diagonal_n_steps=1024, K=1, G=64, bound=1.0, stepsize_portion=0.0, rays_o=o, rays_d=d, t_starts=t0,
             t_ends=t1, noises=noise, bitfield=bits)
    q = _first_cut(full_n, t1 > t0, total)
    assert q is not None and q > 1024
    queue = torch.zeros(1, dtype=torch.int32, device="cuda")
    # a first call (8192 leading rays), the word it leaves (1.25 q + 512), and a word that makes
    # the lead fall short (513 rays: the rest find the budget full only as the frontier moves)
    for word in (0, None, 1):
        if word is not None:
            queue.fill_(word)
        got = _march_train(z, total, queue=queue)
        assert int(queue[0]) == q
        _assert_sequential(z, total, got)
        print(f"queue word {word}: {int(got[0][0])} samples requested, {int((got[3] > 0).sum())} of {n} rays fit, "
              f"first cut at ray {q}")


@pytest.mark.parametrize("budget_frac", [None, 0.3])
def test_march_rays_train_coarse_shortcut(vr, budget_frac):
    """With coarse occupancy blocks the training marcher finishes rays that cross no occupied
    block at once and crosses empty blocks in one step; on a grid of a few blobs (most rays miss
    them) every buffer is still the one-at-a-time schedule's, bit for bit, and the same as without
    the coarse grid."""
    from jaxngp_gb300 import _lib as L
    from tests.test_oracle_proposal import blob_bitfield
    rng = np.random.default_rng(22)
    n, G = 8000, 128
    o, d, t0, t1 = make_rays(rng, n, 1.0)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = blob_bitfield(G, [(0.3, -0.2, 0.1), (-0.4, 0.35, -0.3), (0.05, 0.5, -0.5)], 0.12)
    full_n = V.march_rays(1 << 24, 1024, 1, G, 1.0, 0.0, o, d, t0, t1, noise, bits, early_exit=False)[2]
    assert (full_n == 0).mean() > 0.3 and (full_n > 0).sum() > 100
    coarse = torch.zeros((G // 8) ** 3, dtype=torch.uint8, device="cuda")
    L.call("ngp_proposal_coarse", [dev(bits), coarse],
           L.NgpProposalDescriptor(0, 48, G, 1.0, 0, 0, 0, 3, 1, 0, 0.1))
    total = (1 << 24) if budget_frac is None else max(1, int(full_n.sum() * budget_frac))
    z = dict(diagonal_n_steps=1024, K=1, G=G, bound=1.0, stepsize_portion=0.0, rays_o=o, rays_d=d, t_starts=t0,
             t_ends=t1, noises=noise, bitfield=bits)
    with_c = _march_train(z, total, coarse)
    _assert_sequential(z, total, with_c)
    without = _march_train(z, total)
    for x, y in zip(with_c, without):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("n_blobs,radius,cam", [(3, 0.12, 4.0), (20, 0.1, 4.0), (60, 0.08, 4.0), (20, 0.1, 2.0)])
def test_march_block_skip_bitexact(vr, n_blobs, radius, cam):
    """The coarse grid's one-step skip over empty 8^3 blocks lands where the reference's cell-by-cell
    march lands: every ray's validity, count and every sample (position, step, t) equal the oracle's
    bit for bit, for rays from cameras at radius `cam` (t then crosses the power of two at 4 or 2,
    where the skip must fall back) over grids of blobs from sparse to dense."""
    from jaxngp_gb300 import _lib as L
    from golden_inputs import near_far
    from tests.test_oracle_proposal import blob_bitfield
    rng = np.random.default_rng(100 + n_blobs)
    n, G = 12000, 128
    o = rng.normal(size=(n, 3))
    o = (o / np.linalg.norm(o, axis=-1, keepdims=True) * cam).astype(np.float32)
    tgt = rng.uniform(-0.9, 0.9, size=(n, 3))
    d = tgt - o
    d = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    t0, t1 = near_far(1.0, o, d)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = blob_bitfield(G, [tuple(c) for c in rng.uniform(-0.7, 0.7, size=(n_blobs, 3))], radius)
    ref = V.march_rays(1 << 24, 1024, 1, G, 1.0, 0.0, o, d, t0, t1, noise, bits, early_exit=False)
    coarse = torch.zeros((G // 8) ** 3, dtype=torch.uint8, device="cuda")
    L.call("ngp_proposal_coarse", [dev(bits), coarse], L.NgpProposalDescriptor(0, 48, G, 1.0, 0, 0, 0, 3, 1, 0, 0.1))
    empty_blocks = float((coarse == 0).float().mean())
    z = dict(diagonal_n_steps=1024, K=1, G=G, bound=1.0, stepsize_portion=0.0, rays_o=o, rays_d=d, t_starts=t0,
             t_ends=t1, noises=noise, bitfield=bits)
    c0, c1, valid, ns, st, idcs, xyzs, dirs, dss, zs = _march_train(z, 1 << 24, coarse)
    assert np.array_equal(valid, ref[1]) and np.array_equal(ns, ref[2])
    has = np.nonzero(ns)[0]
    og = np.concatenate([np.arange(st[r], st[r] + ns[r]) for r in has])
    orf = np.concatenate([np.arange(ref[3][r], ref[3][r] + ns[r]) for r in has])
    for a_, b_ in ((xyzs, ref[5]), (dss, ref[7]), (zs, ref[8])):
        assert np.array_equal(a_[og], b_[orf])
    print(f"\nblock skip: {n_blobs} blobs, camera radius {cam}: empty coarse blocks {empty_blocks:.2f}, "
          f"rays with samples {len(has)}, samples {int(ns.sum())}")


def _march_list(o, d, t0, t1, noise, bits, listed, n, total, K, G, bound, sp, start_at=17):
    """ngp_march_rays_fallback over `listed`; counters start at (start_at, 0), ray outputs at -1."""
    from jaxngp_gb300 import _lib as L
    i32 = dict(dtype=torch.int32, device="cuda")
    ctr = torch.tensor([start_at, 0], **i32)
    out = [torch.zeros(n, dtype=torch.bool, device="cuda"), torch.full((n,), -1, **i32), torch.full((n,), -1, **i32),
           torch.zeros(total, **i32), torch.zeros(total, 3, device="cuda"), torch.zeros(total, 3, device="cuda"),
           torch.zeros(total, device="cuda"), torch.zeros(total, device="cuda")]
    extra = [torch.zeros(1, **i32), dev(listed), torch.tensor([len(listed)], **i32)]
    L.call("ngp_march_rays_fallback", [dev(o), dev(d), dev(t0), dev(t1), dev(noise), dev(bits), ctr[0:1], ctr[1:2]]
           + out + extra, L.MarchingDescriptor(n, total, 1024, K, G, bound, sp))
    return host(ctr), [host(x) for x in out]


@pytest.mark.parametrize("K,G,bound,sp,occ", [(1, 128, 1.0, 0.0, 0.3), (1, 64, 1.0, 0.0, 1.0),
                                              (3, 64, 4.0, 1 / 256, 0.25)])
def test_march_list_vs_oracle(K, G, bound, sp, occ):
    """The list form of the training march (a warp per listed ray, 32-step lookahead): every listed
    ray's count, validity and samples are the oracle march's bit for bit -- through a fully
    occupied grid (runs of up to 1024 samples) and with cascades and a t-dependent step too; slots
    are allocated after what the counters already hold; rays not listed are left alone."""
    rng = np.random.default_rng(40 + K + G)
    n = 3000
    o, d, t0, t1 = make_rays(rng, n, bound)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, K, G, occ)
    total = 1 << 22
    a = V.march_rays(total, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits)
    listed = rng.permutation(n)[:1000].astype(np.uint32)
    ctr, (valid, ns, st, idcs, X, _, Ds, Z) = _march_list(o, d, t0, t1, noise, bits, listed, n, total, K, G, bound, sp)
    unlisted = np.setdiff1d(np.arange(n), listed)
    assert (ns[unlisted] == 0xFFFFFFFF).all() and (st[unlisted] == 0xFFFFFFFF).all()
    assert np.array_equal(valid[listed], a[1][listed]) and np.array_equal(ns[listed], a[2][listed])
    assert ctr[0] == 17 + a[2][listed].sum() and ctr[1] == 0
    if occ == 1.0:
        assert a[2][listed].max() > 256
    for r in listed[a[2][listed] > 0]:
        x0, y0, k = st[r], a[3][r], ns[r]
        assert x0 >= 17 and (idcs[x0:x0 + k] == r).all()
        assert np.array_equal(Z[x0:x0 + k], a[8][y0:y0 + k]) and np.array_equal(Ds[x0:x0 + k], a[7][y0:y0 + k])
        assert np.array_equal(X[x0:x0 + k], a[5][y0:y0 + k])


def test_march_list_over_budget():
    """A budget of half the listed rays' demand: each listed ray is either valid with exactly the
    oracle's samples inside the budget, or invalid with none; the counters keep
    next - exceeded = the samples written."""
    rng = np.random.default_rng(77)
    n, K, G = 3000, 1, 128
    o, d, t0, t1 = make_rays(rng, n, 1.0)
    noise = rng.uniform(size=n).astype(np.float32)
    bits = random_bitfield(rng, K, G, 0.3)
    a = V.march_rays(1 << 22, 1024, K, G, 1.0, 0.0, o, d, t0, t1, noise, bits)
    listed = rng.permutation(n)[:1500].astype(np.uint32)
    total = int(a[2][listed].sum()) // 2
    ctr, (valid, ns, st, _, _, _, _, Z) = _march_list(o, d, t0, t1, noise, bits, listed, n, total, K, G, 1.0, 0.0,
                                                      start_at=0)
    written = 0
    for r in listed:
        if valid[r] and ns[r] > 0:
            assert ns[r] == a[2][r] and st[r] + ns[r] <= total
            assert np.array_equal(Z[st[r]:st[r] + ns[r]], a[8][a[3][r]:a[3][r] + a[2][r]])
            written += int(ns[r])
        elif not valid[r]:   # over the budget (or, as in the oracle, an empty interval)
            assert ns[r] == 0 and (a[2][r] > 0 or not a[1][r])
    assert 0 < written <= total and int(ctr[0]) - int(ctr[1]) == written
