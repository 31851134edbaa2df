"""The CPU oracle against the golden fixtures made from the reference's own code, and against the
reference's kernels compiled for the CPU on fresh random cases (where the checkout exists)."""
import numpy as np
import pytest

from golden_inputs import (FIELD_CASE, HASHGRID_CASES, field_inputs, hashgrid_inputs, make_rays,
                           random_bitfield)
from oracle import field as Fd
from oracle import hashgrid as H
from oracle import volrend as V

from tests.golden_util import load


def test_packbits_morton_golden():
    z = load("volrend_packbits_morton")
    mask, bits = V.packbits(z["threshold"], z["density"])
    assert np.array_equal(mask, z["mask"]) and np.array_equal(bits, z["bits"])
    assert np.array_equal(V.morton3d(z["xyz"]), z["codes"])
    assert np.array_equal(V.morton3d_invert(z["codes_in"]), z["inv"])
    assert np.array_equal(V.morton3d_invert(z["codes"]), z["xyz"])


@pytest.mark.parametrize("tag", ["k1", "k2", "empty", "full"])
def test_march_rays_golden(tag):
    z = load(f"volrend_march_{tag}")
    out, counters = V.march_rays(1 << 18, int(z["diagonal_n_steps"]), int(z["K"]), int(z["G"]),
                                 float(z["bound"]), float(z["stepsize_portion"]), z["rays_o"],
                                 z["rays_d"], z["t_starts"], z["t_ends"], z["noises"], z["bitfield"],
                                 return_counters=True)
    m, valid, ns, st, idcs, xyzs, dirs, dss, zs = out
    used = int(z["counters"][0])
    assert np.array_equal(counters, z["counters"])
    assert m == z["counters"][0] - z["counters"][1]
    for name, a in [("ray_is_valid", valid), ("rays_n_samples", ns), ("rays_sample_startidx", st)]:
        assert np.array_equal(a, z[name]), name
    for name, a in [("idcs", idcs), ("xyzs", xyzs), ("dirs", dirs), ("dss", dss), ("z_vals", zs)]:
        assert np.array_equal(a[:used], z[name]), name
        assert not np.any(a[used:]), name


def test_march_rays_inference_golden():
    z = load("volrend_march_inference")
    for k in range(2):
        r = V.march_rays_inference(int(z["diagonal_n_steps"]), int(z["K"]), int(z["G"]),
                                   int(z["cap"]), float(z["bound"]), float(z["stepsize_portion"]),
                                   z["rays_o"], z["rays_d"], z[f"it{k}_t_starts_in"], z["t_ends"],
                                   z["bitfield"], z[f"it{k}_next_ray_index_in"],
                                   z[f"it{k}_terminated_in"], z[f"it{k}_indices_in"])
        names = ["next_ray_index", "indices", "n_samples", "t_starts", "xyzs", "dss", "z_vals"]
        for name, a in zip(names, r):
            assert np.array_equal(a, z[f"it{k}_{name}"]), (k, name)


def test_integrate_golden():
    z = load("volrend_integrate")
    args = (z["near_distance"], z["rays_sample_startidx"], z["rays_n_samples"], z["bgs"], z["dss"],
            z["z_vals"], z["drgbs"])
    m, rgbd, opac = V.integrate_rays(*args)
    assert m == z["measured_batch_size"]
    assert np.array_equal(rgbd, z["final_rgbds"]) and np.array_equal(opac, z["final_opacities"])
    gb, gz, gc = V.integrate_rays_backward(*args, rgbd, opac, z["dL_dfinal_rgbds"])
    assert np.array_equal(gb, z["dL_dbgs"])
    assert np.array_equal(gz, z["dL_dz_vals"])
    assert np.array_equal(gc, z["dL_ddrgbs"])


def test_integrate_inference_golden():
    z = load("volrend_integrate_inference")
    cnt, term, rgbd, T = V.integrate_rays_inference(z["rays_bg"], z["rays_rgbd"], z["rays_T"],
                                                    z["n_samples"], z["indices"], z["dss"],
                                                    z["z_vals"], z["drgbs"])
    assert cnt == z["terminate_cnt"]
    assert np.array_equal(term, z["terminated"])
    assert np.array_equal(rgbd, z["rays_rgbd_out"]) and np.array_equal(T, z["rays_T_out"])


@pytest.mark.parametrize("case", HASHGRID_CASES, ids=lambda c: c["tag"])
def test_hashgrid_golden(case):
    pos, lat, tab, b = hashgrid_inputs(case)
    enc = H.encode(pos, lat, b, tab)
    assert np.array_equal(enc, load(f"hashgrid_{case['tag']}")["encodings"])


def test_field_golden():
    pos, dirs, lat, w, tab, b = field_inputs(FIELD_CASE)
    z = load("field_ngp")
    enc = H.encode(pos, lat, b, tab)
    drgb, _ = Fd.forward(enc, dirs, w)
    np.testing.assert_allclose(drgb, z["drgb"], rtol=1e-6, atol=0)
    np.testing.assert_allclose(Fd.density_only(enc, w), z["density"][:, 0], rtol=1e-6, atol=0)


def test_level_tables():
    """encoders.py:89-114 at the training configuration: 5 dense levels, P = 6,098,120."""
    t = H.LevelTable(16, 2**19, 2, 16, 2048)
    assert t.first_hash_level == 5 and t.n_params == 6098120
    assert abs(t.b - 1.3819128800) < 1e-9
    t2 = H.LevelTable(16, 2**19, 2, 16, 2048, per_level_scale=1.447)
    assert t2.n_params == 6299960


# ------------------------------------------------- fresh random cases against the reference build

@pytest.mark.parametrize("seed,K,G,bound,sp", [(0, 1, 64, 1.0, 0.0), (1, 3, 32, 4.0, 1 / 256),
                                               (2, 2, 16, 1.5, 5e-3)])
def test_march_oracle_vs_reference(ref_backend, seed, K, G, bound, sp):
    rng = np.random.default_rng(seed)
    o, d, t0, t1 = make_rays(rng, 1500, bound)
    noise = rng.uniform(size=1500).astype(np.float32)
    bits = random_bitfield(rng, K, G, 0.3)
    a = V.march_rays(1 << 22, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits)
    b = V.march_rays(1 << 22, 1024, K, G, bound, sp, o, d, t0, t1, noise, bits, backend="ref")
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_march_overflow_oracle_vs_reference(ref_backend):
    """Sample budget smaller than the demand: overflowed rays and the early exit (marching.cu:135,
    :205-209), with ray-order atomics."""
    rng = np.random.default_rng(5)
    o, d, t0, t1 = make_rays(rng, 2000, 1.0)
    bits = random_bitfield(rng, 1, 32, 0.5)
    a, ca = V.march_rays(20000, 1024, 1, 32, 1.0, 0.0, o, d, t0, t1, 0.5, bits, return_counters=True)
    b, cb = V.march_rays(20000, 1024, 1, 32, 1.0, 0.0, o, d, t0, t1, 0.5, bits, backend="ref",
                         return_counters=True)
    assert np.array_equal(ca, cb) and ca[1] > 0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_integrate_oracle_vs_reference(ref_backend):
    rng = np.random.default_rng(7)
    n = 2048
    ns = rng.integers(0, 200, size=n).astype(np.uint32)
    st = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.uint32)
    S = int(ns.sum())
    dss = rng.uniform(0.001, 0.02, S).astype(np.float32)
    zs = np.cumsum(dss).astype(np.float32) * 0.3
    drgbs = np.concatenate([rng.exponential(20, (S, 1)), rng.uniform(size=(S, 3))], -1).astype(np.float32)
    bgs = rng.uniform(size=(n, 3)).astype(np.float32)
    a = V.integrate_rays(0.3, st, ns, bgs, dss, zs, drgbs)
    b = V.integrate_rays(0.3, st, ns, bgs, dss, zs, drgbs, backend="ref")
    assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    g = rng.normal(size=(n, 4)).astype(np.float32)
    ga = V.integrate_rays_backward(0.3, st, ns, bgs, dss, zs, drgbs, a[1], a[2], g)
    gb = V.integrate_rays_backward(0.3, st, ns, bgs, dss, zs, drgbs, a[1], a[2], g, backend="ref")
    for x, y in zip(ga, gb):
        assert np.array_equal(x, y)
