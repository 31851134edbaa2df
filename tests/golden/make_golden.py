"""Generate the golden fixtures in tests/golden/ from the reference's own code.

TEST INFRASTRUCTURE ONLY; run in a container that holds the reference checkout:

    python tests/golden/make_golden.py REFERENCE_ROOT [volrend] [field] [tv] [sh]

(REFERENCE_ROOT may be left out when the environment variable NGP_REFERENCE_ROOT names it.)

* ``volrend_*.npz``: inputs and outputs of the reference's ``marching.cu``, ``integrating.cu`` and
  ``packbits.cu`` kernels, compiled for the CPU by ``oracle/build_ref.sh`` and run thread by
  thread (one rounding per floating-point operation).
* ``hashgrid_*.npz`` and ``field_*.npz``: outputs of the reference's ``HashGridEncoder``
  (models/encoders.py) and ``make_nerf_ngp`` field (models/nerfs.py), executed unmodified on the
  NumPy stand-in for jax/flax in ``jax_numpy_shim.py``.
* ``sh_encodings.npz``: the reference's ``SphericalHarmonicsEncoder`` (models/encoders.py) for
  degrees 1..8, run the same way.
* ``tv_*.npz``: the total-variation term the same ``HashGridEncoder`` returns with tv_scale > 0.

``python tests/golden/make_golden.py REF tv`` regenerates only the ``tv_*`` files.

Large inputs (hash tables, MLP weights) are not stored: the tests regenerate them from the seeds
recorded in each file with ``golden_inputs.py``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from golden_inputs import (FIELD_CASE, HASHGRID_CASES, TV_CASES, field_inputs, hashgrid_inputs,  # noqa: E402
                           make_rays, random_bitfield, tv_inputs)


def _save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}: {os.path.getsize(path) / 1024:.1f} KiB")


def volrend(ref_root: str):
    from oracle import volrend as V
    V.build_ref(ref_root)
    rng = np.random.default_rng(1234)

    # packbits / morton
    n_bytes = 4096
    dens = rng.normal(size=n_bytes * 8).astype(np.float32)
    thr = np.float32(0.25)
    mask, bits = V.packbits(thr, dens, backend="ref")
    xyz = rng.integers(0, 1024, size=(8192, 3)).astype(np.uint32)
    codes = V.morton3d(xyz, backend="ref")
    codes_in = rng.integers(0, 2**30, size=8192).astype(np.uint32)
    inv = V.morton3d_invert(codes_in, backend="ref")
    _save("volrend_packbits_morton.npz", density=dens, threshold=np.float32(thr), mask=mask,
          bits=bits, xyz=xyz, codes=codes, codes_in=codes_in, inv=inv)

    # march_rays: three scenes, nothing overflows
    cases = [
        dict(tag="k1", K=1, G=32, bound=1.0, sp=0.0, dns=1024, n=256, density=0.35),
        dict(tag="k2", K=2, G=16, bound=2.0, sp=1 / 256, dns=512, n=256, density=0.5),
        dict(tag="empty", K=1, G=16, bound=1.0, sp=0.0, dns=256, n=64, density=0.0),
        dict(tag="full", K=1, G=16, bound=1.0, sp=0.0, dns=256, n=64, density=1.0),
    ]
    for c in cases:
        o, d, t0, t1 = make_rays(rng, c["n"], c["bound"])
        t0[:3] = t1[:3]  # rays with t_end <= t_start
        noise = rng.uniform(size=c["n"]).astype(np.float32)
        bits = random_bitfield(rng, c["K"], c["G"], c["density"])
        total = 1 << 18
        out, counters = V.march_rays(total, c["dns"], c["K"], c["G"], c["bound"], c["sp"], o, d,
                                     t0, t1, noise, bits, backend="ref", return_counters=True)
        m, valid, ns, st, idcs, xyzs, dirs, dss, zs = out
        used = int(counters[0])
        assert used <= total and counters[1] == 0
        _save(f"volrend_march_{c['tag']}.npz", K=c["K"], G=c["G"], bound=np.float32(c["bound"]),
              stepsize_portion=np.float32(c["sp"]), diagonal_n_steps=c["dns"], rays_o=o, rays_d=d,
              t_starts=t0, t_ends=t1, noises=noise, bitfield=bits, counters=counters,
              ray_is_valid=valid, rays_n_samples=ns, rays_sample_startidx=st, idcs=idcs[:used],
              xyzs=xyzs[:used], dirs=dirs[:used], dss=dss[:used], z_vals=zs[:used])

    # march_rays_inference: two refill iterations over 200 rays with 64 slots, cap 8
    c = dict(K=1, G=32, bound=1.0, sp=0.0, dns=1024, n_total=200, n_rays=64, cap=8)
    o, d, t0, t1 = make_rays(rng, c["n_total"], c["bound"])
    bits = random_bitfield(rng, c["K"], c["G"], 0.2)
    term = np.ones(c["n_rays"], bool)
    idx = np.zeros(c["n_rays"], np.uint32)
    nri = np.zeros(1, np.uint32)
    it = {}
    t_cur = t0.copy()
    for k in range(2):
        r = V.march_rays_inference(c["dns"], c["K"], c["G"], c["cap"], c["bound"], c["sp"], o, d,
                                   t_cur, t1, bits, nri, term, idx, backend="ref")
        nri_out, idx_out, ns, t_new, xyzs, dss, zs = r
        it.update({f"it{k}_terminated_in": term, f"it{k}_indices_in": idx,
                   f"it{k}_next_ray_index_in": nri, f"it{k}_t_starts_in": t_cur,
                   f"it{k}_next_ray_index": nri_out, f"it{k}_indices": idx_out,
                   f"it{k}_n_samples": ns, f"it{k}_t_starts": t_new, f"it{k}_xyzs": xyzs,
                   f"it{k}_dss": dss, f"it{k}_z_vals": zs})
        # next iteration: rays with fewer samples than the cap are finished
        term = ns < c["cap"]
        idx, nri, t_cur = idx_out, nri_out, t_new
    _save("volrend_march_inference.npz", K=c["K"], G=c["G"], bound=np.float32(c["bound"]),
          stepsize_portion=np.float32(c["sp"]), diagonal_n_steps=c["dns"], cap=c["cap"],
          rays_o=o, rays_d=d, t_ends=t1, bitfield=bits, **it)

    # integrate_rays forward + backward
    n = 512
    ns = rng.integers(0, 64, size=n).astype(np.uint32)
    ns[:8] = 0
    st = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.uint32)
    S = int(ns.sum())
    dss = rng.uniform(0.001, 0.02, S).astype(np.float32)
    zs = (np.cumsum(dss) * 0.5 + 0.05).astype(np.float32)
    sig = np.where(rng.uniform(size=S) < 0.5, rng.exponential(80, S), rng.exponential(2, S))
    drgbs = np.concatenate([sig[:, None], rng.uniform(size=(S, 3))], -1).astype(np.float32)
    bgs = rng.uniform(size=(n, 3)).astype(np.float32)
    near = np.float32(0.3)
    meas, rgbd, opac = V.integrate_rays(near, st, ns, bgs, dss, zs, drgbs, backend="ref")
    g = rng.normal(size=(n, 4)).astype(np.float32)
    gb, gz, gc = V.integrate_rays_backward(near, st, ns, bgs, dss, zs, drgbs, rgbd, opac, g,
                                           backend="ref")
    _save("volrend_integrate.npz", near_distance=near, rays_sample_startidx=st, rays_n_samples=ns,
          bgs=bgs, dss=dss, z_vals=zs, drgbs=drgbs, measured_batch_size=np.uint32(meas),
          final_rgbds=rgbd, final_opacities=opac, dL_dfinal_rgbds=g, dL_dbgs=gb, dL_dz_vals=gz,
          dL_ddrgbs=gc)

    # integrate_rays_inference
    n_total, n_rays, cap = 300, 128, 8
    rays_bg = rng.uniform(size=(n_total, 3)).astype(np.float32)
    rays_rgbd = (rng.uniform(size=(n_total, 4)) * 0.3).astype(np.float32)
    rays_T = rng.uniform(0.0, 1.0, size=n_total).astype(np.float32)
    ns = rng.integers(0, cap + 1, size=n_rays).astype(np.uint32)
    idx = rng.permutation(n_total + 20)[:n_rays].astype(np.uint32)  # a few out-of-range slots
    dss = rng.uniform(0.001, 0.05, (n_rays, cap)).astype(np.float32)
    zs = np.cumsum(dss, axis=1).astype(np.float32)
    sig = rng.exponential(30, (n_rays, cap, 1))
    drgbs = np.concatenate([sig, rng.uniform(size=(n_rays, cap, 3))], -1).astype(np.float32)
    cnt, term, rgbd_new, T_new = V.integrate_rays_inference(rays_bg, rays_rgbd, rays_T, ns, idx,
                                                            dss, zs, drgbs, backend="ref")
    _save("volrend_integrate_inference.npz", rays_bg=rays_bg, rays_rgbd=rays_rgbd, rays_T=rays_T,
          n_samples=ns, indices=idx, dss=dss, z_vals=zs, drgbs=drgbs, terminate_cnt=np.uint32(cnt),
          terminated=term, rays_rgbd_out=rgbd_new, rays_T_out=T_new)


def field(ref_root: str):
    import jax_numpy_shim as shim
    shim.install()
    enc_mod = shim.load_reference_module("models.encoders",
                                         os.path.join(ref_root, "models", "encoders.py"))
    nerf_mod = shim.load_reference_module("models.nerfs", os.path.join(ref_root, "models", "nerfs.py"))

    for case in HASHGRID_CASES:
        pos, latents, tab, bound = hashgrid_inputs(case)
        enc = enc_mod.HashGridEncoder(L=tab.L, T=tab.T, F=tab.F, N_min=tab.N_min, N_max=tab.N_max,
                                      tv_scale=0.0)
        enc.bind({"latent codes stored on grid vertices": latents})
        out, tv = enc(pos, bound)
        _save(f"hashgrid_{case['tag']}.npz", encodings=np.asarray(out, np.float32),
              **{k: v for k, v in case.items() if k != "tag"})

    pos, dirs, latents, w, tab, bound = field_inputs(FIELD_CASE)
    from oracle.field import to_flax_params
    model = nerf_mod.make_nerf_ngp(bound=bound, inference=False)
    params = {"position_encoder": {"latent codes stored on grid vertices": latents},
              **to_flax_params(w)}
    model.bind(params)
    drgb, _ = model(pos, dirs, np.zeros(0, np.float32))
    density, _ = model(pos, None, None)
    _save("field_ngp.npz", drgb=np.asarray(drgb, np.float32),
          density=np.asarray(density, np.float32), **{k: v for k, v in FIELD_CASE.items()})


def total_variation(ref_root: str):
    import jax_numpy_shim as shim
    shim.install()
    enc_mod = shim.load_reference_module("models.encoders",
                                         os.path.join(ref_root, "models", "encoders.py"))
    for case in TV_CASES:
        pos, latents, tab, bound = tv_inputs(case)
        enc = enc_mod.HashGridEncoder(L=tab.L, T=tab.T, F=tab.F, N_min=tab.N_min, N_max=tab.N_max,
                                      tv_scale=case["tv_scale"])
        enc.bind({"latent codes stored on grid vertices": latents})
        _, tv = enc(pos, bound)
        _save(f"{case['tag']}.npz", tv=np.asarray(tv, np.float32), **{k: v for k, v in case.items() if k != "tag"})


def spherical_harmonics(ref_root: str):
    """The reference's SphericalHarmonicsEncoder (models/encoders.py:361-406) for every degree it
    supports (1..8) on unit directions: random ones and the axis-aligned and diagonal ones."""
    import jax_numpy_shim as shim
    shim.install()
    enc_mod = shim.load_reference_module("models.encoders", os.path.join(ref_root, "models", "encoders.py"))
    rng = np.random.default_rng(41)
    d = rng.normal(size=(300, 3))
    edge = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [1, 1, 1], [-1, 1, -1],
                     [1, -1, 0], [0, 1, 1]], np.float64)
    d = np.concatenate([edge, d])
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    out = {"dirs": dirs}
    for L in range(1, 9):
        out[f"deg{L}"] = np.asarray(enc_mod.SphericalHarmonicsEncoder(L=L)(dirs), np.float32)
    _save("sh_encodings.npz", **out)


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] not in ("volrend", "field", "tv", "sh"):
        ref = args.pop(0)
    elif os.environ.get("NGP_REFERENCE_ROOT"):
        ref = os.environ["NGP_REFERENCE_ROOT"]
    else:
        sys.exit("usage: make_golden.py REFERENCE_ROOT [volrend] [field] [tv] [sh]  (or set NGP_REFERENCE_ROOT)")
    parts = args or ["volrend", "field", "tv", "sh"]
    if "volrend" in parts:
        volrend(ref)
    if "field" in parts:
        field(ref)
    if "tv" in parts:
        total_variation(ref)
    if "sh" in parts:
        spherical_harmonics(ref)
