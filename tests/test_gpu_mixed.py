"""Mixed precision on the GPU (the ``*_mixed`` entry points, through the C ABI): the FP16
tensor-core field MLP, 16-bit encodings and 16-bit working copies of the latent table, the dynamic
loss scale, and the errors of each precision's whole chain against the FP64 oracle.

Bars.  FP16 field against the oracle's FP16 restatement: as the BF16 one (99% of outputs within
1e-5 of the column's scale, all within 1e-2), weight gradients within 3e-3 of their scale (an FP32
accumulation and the restatement's exact one round to neighbouring FP16 values more often than to
neighbouring BF16 values, since FP16's steps are 8 times finer).  16-bit encodings are
the FP32 encodings rounded on their way into the first MMA, so feeding them already rounded gives
bit-identical outputs and weight gradients, and dL/dencodings equal to the FP32 ones rounded once.
A 16-bit table copy is widened to FP32 before the FP32 interpolation, so the encoder's output
equals the FP32 encoder's on the widened table, bit for bit.  The mixed Adam equals ngp_adam bit
for bit without a loss scale, and to FP32 rounding of its bias corrections with one (the scale is
a power of two, so unscaling is exact).  Whole-chain errors against FP64 are norm-relative
(||x - x64|| / ||x64||); the bounds beside each form are about twice the values measured on a
GB300 (the BF16/FP16 gradient errors are dominated by ReLU units whose sign flips when their input
is rounded, and by the cancellation in sums of random-sign terms)."""
import numpy as np
import pytest
import torch

from oracle import adjoint as A
from oracle import field as Fd
from oracle import hashgrid as H

pytestmark = pytest.mark.gpu

HALF = {"bf16": torch.bfloat16, "fp16": torch.float16}


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def colwise(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b).max(axis=0, keepdims=True), 1e-30)


def nrel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def inputs(n, seed, gscale=1.0):
    rng = np.random.default_rng(seed)
    enc = rng.normal(scale=0.5, size=(n, 32)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    g = (rng.normal(size=(n, 4)) * gscale).astype(np.float32)
    return enc, dirs, g


def packed(w):
    from jaxngp_gb300.field import pack_weights
    return pack_weights({k: torch.from_numpy(v) for k, v in w.items()}).cuda()


def flat_grads(dw):
    out, off = {}, 0
    for k, s in Fd.SHAPES.items():
        out[k] = dw[off:off + s[0] * s[1]].reshape(s)
        off += s[0] * s[1]
    return out


# ------------------------------------------------------------------------------ FP16 field MLP

@pytest.mark.parametrize("n", [1000, (1 << 16) + 77])
def test_f16_forward_matches_restatement(n):
    from jaxngp_gb300.field import field_forward
    enc, dirs, _ = inputs(n, 11)
    w = Fd.init_weights(12)
    out = field_forward(cu(enc), cu(dirs), packed(w), precision="fp16").cpu().numpy()
    emu, _ = Fd.forward_half(enc, dirs, w, "fp16")
    e = colwise(out, emu)
    assert np.quantile(e, 0.99, axis=0).max() <= 1e-5, np.quantile(e, 0.99, axis=0)
    assert e.max() <= 1e-2, e.max(axis=0)
    # the FP16 form against FP64 (10 mantissa bits: an order tighter than BF16)
    ref, _ = Fd.forward(enc, dirs, w, dtype=np.float64)
    assert np.abs(out[:, 1:] - ref[:, 1:]).max() <= 2e-3
    assert colwise(out[:, :1], ref[:, :1]).max() <= 5e-3


@pytest.mark.parametrize("n", [3000, (1 << 16) + 77])
def test_f16_backward_with_loss_scale_matches_restatement(n):
    """Gradients of the size training produces (dL/ddrgb ~ 1/n_rays) through FP16 with the loss
    scale 2^16: the kernel's gradients are the restatement's at the scaled magnitude."""
    from jaxngp_gb300.field import field_backward
    from jaxngp_gb300.precision import LossScale
    enc, dirs, g = inputs(n, 17, gscale=2.0 ** -18)
    w = Fd.init_weights(18)
    ls = LossScale("cuda", init=2.0 ** 16)
    denc, dw = field_backward(cu(enc), cu(dirs), packed(w), cu(g), precision="fp16", loss_scale=ls)
    _, cache = Fd.forward_half(enc, dirs, w, "fp16")
    denc_emu, gw_emu = Fd.backward_half(g, cache, grad_scale=2.0 ** 16)
    e = colwise(denc.cpu().numpy(), denc_emu)
    assert np.quantile(e, 0.99, axis=0).max() <= 1e-5, np.quantile(e, 0.99, axis=0).max()
    assert e.max() <= 2e-2, e.max()
    got = flat_grads(dw.cpu().numpy())
    for k in Fd.SHAPES:
        err = np.abs(got[k] - gw_emu[k]).max() / np.abs(gw_emu[k]).max()
        assert err <= 3e-3, (k, err)
    assert ls.read()["overflow"] == 0


def test_f16_loss_scale_recovers_underflowing_gradients():
    """Without the scale, FP16 flushes most of these gradients' low bits; with 2^16 the weight
    gradients are several times closer to FP64."""
    from jaxngp_gb300.field import field_backward
    from jaxngp_gb300.precision import LossScale
    n = 20000
    enc, dirs, g = inputs(n, 19, gscale=2.0 ** -18)
    w = Fd.init_weights(20)
    _, c64 = Fd.forward(enc, dirs, w, dtype=np.float64)
    _, gw64 = Fd.backward(g, c64, w)
    ls = LossScale("cuda", init=2.0 ** 16)
    _, dws = field_backward(cu(enc), cu(dirs), packed(w), cu(g), precision="fp16", loss_scale=ls)
    _, dw0 = field_backward(cu(enc), cu(dirs), packed(w), cu(g), precision="fp16")
    scaled = flat_grads(dws.cpu().numpy() / 2.0 ** 16)
    plain = flat_grads(dw0.cpu().numpy())
    e_s = nrel(np.concatenate([scaled[k].ravel() for k in Fd.SHAPES]), np.concatenate([gw64[k].ravel() for k in Fd.SHAPES]))
    e_0 = nrel(np.concatenate([plain[k].ravel() for k in Fd.SHAPES]), np.concatenate([gw64[k].ravel() for k in Fd.SHAPES]))
    assert e_s * 2 < e_0, (e_s, e_0)
    assert nrel(scaled["W4"], gw64["W4"]) <= 5e-3


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_half_encodings_equal_rounded_fp32(prec):
    from jaxngp_gb300.field import field_backward, field_density, field_forward
    n = 9000
    enc, dirs, g = inputs(n, 21)
    wt = packed(Fd.init_weights(22))
    e32 = cu(enc)
    eh = e32.to(HALF[prec])
    assert torch.equal(field_forward(eh, cu(dirs), wt, precision=prec), field_forward(e32, cu(dirs), wt, precision=prec))
    assert torch.equal(field_density(eh, wt, precision=prec), field_density(e32, wt, precision=prec))
    d32, w32 = field_backward(e32, cu(dirs), wt, cu(g), precision=prec)
    dh, wh = field_backward(eh, cu(dirs), wt, cu(g), precision=prec)
    assert dh.dtype == HALF[prec]
    assert torch.equal(dh, d32.to(HALF[prec]))
    assert torch.equal(wh, w32)


def test_half_encodings_active_count_zeroes_the_tail():
    from jaxngp_gb300.field import field_backward
    n, act = 7000, 4321
    enc, dirs, g = inputs(n, 23)
    wt = packed(Fd.init_weights(24))
    eh = cu(enc).to(torch.bfloat16)
    count = torch.tensor([act], dtype=torch.int32, device="cuda")
    denc = torch.full((n, 32), 3.0, dtype=torch.bfloat16, device="cuda")
    field_backward(eh, cu(dirs), wt, cu(g), count=count, dL_denc=denc, precision="bf16")
    full, _ = field_backward(eh[:act], cu(dirs[:act]), wt, cu(g[:act]), precision="bf16")
    assert torch.equal(denc[:act], full)
    assert (denc[act:] == 0).all()


def test_mixed_rejects_mismatched_types():
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.field import field_forward
    enc, dirs, _ = inputs(128, 25)
    wt = packed(Fd.init_weights(26))
    with pytest.raises(ValueError):
        field_forward(cu(enc).to(torch.bfloat16), cu(dirs), wt, precision="fp16")
    bad = L.NgpFieldMixedDescriptor(128, 0, L.DTYPE_F16, L.DTYPE_BF16)
    out = torch.empty(128, 4, device="cuda")
    with pytest.raises(L.NgpError):
        L.call("ngp_field_forward_mixed", [cu(enc).to(torch.bfloat16), cu(dirs), wt, None, out], bad)
    with pytest.raises(L.NgpError):
        L.call("ngp_field_forward_mixed", [cu(enc), cu(dirs), wt, None, out], L.NgpFieldMixedDescriptor(128, 0, 0, 0))


# ------------------------------------------------------------------------- loss scale and Adam

def _adam(name, bufs, desc):
    from jaxngp_gb300 import _lib as L
    L.call(name, bufs, desc)


def test_overflow_sets_the_flag_and_the_step_is_skipped():
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.field import field_backward
    from jaxngp_gb300.precision import LossScale
    enc, dirs, g = inputs(4000, 27)
    wt = packed(Fd.init_weights(28))
    ls = LossScale("cuda", init=2.0 ** 40)   # FP16 cannot hold gradients this large
    field_backward(cu(enc), cu(dirs), wt, cu(g), precision="fp16", loss_scale=ls)
    assert ls.read()["overflow"] == 1
    n = 4099
    gen = torch.Generator(device="cuda").manual_seed(3)
    p, gr, m, v = (torch.randn(n, device="cuda", generator=gen) for _ in range(4))
    v = v.abs()
    p0, m0, v0 = p.clone(), m.clone(), v.clone()
    ph = torch.zeros(n, dtype=torch.bfloat16, device="cuda")
    d = L.NgpAdamMixedDescriptor(L.NgpAdamDescriptor(n, 5, 1e-2, 0.9, 0.99, 1e-15, 1e-15, 0.0, 1), L.DTYPE_BF16)
    _adam("ngp_adam_mixed", [p, gr, m, v, ls.state, ph], d)
    assert torch.equal(p, p0) and torch.equal(m, m0) and torch.equal(v, v0)
    assert (gr == 0).all() and (ph == 0).all()
    ls.update()
    st = ls.read()
    assert st == {"scale": 2.0 ** 39, "overflow": 0, "good_steps": 0, "skipped_steps": 1}


def test_loss_scale_growth_backoff_and_bounds():
    from jaxngp_gb300.precision import LossScale
    ls = LossScale("cuda", init=4.0, growth_interval=3, max_scale=16.0, min_scale=2.0)
    scales = []
    for _ in range(9):
        ls.update()
        scales.append(ls.read()["scale"])
    assert scales == [4, 4, 8, 8, 8, 16, 16, 16, 16]
    for want in (8.0, 4.0, 2.0, 2.0):
        ls.state[1] = 1
        ls.update()
        st = ls.read()
        assert st["scale"] == want and st["overflow"] == 0 and st["good_steps"] == 0
    assert ls.read()["skipped_steps"] == 4


@pytest.mark.parametrize("half", ["fp32", "bf16", "fp16"])
def test_adam_mixed_matches_adam(half):
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.precision import CODE, LossScale
    n = (1 << 20) + 3
    gen = torch.Generator(device="cuda").manual_seed(5)
    p, gr, m, v = (torch.randn(n, device="cuda", generator=gen) * 0.1 for _ in range(4))
    v = v.abs()
    base = L.NgpAdamDescriptor(n, 7, 1e-2, 0.9, 0.99, 1e-15, 1e-15, 1e-6, 0)
    ref = [t.clone() for t in (p, gr, m, v)]
    _adam("ngp_adam", ref, base)
    ph = torch.zeros(n, dtype=HALF[half], device="cuda") if half != "fp32" else None
    # no loss scale: the same arithmetic, bit for bit
    a = [t.clone() for t in (p, gr, m, v)]
    _adam("ngp_adam_mixed", a + [None, ph], L.NgpAdamMixedDescriptor(base, CODE[half]))
    for x, y in zip(a, ref):
        assert torch.equal(x, y)
    if ph is not None:
        assert torch.equal(ph, a[0].to(HALF[half]))
    # scaled gradients: unscaling by a power of two is exact; the bias corrections come from the
    # device's powf (two skipped steps: step 9 updates like step 7)
    ls = LossScale("cuda", init=2.0 ** 16)
    ls.state[3] = 2
    b = [p.clone(), gr * 2.0 ** 16, m.clone(), v.clone()]
    d9 = L.NgpAdamDescriptor(n, 9, 1e-2, 0.9, 0.99, 1e-15, 1e-15, 1e-6, 0)
    _adam("ngp_adam_mixed", b + [ls.state, ph], L.NgpAdamMixedDescriptor(d9, CODE[half]))
    assert torch.equal(b[2], ref[2]) and torch.equal(b[3], ref[3])
    assert torch.allclose(b[0], ref[0], rtol=0, atol=1e-6)
    if ph is not None:
        assert torch.equal(ph, b[0].to(HALF[half]))


# ------------------------------------------------------------------ 16-bit table and encodings

@pytest.mark.parametrize("table,enc_t", [("bf16", "fp32"), ("fp16", "fp32"), ("bf16", "bf16"), ("fp16", "fp16"),
                                         ("fp32", "bf16"), ("fp32", "fp16")])
def test_hashgrid_forward_mixed_equals_widened_fp32(table, enc_t):
    from jaxngp_gb300.encoders import LevelTable, hashgrid_forward
    tab = LevelTable(16, 1 << 14, 2, 16, 2048)
    gen = torch.Generator(device="cuda").manual_seed(7)
    lat = (torch.rand(tab.n_params, 2, device="cuda", generator=gen) - 0.5) * 0.6
    pos = (torch.rand(100003, 3, device="cuda", generator=gen) * 2 - 1) * 1.02   # a few outside the box
    lat_t = lat.to(HALF[table]) if table != "fp32" else lat
    edt = HALF[enc_t] if enc_t != "fp32" else torch.float32
    got = hashgrid_forward(tab, pos, lat_t, 1.0, enc_dtype=edt)
    want = hashgrid_forward(tab, pos, lat_t.float(), 1.0)
    assert got.dtype == edt
    assert torch.equal(got, want.to(edt))


@pytest.mark.parametrize("enc_t", ["bf16", "fp16"])
def test_hashgrid_backward_half_gradient(enc_t):
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward
    tab = LevelTable(16, 1 << 14, 2, 16, 2048)
    gen = torch.Generator(device="cuda").manual_seed(8)
    n = 60001
    pos = torch.rand(n, 3, device="cuda", generator=gen) * 2 - 1
    gh = torch.randn(n, 32, device="cuda", generator=gen).to(HALF[enc_t])
    count = torch.tensor([n - 1000], dtype=torch.int32, device="cuda")
    got = hashgrid_backward(tab, pos, gh, 1.0, count=count)
    want = hashgrid_backward(tab, pos, gh.float(), 1.0, count=count)
    scale = want.abs().max()
    assert torch.allclose(got, want, rtol=1e-5, atol=1e-6 * float(scale))


# ------------------------------------------------------------------ whole chain against FP64

FORMS = {
    # name: (mlp, table, 16-bit activations, initial loss scale)
    "fp32": ("fp32", "fp32", False, None),
    "bf16": ("bf16", "fp32", False, None),
    "bf16-mixed": ("bf16", "bf16", True, None),
    "fp16-mixed": ("fp16", "fp16", True, 2.0 ** 16),
    "fp16-mixed-unscaled": ("fp16", "fp16", True, None),
}

# norm-relative error bounds: colour, transmittance, dL/ddrgb, dL/dW, dL/dlatents (measured on a
# GB300: fp32 1.8e-7 6.3e-7 1.5e-6 4.6e-7 8.4e-7; bf16 1.1e-4 4.8e-5 2.1e-4 9.4e-3 3.3e-2;
# bf16-mixed 1.1e-4 5.7e-5 2.3e-4 9.5e-3 3.6e-2; fp16-mixed 1.3e-5 1.1e-5 3.0e-5 3.7e-3 1.5e-2)
BOUNDS = {
    "fp32": (1e-6, 2e-6, 5e-6, 2e-6, 3e-6),
    "bf16": (3e-4, 1.5e-4, 5e-4, 2e-2, 7e-2),
    "bf16-mixed": (3e-4, 1.5e-4, 5e-4, 2e-2, 8e-2),
    "fp16-mixed": (3e-5, 3e-5, 6e-5, 8e-3, 3e-2),
}


def chain_errors(form: str, R: int = 256, n: int = 64, seed: int = 41) -> dict:
    """positions -> encoder -> field -> integrator (exact adjoint) -> L = g . rgbd with
    dL/drgbd ~ N(0, 1) / 2^18 (the size of a training step's per-ray gradient), at one form,
    against the same chain in FP64.  Returns norm-relative errors."""
    from jaxngp_gb300 import volrendjax as vr
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward, hashgrid_forward
    from jaxngp_gb300.field import field_backward, field_forward
    from jaxngp_gb300.precision import LossScale
    mlp, table, half_act, ls0 = FORMS[form]
    rng = np.random.default_rng(seed)
    tab_np = H.LevelTable(16, 1 << 14, 2, 16, 2048)
    tab = LevelTable(16, 1 << 14, 2, 16, 2048)
    lat = rng.uniform(-0.3, 0.3, size=(tab_np.n_params, 2)).astype(np.float32)
    w = Fd.init_weights(seed + 1)
    o = rng.uniform(-0.6, 0.6, size=(R, 3))
    d = rng.normal(size=(R, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ts = 0.02 * (np.arange(n) + 0.5)
    pos = (o[:, None, :] + ts[None, :, None] * d[:, None, :]).astype(np.float32).reshape(-1, 3)
    dirs = np.repeat(d[:, None, :], n, 1).astype(np.float32).reshape(-1, 3)
    dt = np.full((R, n), 0.02, np.float32)
    z = np.broadcast_to(ts.astype(np.float32), (R, n)).copy()
    bg = rng.uniform(size=(R, 3)).astype(np.float32)
    g = (rng.normal(size=(R, 4)) * 2.0 ** -18).astype(np.float32)

    # FP64
    enc64 = H.encode_as_f32(pos, lat.astype(np.float64), 1.0, tab_np)
    drgb64, c64 = Fd.forward(enc64, dirs, w, dtype=np.float64)
    d64 = drgb64.reshape(R, n, 4)
    out64, op64, _ = A.integrate_forward64(d64[..., 0], d64[..., 1:], dt, z, bg)
    gd64 = np.zeros((R, n, 4))
    for r in range(R):
        gs, grgb, _, _ = A.ray_adjoint64(d64[r, :, 0], d64[r, :, 1:], dt[r], z[r], bg[r], g[r].astype(np.float64))
        gd64[r, :, 0], gd64[r, :, 1:] = gs, grgb
    denc64, gw64 = Fd.backward(gd64.reshape(-1, 4), c64, w)
    glat64 = H.encode_backward(pos, denc64, 1.0, tab_np)

    # GPU at the form's precision
    lat_t = cu(lat) if table == "fp32" else cu(lat).to(HALF[table])
    act = HALF[mlp] if half_act else torch.float32
    wt = packed(w)
    enc = hashgrid_forward(tab, cu(pos), lat_t, 1.0, enc_dtype=act)
    drgb = field_forward(enc, cu(dirs), wt, precision=mlp)
    start = torch.arange(R, dtype=torch.int32, device="cuda") * n
    ns = torch.full((R,), n, dtype=torch.int32, device="cuda")
    _, rgbd, opac = vr.integrate_rays(0.0, start, ns, cu(bg), cu(dt.reshape(-1)), cu(z.reshape(-1)), drgb)
    _, _, gd = vr.integrate_rays_backward(0.0, start, ns, cu(bg), cu(dt.reshape(-1)), cu(z.reshape(-1)), drgb, rgbd,
                                          opac, cu(g), exact=True)
    ls = LossScale("cuda", init=ls0) if ls0 else None
    denc, dw = field_backward(enc, cu(dirs), wt, gd, precision=mlp, loss_scale=ls)
    glat = hashgrid_backward(tab, cu(pos), denc, 1.0)
    s = ls0 or 1.0
    dw = dw.cpu().numpy().astype(np.float64) / s
    glat = glat.cpu().numpy().astype(np.float64) / s
    gw64_flat = np.concatenate([gw64[k].ravel() for k in Fd.SHAPES])
    return {
        "colour": nrel(rgbd.cpu().numpy()[:, :3], out64[:, :3]),
        "transmittance": nrel(1 - opac.cpu().numpy(), 1 - op64),
        "dL_ddrgb": nrel(gd.cpu().numpy().reshape(R, n, 4), gd64),
        "dL_dW": nrel(dw, gw64_flat),
        "dL_dlatents": nrel(glat, glat64),
        "overflow": ls.read()["overflow"] if ls is not None else 0,
    }


@pytest.mark.parametrize("form", list(BOUNDS))
def test_chain_errors_vs_fp64(form):
    e = chain_errors(form)
    print(form, {k: f"{v:.2e}" for k, v in e.items()})
    keys = ("colour", "transmittance", "dL_ddrgb", "dL_dW", "dL_dlatents")
    for k, b in zip(keys, BOUNDS[form]):
        assert e[k] <= b, (form, k, e[k], b)
    assert e["overflow"] == 0


def test_chain_fp16_needs_the_loss_scale():
    scaled = chain_errors("fp16-mixed")
    plain = chain_errors("fp16-mixed-unscaled")
    assert scaled["dL_dlatents"] * 2 < plain["dL_dlatents"], (scaled, plain)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_tma_tiles_equal_register_tiles(prec):
    """16-bit encodings of a buffer whose row count is a multiple of 8 reach the MMAs through TMA
    tile copies (a 4-D tensor map whose box lands in the operand's core-matrix layout); other row
    counts through per-thread loads.  The same rows give bit-identical outputs, dL/denc and
    weight gradients either way (the active count keeps the work the same), whatever the buffer
    holds past the active count."""
    from jaxngp_gb300.field import field_backward, field_forward
    n = 3 * 8192 + 40   # several tiles per warpgroup, a partial last tile
    enc, dirs, g = inputs(n + 1, 31)
    wt = packed(Fd.init_weights(32))
    eh = cu(enc).to(HALF[prec])
    act = torch.tensor([n], dtype=torch.int32, device="cuda")
    a = field_forward(eh[:n].contiguous(), cu(dirs[:n]), wt, precision=prec)            # n % 8 == 0: TMA
    b = field_forward(eh, cu(dirs), wt, count=act, precision=prec)                     # n + 1 rows: loads
    assert torch.equal(a, b[:n])
    da, wa = field_backward(eh[:n].contiguous(), cu(dirs[:n]), wt, cu(g[:n]), precision=prec)
    db, wb = field_backward(eh, cu(dirs), wt, cu(g), count=act, precision=prec)
    assert torch.equal(da, db[:n]) and torch.equal(wa, wb)
    # a TMA-eligible buffer whose rows past the active count hold NaN (stale memory): the tile's
    # inactive rows are zeroed before the MMAs, so nothing of them reaches the outputs
    pad = torch.full((8, 32), float("nan"), dtype=HALF[prec], device="cuda")
    en = torch.cat([eh[:n], pad]).contiguous()
    dn = torch.cat([cu(dirs[:n]), torch.zeros(8, 3, device="cuda")]).contiguous()
    gn = torch.cat([cu(g[:n]), torch.full((8, 4), float("nan"), device="cuda")]).contiguous()
    c = field_forward(en, dn, wt, count=act, precision=prec)
    assert torch.equal(c[:n], a)
    dc, wc = field_backward(en, dn, wt, gn, count=act, precision=prec)
    assert torch.equal(dc[:n], da) and torch.equal(wc, wa) and bool(torch.isfinite(wc).all())
    from jaxngp_gb300 import _lib as L
    assert L.lib().ngp_device_status() == 0
