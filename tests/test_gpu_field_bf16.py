"""GPU checks of the BF16 tensor-core field MLP (ngp_field_*_bf16, through the C ABI).

Bar: against the oracle's BF16 restatement (every MMA operand rounded to bfloat16, exact
accumulation), 99% of the outputs agree to 1e-5 and all to 1e-2 of the column's scale: the GPU
accumulates in FP32 and rounds each layer's input to BF16, so an intermediate that sits on a BF16
rounding boundary can land one BF16 step away from the restatement's and move that sample's
outputs by ~1e-3.  Weight gradients, sums over every sample, agree to 1e-3.  Against FP64 the
errors are the BF16 form's own and are bounded here as stated beside each assertion.
"""
import numpy as np
import pytest
import torch

from oracle import field as Fd

pytestmark = pytest.mark.gpu


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def colwise(a, b):
    """|a - b| / max|b| per column."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b).max(axis=0, keepdims=True), 1e-30)


def inputs(n, seed):
    rng = np.random.default_rng(seed)
    enc = rng.normal(scale=0.5, size=(n, 32)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    g = rng.normal(size=(n, 4)).astype(np.float32)
    return enc, dirs, g


def packed(w):
    from jaxngp_gb300.field import pack_weights
    return pack_weights({k: torch.from_numpy(v) for k, v in w.items()}).cuda()


@pytest.mark.parametrize("n", [1000, (1 << 16) + 77])
def test_bf16_forward_matches_restatement(n):
    from jaxngp_gb300.field import field_forward
    enc, dirs, _ = inputs(n, 11)
    w = Fd.init_weights(12)
    out = field_forward(cu(enc), cu(dirs), packed(w), precision="bf16").cpu().numpy()
    emu, _ = Fd.forward_bf16(enc, dirs, w)
    e = colwise(out, emu)
    assert np.quantile(e, 0.99, axis=0).max() <= 1e-5, np.quantile(e, 0.99, axis=0)
    assert e.max() <= 1e-2, e.max(axis=0)
    # the BF16 form against FP64: colour within 1e-2 absolute, density within 2% of its scale
    ref, _ = Fd.forward(enc, dirs, w, dtype=np.float64)
    assert np.abs(out[:, 1:] - ref[:, 1:]).max() <= 1e-2
    assert colwise(out[:, :1], ref[:, :1]).max() <= 2e-2


def test_bf16_forward_active_count():
    from jaxngp_gb300.field import field_forward
    n, act = 5000, 3333
    enc, dirs, _ = inputs(n, 13)
    w = Fd.init_weights(14)
    out = torch.full((n, 4), -7.0, device="cuda")
    count = torch.tensor([act], dtype=torch.int32, device="cuda")
    field_forward(cu(enc), cu(dirs), packed(w), count=count, out=out, precision="bf16")
    full = field_forward(cu(enc), cu(dirs), packed(w), precision="bf16")
    assert torch.equal(out[:act], full[:act])
    assert (out[act:] == -7.0).all()


def test_bf16_density_matches_forward():
    from jaxngp_gb300.field import field_density, field_forward
    n = 20000
    enc, dirs, _ = inputs(n, 15)
    w = Fd.init_weights(16)
    sig = field_density(cu(enc), packed(w), precision="bf16")
    drgb = field_forward(cu(enc), cu(dirs), packed(w), precision="bf16")
    assert torch.equal(sig, drgb[:, 0])
    emu, _ = Fd.forward_bf16(enc, dirs, w)
    e = colwise(sig.cpu().numpy()[:, None], emu[:, :1])
    assert np.quantile(e, 0.99) <= 1e-5 and e.max() <= 1e-2


@pytest.mark.parametrize("n", [3000, (1 << 16) + 77])
def test_bf16_backward_matches_restatement(n):
    from jaxngp_gb300.field import field_backward
    enc, dirs, g = inputs(n, 17)
    w = Fd.init_weights(18)
    gs = torch.tensor([0.5], device="cuda")
    denc, dw = field_backward(cu(enc), cu(dirs), packed(w), cu(g), grad_scale=gs, precision="bf16")
    _, cache = Fd.forward_bf16(enc, dirs, w)
    denc_emu, gw_emu = Fd.backward_bf16(g, cache, grad_scale=0.5)
    e = colwise(denc.cpu().numpy(), denc_emu)
    assert np.quantile(e, 0.99, axis=0).max() <= 1e-5, np.quantile(e, 0.99, axis=0).max()
    assert e.max() <= 2e-2, e.max()
    dw = dw.cpu().numpy()
    off = 0
    for k, s in Fd.SHAPES.items():
        sz = s[0] * s[1]
        got = dw[off:off + sz].reshape(s)
        err = np.abs(got - gw_emu[k]).max() / np.abs(gw_emu[k]).max()
        assert err <= 1e-3, (k, err)
        off += sz


def test_bf16_backward_deterministic_and_accumulates():
    from jaxngp_gb300.field import field_backward
    n = 40000
    enc, dirs, g = inputs(n, 19)
    wt = packed(Fd.init_weights(20))
    a = field_backward(cu(enc), cu(dirs), wt, cu(g), precision="bf16")
    b = field_backward(cu(enc), cu(dirs), wt, cu(g), precision="bf16")
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
    acc = torch.ones_like(a[1])
    field_backward(cu(enc), cu(dirs), wt, cu(g), dL_dw=acc, accumulate=True, precision="bf16")
    assert torch.equal(acc, a[1] + 1)


def test_bf16_backward_active_count():
    """Rows past the active count contribute nothing and get zero dL/denc."""
    from jaxngp_gb300.field import field_backward
    n, act = 9000, 6001
    enc, dirs, g = inputs(n, 21)
    wt = packed(Fd.init_weights(22))
    count = torch.tensor([act], dtype=torch.int32, device="cuda")
    denc, dw = field_backward(cu(enc), cu(dirs), wt, cu(g), count=count, precision="bf16")
    denc2, dw2 = field_backward(cu(enc[:act]), cu(dirs[:act]), wt, cu(g[:act]), precision="bf16")
    assert torch.equal(denc[:act], denc2)
    assert (denc[act:] == 0).all()
    assert torch.allclose(dw, dw2, rtol=1e-5, atol=1e-7)


def test_bf16_empty_batch_and_status():
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.field import field_backward, field_forward
    enc, dirs, g = inputs(1, 23)
    wt = packed(Fd.init_weights(24))
    zero = torch.zeros(1, dtype=torch.int32, device="cuda")
    field_forward(cu(enc), cu(dirs), wt, count=zero, precision="bf16")
    denc, dw = field_backward(cu(enc), cu(dirs), wt, cu(g), count=zero, precision="bf16")
    assert (denc == 0).all() and (dw == 0).all()
    assert L.lib().ngp_device_status() == 0
