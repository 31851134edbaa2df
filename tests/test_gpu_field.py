"""GPU parity of the hash-grid encoder and the field MLP (through the C ABI).

Bar: encodings bit-exact against the reference's HashGridEncoder (golden fixtures made by running
models/encoders.py) and the float32 oracle; table gradients, MLP outputs and MLP gradients within
1e-5 relative error against the FP64 oracle, measured column-wise as
max|gpu - fp64| / max|fp64| (atomics and matmul blocking reorder float32 sums).

MLP gradients are compared on samples whose ReLU pre-activations are all at least KINK * max|a|
away from zero: closer than that, a float32 evaluation (the reference's as much as ours) may land
on the other side of the kink than FP64 and the gradient jumps there.
"""
import numpy as np
import pytest
import torch

from golden_inputs import FIELD_CASE, HASHGRID_CASES, TV_CASES, field_inputs, hashgrid_inputs, tv_inputs
from oracle import field as Fd
from oracle import hashgrid as H
from tests.golden_util import load

pytestmark = pytest.mark.gpu

RTOL = 1e-5
KINK = 1e-4


def rel_err(a, b, axis=0):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b).max(axis=axis, keepdims=True), 1e-30)
    return (np.abs(a - b) / scale).max()


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("case", HASHGRID_CASES, ids=lambda c: c["tag"])
def test_hashgrid_forward_golden(case):
    from jaxngp_gb300.encoders import LevelTable, hashgrid_forward
    pos, lat, tab, b = hashgrid_inputs(case)
    t = LevelTable(tab.L, tab.T, tab.F, tab.N_min, tab.N_max)
    enc = hashgrid_forward(t, cu(pos), cu(lat), b).cpu().numpy()
    assert np.array_equal(enc, load(f"hashgrid_{case['tag']}")["encodings"])


@pytest.mark.parametrize("L", [1, 2, 3, 5, 8, 12])
def test_hashgrid_forward_level_counts(L):
    """Tables with fewer levels than the kernel's 8 warps split a tile into sub-tiles of 32 points
    (L = 1, 2, 3: 8, 4, 2 sub-tiles; L = 3 leaves two warps idle); L >= 8 loops warps over levels.
    Ragged point counts and a device count below n: bit-exact against the oracle, rows past the
    count untouched; the 16-bit encodings are the FP32 ones rounded."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_forward
    rng = np.random.default_rng(40 + L)
    n = 32 * 8 * 5 + 37
    pos = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
    tab = H.LevelTable(L, 2 ** 12, 2, 4, 256, per_level_scale=1.5)   # explicit scale: L = 1 has no ratio
    lat = rng.uniform(-1, 1, size=(tab.n_params, 2)).astype(np.float32)
    ref = H.encode(pos, lat, 1.0, tab)
    t = LevelTable(L, 2 ** 12, 2, 4, 256, per_level_scale=1.5)
    assert np.array_equal(hashgrid_forward(t, cu(pos), cu(lat), 1.0).cpu().numpy(), ref)
    m = n - 301
    out = torch.full((n, 2 * L), 7.0, device="cuda")
    hashgrid_forward(t, cu(pos), cu(lat), 1.0, count=torch.tensor([m], dtype=torch.int32, device="cuda"), out=out)
    got = out.cpu().numpy()
    assert np.array_equal(got[:m], ref[:m]) and (got[m:] == 7.0).all()
    h = hashgrid_forward(t, cu(pos), cu(lat), 1.0, enc_dtype=torch.bfloat16)
    assert torch.equal(h, torch.from_numpy(ref).cuda().to(torch.bfloat16))


@pytest.mark.parametrize("case", TV_CASES, ids=lambda c: c["tag"])
def test_hashgrid_tv_golden(case):
    """The TV term against the reference's HashGridEncoder (fixtures made by running encoders.py)."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_tv
    pos, lat, tab, b = tv_inputs(case)
    t = LevelTable(tab.L, tab.T, tab.F, tab.N_min, tab.N_max)
    tv = float(hashgrid_tv(t, cu(pos), cu(lat), b, case["tv_scale"]))
    want = float(load(case["tag"])["tv"])
    assert abs(tv - want) <= RTOL * abs(want)


def test_hashgrid_tv_vs_fp64():
    """Value and gradient against the FP64 oracle on points inside, on and outside the box (the
    saturating coordinate conversion at the low faces); the gradient is scaled by a device scalar
    and added to what the buffer holds; tv_scale = 0 writes 0 and leaves the gradient alone."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_tv
    rng = np.random.default_rng(17)
    n = 40000
    pos = rng.uniform(-1.2, 1.2, size=(n, 3)).astype(np.float32)
    pos[:64] = np.float32(-1.0)                       # the low corner of the box
    tab = H.LevelTable(16, 2 ** 16, 2, 16, 2048)
    t = LevelTable(16, 2 ** 16, 2, 16, 2048)
    lat = rng.uniform(-1, 1, size=(tab.n_params, 2)).astype(np.float32)
    s = 0.05
    want = H.total_variation(pos, lat, 1.0, tab, s, dtype=np.float64)
    gwant = H.total_variation_grad(pos, lat, 1.0, tab, s)
    grad = torch.zeros(tab.n_params, 2, device="cuda")
    three = torch.tensor([3.0], device="cuda")
    tv = hashgrid_tv(t, cu(pos), cu(lat), 1.0, s, grad=grad, grad_scale=three)
    assert abs(float(tv) - want) <= RTOL * want
    first = grad.cpu().numpy()
    assert rel_err(first, 3.0 * gwant) <= RTOL
    hashgrid_tv(t, cu(pos), cu(lat), 1.0, s, grad=grad, grad_scale=three)   # adds to what is there
    assert rel_err(grad.cpu().numpy(), 2.0 * first) <= RTOL
    before = grad.clone()
    tv0 = hashgrid_tv(t, cu(pos), cu(lat), 1.0, 0.0, grad=grad)
    assert float(tv0) == 0.0 and torch.equal(grad, before)


def test_hashgrid_encoder_module_tv():
    """HashGridEncoder(tv_scale > 0) returns (encodings, tv) with tv differentiable w.r.t. the table,
    as the reference's flax module; the upstream gradient of tv scales the table gradient."""
    from jaxngp_gb300.encoders import HashGridEncoder
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    enc_mod = HashGridEncoder(16, 2 ** 14, 2, 16, 2048, tv_scale=0.2, generator=g)
    with torch.no_grad():
        enc_mod.latents.uniform_(-1, 1, generator=g)
    rng = np.random.default_rng(4)
    pos = rng.uniform(-1, 1, size=(5000, 3)).astype(np.float32)
    enc, tv = enc_mod(cu(pos), 1.0)
    lat = enc_mod.latents.detach().cpu().numpy()
    tab = H.LevelTable(16, 2 ** 14, 2, 16, 2048)
    tv_value = float(tv.detach())
    assert abs(tv_value - H.total_variation(pos, lat, 1.0, tab, 0.2, dtype=np.float64)) <= RTOL * tv_value
    (2.5 * tv).backward()
    gw = H.total_variation_grad(pos, lat, 1.0, tab, 0.2)
    assert rel_err(enc_mod.latents.grad.cpu().numpy(), 2.5 * gw) <= RTOL


def test_hashgrid_forward_large_bitexact():
    """2^18 points at the training configuration (L=16, T=2^19, N_max=2048): bit-exact against the oracle."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_forward
    rng = np.random.default_rng(0)
    n = 1 << 18
    pos = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
    tab = H.LevelTable(16, 2 ** 19, 2, 16, 2048)
    lat = rng.uniform(-1e-4, 1e-4, size=(tab.n_params, 2)).astype(np.float32)
    ref = H.encode(pos, lat, 1.0, tab)
    enc = hashgrid_forward(LevelTable(16, 2 ** 19, 2, 16, 2048), cu(pos), cu(lat), 1.0).cpu().numpy()
    assert np.array_equal(enc, ref)


@pytest.mark.parametrize("scale", [None, 1.447])
def test_hashgrid_backward_vs_fp64(scale):
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward
    rng = np.random.default_rng(1)
    n = 1 << 15
    pos = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
    g = rng.normal(size=(n, 32)).astype(np.float32)
    tab = H.LevelTable(16, 2 ** 19, 2, 16, 2048, per_level_scale=scale)
    ref = H.encode_backward(pos, g, 1.0, tab, dtype=np.float64)
    out = hashgrid_backward(LevelTable(16, 2 ** 19, 2, 16, 2048, per_level_scale=scale), cu(pos), cu(g), 1.0)
    assert rel_err(out.cpu().numpy(), ref) <= RTOL


def test_hashgrid_active_count():
    """Rows past the active count are neither computed nor scattered."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward, hashgrid_forward
    rng = np.random.default_rng(2)
    n, k = 1000, 613
    pos = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
    tab = LevelTable(16, 2 ** 16, 2, 16, 2048)
    lat = rng.uniform(-1, 1, size=(tab.n_params, 2)).astype(np.float32)
    cnt = torch.tensor([k], dtype=torch.int32, device="cuda")
    out = torch.full((n, 32), 7.0, device="cuda")
    hashgrid_forward(tab, cu(pos), cu(lat), 1.0, count=cnt, out=out)
    full = hashgrid_forward(tab, cu(pos), cu(lat), 1.0)
    assert torch.equal(out[:k], full[:k]) and bool((out[k:] == 7.0).all())
    g = rng.normal(size=(n, 32)).astype(np.float32)
    a = hashgrid_backward(tab, cu(pos), cu(g), 1.0, count=cnt)
    b = hashgrid_backward(tab, cu(pos[:k]), cu(g[:k]), 1.0)
    assert torch.allclose(a, b, rtol=1e-5, atol=1e-6)


def test_field_forward_golden():
    from jaxngp_gb300.encoders import LevelTable, hashgrid_forward
    from jaxngp_gb300.field import field_density, field_forward, pack_weights
    pos, dirs, lat, w, tab, b = field_inputs(FIELD_CASE)
    z = load("field_ngp")
    enc = hashgrid_forward(LevelTable(tab.L, tab.T, tab.F, tab.N_min, tab.N_max), cu(pos), cu(lat), b)
    wt = pack_weights({k: torch.from_numpy(v) for k, v in w.items()}).cuda()
    drgb = field_forward(enc, cu(dirs), wt).cpu().numpy()
    ref64, _ = Fd.forward(H.encode(pos, lat, b, tab), dirs, w, dtype=np.float64)
    assert rel_err(drgb, z["drgb"]) <= RTOL
    assert rel_err(drgb, ref64) <= RTOL
    sig = field_density(enc, wt).cpu().numpy()
    assert rel_err(sig, z["density"][:, 0]) <= RTOL


@pytest.mark.parametrize("n", [1000, 1 << 17])
def test_field_backward_vs_fp64(n):
    from jaxngp_gb300.field import field_backward, pack_weights
    rng = np.random.default_rng(3)
    enc = rng.normal(scale=0.5, size=(n, 32)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    w = Fd.init_weights(4)
    g = rng.normal(size=(n, 4)).astype(np.float32)
    keep = Fd.kink_distance(enc, dirs, w) > KINK
    assert keep.mean() > 0.9
    enc, dirs, g = enc[keep], dirs[keep], g[keep]
    _, cache = Fd.forward(enc, dirs, w, dtype=np.float64)
    denc_ref, gw_ref = Fd.backward(g, cache, w, dtype=np.float64)
    wt = pack_weights({k: torch.from_numpy(v) for k, v in w.items()}).cuda()
    denc, dw = field_backward(cu(enc), cu(dirs), wt, cu(g))
    assert rel_err(denc.cpu().numpy(), denc_ref) <= RTOL
    dw = dw.cpu().numpy()
    off = 0
    for k, s in Fd.SHAPES.items():
        sz = s[0] * s[1]
        assert rel_err(dw[off:off + sz].reshape(s), gw_ref[k], axis=None) <= RTOL, k
        off += sz


def test_field_backward_deterministic():
    from jaxngp_gb300.field import field_backward, pack_weights
    rng = np.random.default_rng(5)
    n = 50000
    enc = cu(rng.normal(size=(n, 32)).astype(np.float32))
    d = rng.normal(size=(n, 3))
    dirs = cu((d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32))
    w = pack_weights({k: torch.from_numpy(v) for k, v in Fd.init_weights(6).items()}).cuda()
    g = cu(rng.normal(size=(n, 4)).astype(np.float32))
    a = field_backward(enc, dirs, w, g)
    b = field_backward(enc, dirs, w, g)
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_field_module_autograd():
    """NGPField end to end through autograd: gradients of a scalar loss match FP64."""
    from jaxngp_gb300.field import NGPField, unpack_weights
    torch.manual_seed(0)
    f = NGPField(1.0, T=2 ** 14, device="cuda", seed=3)
    with torch.no_grad():
        f.position_encoder.latents.uniform_(-1, 1)
    rng = np.random.default_rng(7)
    n = 4096
    pos = rng.uniform(-1, 1, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    gout = rng.normal(size=(n, 4)).astype(np.float32)
    tab = H.LevelTable(16, 2 ** 14, 2, 16, 2048)
    lat = f.position_encoder.latents.detach().cpu().numpy()
    w = {k: v.cpu().numpy() for k, v in unpack_weights(f.weights.detach()).items()}
    keep = Fd.kink_distance(H.encode(pos, lat, 1.0, tab, dtype=np.float64), dirs, w) > KINK
    pos, dirs, gout = pos[keep], dirs[keep], gout[keep]
    drgb = f(cu(pos), cu(dirs))
    (drgb * cu(gout)).sum().backward()
    enc64 = H.encode(pos, lat, 1.0, tab, dtype=np.float64)
    _, cache = Fd.forward(enc64, dirs, w, dtype=np.float64)
    denc, gw = Fd.backward(gout, cache, w, dtype=np.float64)
    glat = H.encode_backward(pos, denc, 1.0, tab, dtype=np.float64)
    assert rel_err(f.position_encoder.latents.grad.cpu().numpy(), glat) <= 1e-4
    gwt = unpack_weights(f.weights.grad)
    for k in gw:
        assert rel_err(gwt[k].cpu().numpy(), gw[k], axis=None) <= 1e-4, k


def test_hashgrid_points_outside_the_box():
    """Points outside [-bound, bound] (negative scaled coordinates at the coarse levels): the
    weights follow modf's signed fractional part and the clip of encoders.py:204-212."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_forward
    rng = np.random.default_rng(21)
    tab = H.LevelTable(16, 1 << 14, 2, 16, 2048)
    t = LevelTable(16, 1 << 14, 2, 16, 2048)
    lat = rng.uniform(-1, 1, size=(tab.n_params, 2)).astype(np.float32)
    pos = rng.uniform(-1.6, 1.6, size=(20000, 3)).astype(np.float32)
    want = H.encode(pos, lat, 1.0, tab)
    got = hashgrid_forward(t, cu(pos), cu(lat), 1.0).cpu().numpy()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
def test_hashgrid_paired_and_single_row_paths_agree(dtype):
    """A 16-bit table whose base is aligned to a pair of rows fetches the two x-neighbour corners of
    an aligned row pair with one 8-byte load; a table that is not aligned (and every FP32 table)
    takes one load per corner.  Both give the oracle's encodings on the widened table; samples
    along rays make neighbouring lanes share corners, so the backward's segmented runs are
    exercised too."""
    from jaxngp_gb300.encoders import LevelTable, hashgrid_backward, hashgrid_forward
    rng = np.random.default_rng(7)
    tab_np = H.LevelTable(16, 2 ** 16, 2, 16, 2048)
    tab = LevelTable(16, 2 ** 16, 2, 16, 2048)
    R, m = 512, 64
    o = rng.uniform(-0.9, 0.9, size=(R, 1, 3))
    d = rng.normal(size=(R, 1, 3))
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    pos = (o + d * (0.01 * np.arange(m))[None, :, None]).reshape(-1, 3).astype(np.float32)
    lat = cu(rng.uniform(-1, 1, size=(tab_np.n_params, 2)).astype(np.float32)).to(dtype)
    store = torch.zeros(tab_np.n_params + 1, 2, dtype=dtype, device="cuda")
    store[1:] = lat
    single = store[1:]   # one row past an aligned base: not aligned to a pair of rows
    assert single.data_ptr() % (4 * single.element_size()) != 0
    a = hashgrid_forward(tab, cu(pos), lat, 1.0)
    b = hashgrid_forward(tab, cu(pos), single, 1.0)
    assert torch.equal(a, b)
    assert np.array_equal(a.cpu().numpy(), H.encode(pos, lat.float().cpu().numpy(), 1.0, tab_np))
    g = rng.normal(size=(R * m, 32)).astype(np.float32)
    ref = H.encode_backward(pos, g, 1.0, tab_np, dtype=np.float64)
    ga = hashgrid_backward(tab, cu(pos), cu(g), 1.0)
    assert rel_err(ga.cpu().numpy(), ref) <= RTOL
