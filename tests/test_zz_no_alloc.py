"""ngp_field_backward_noalloc: the field-MLP backward for callers that cannot allocate device memory
(an XLA custom call bound through the legacy signature gets only its operand and result buffers;
an embedder with a fixed memory budget may not call cudaMalloc).  Its scratch is a static array
inside the library, so this file runs last: the array must give the same results whether it is
touched for the first time here (a fresh process) or after every other test.

Bar: the same tolerance as the other field-MLP gradient tests, 1e-5 relative (column-wise
max|a - b| / max|b|), against ngp_field_backward with a caller-provided scratch buffer, on two
calls in a row with different inputs.
"""
import numpy as np
import pytest
import torch

from oracle import field as Fd

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def rel_err(a, b, axis=0):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b).max(axis=axis, keepdims=True), 1e-30)
    return (np.abs(a - b) / scale).max()


def _inputs(seed, n):
    rng = np.random.default_rng(seed)
    enc = torch.from_numpy(rng.normal(scale=0.5, size=(n, 32)).astype(np.float32)).cuda()
    d = rng.normal(size=(n, 3))
    dirs = torch.from_numpy((d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)).cuda()
    g = torch.from_numpy(rng.normal(size=(n, 4)).astype(np.float32)).cuda()
    from jaxngp_gb300.field import pack_weights
    w = pack_weights({k: torch.from_numpy(v) for k, v in Fd.init_weights(seed).items()}).cuda()
    return enc, dirs, w, g


def _with_scratch(enc, dirs, w, g, count=None, scale=None):
    from jaxngp_gb300 import _lib as L
    n = enc.shape[0]
    denc = torch.empty(n, 32, device="cuda")
    dw = torch.empty(L.MLP_WEIGHTS, device="cuda")
    scratch = torch.empty(L.field_backward_scratch_floats(), device="cuda")
    L.call("ngp_field_backward", [enc, dirs, w, g, count, scale, scratch, denc, dw], L.NgpMlpDescriptor(n, 0))
    return denc, dw


def _no_alloc(enc, dirs, w, g, count=None, scale=None):
    from jaxngp_gb300 import _lib as L
    n = enc.shape[0]
    denc = torch.empty(n, 32, device="cuda")
    dw = torch.empty(L.MLP_WEIGHTS, device="cuda")
    L.call("ngp_field_backward_noalloc", [enc, dirs, w, g, count, scale, denc, dw], L.NgpMlpDescriptor(n, 0))
    return denc, dw


def test_noalloc_matches_scratch_entry_twice():
    """Two calls in a row (different sizes, so the second reuses a prefix of what the first wrote),
    each against the scratch-taking entry point."""
    for seed, n in [(1, 300000), (2, 70001)]:
        enc, dirs, w, g = _inputs(seed, n)
        a_enc, a_w = _no_alloc(enc, dirs, w, g)
        b_enc, b_w = _with_scratch(enc, dirs, w, g)
        torch.cuda.synchronize()
        assert rel_err(a_enc.cpu().numpy(), b_enc.cpu().numpy()) <= RTOL
        assert rel_err(a_w.cpu().numpy(), b_w.cpu().numpy(), axis=None) <= RTOL


def test_noalloc_active_count_and_scale():
    enc, dirs, w, g = _inputs(3, 5000)
    cnt = torch.tensor([3777], dtype=torch.int32, device="cuda")
    scale = torch.tensor([0.25], dtype=torch.float32, device="cuda")
    a_enc, a_w = _no_alloc(enc, dirs, w, g, cnt, scale)
    b_enc, b_w = _with_scratch(enc, dirs, w, g, cnt, scale)
    assert rel_err(a_enc.cpu().numpy(), b_enc.cpu().numpy()) <= RTOL
    assert rel_err(a_w.cpu().numpy(), b_w.cpu().numpy(), axis=None) <= RTOL
    assert not a_enc[3777:].any()


def test_noalloc_rejects_oversized_batch():
    from jaxngp_gb300 import _lib as L
    n = 524288 + 1
    x = torch.zeros(n, 32, device="cuda")
    with pytest.raises(L.NgpError) as e:
        L.call("ngp_field_backward_noalloc", [x, torch.zeros(n, 3, device="cuda"), torch.zeros(L.MLP_WEIGHTS, device="cuda"),
                                              torch.zeros(n, 4, device="cuda"), None, None, x,
                                              torch.zeros(L.MLP_WEIGHTS, device="cuda")], L.NgpMlpDescriptor(n, 0))
    assert e.value.status == 5 and "524288" in str(e.value)
