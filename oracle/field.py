"""CPU oracle for the NeRF field (density MLP, SH encoding, colour MLP).  TEST INFRASTRUCTURE ONLY.

NumPy restatement of ``make_nerf_ngp`` (models/nerfs.py:422-454) / ``NeRF.__call__``
(nerfs.py:39-86) / ``CoordinateBasedMLP`` (nerfs.py:89-128), the truncated exponential
(nerfs.py:216-238), ``SphericalHarmonicsEncoder`` degree 4 (models/encoders.py:360-406), with the
hand-derived backward that JAX's autodiff computes for it.  All layers are bias-free Dense layers
(kernel ``[in, out]``):

    density:  h1 = relu(enc @ W0)  (32->64);   x = h1 @ W1  (64->16);   sigma = exp(x[:, 0])
    colour:   h2 = relu([x, SH4(dir)] @ W2)  (32->64);   h3 = relu(h2 @ W3)  (64->64)
              rgb = sigmoid(h3 @ W4)  (64->3)
    output:   drgb = [sigma, rgb]

The backward of sigma uses exp(clip(x0, -15, 15)) (nerfs.py:230-234); relu passes gradient where
its input is > 0.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

SHAPES = {"W0": (32, 64), "W1": (64, 16), "W2": (32, 64), "W3": (64, 64), "W4": (64, 3)}


def glorot_uniform(rng: np.random.Generator, shape, dtype=np.float32) -> np.ndarray:
    lim = np.sqrt(6.0 / (shape[0] + shape[1]))
    return rng.uniform(-lim, lim, size=shape).astype(dtype)


def init_weights(seed: int = 0, dtype=np.float32) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    return {k: glorot_uniform(rng, s, dtype) for k, s in SHAPES.items()}


def to_flax_params(w: Dict[str, np.ndarray]) -> dict:
    """The reference's parameter tree for these weights (flax names Dense_i/kernel)."""
    return {
        "density_mlp": {"Dense_0": {"kernel": w["W0"]}, "Dense_1": {"kernel": w["W1"]}},
        "rgb_mlp": {"Dense_0": {"kernel": w["W2"]}, "Dense_1": {"kernel": w["W3"]},
                    "Dense_2": {"kernel": w["W4"]}},
    }


def sh4(d: np.ndarray) -> np.ndarray:
    """encoders.py:375-406, degrees 0..3 (16 outputs), in the input's dtype."""
    d = np.asarray(d)
    t = d.dtype.type
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    xy, xz, yz = x * y, x * z, y * z
    x2, y2, z2 = x * x, y * y, z * z
    out = np.empty(d.shape[:-1] + (16,), d.dtype)
    out[..., 0] = t(0.28209479177387814)
    out[..., 1] = t(-0.48860251190291987) * y
    out[..., 2] = t(0.48860251190291987) * z
    out[..., 3] = t(-0.48860251190291987) * x
    out[..., 4] = t(1.0925484305920792) * xy
    out[..., 5] = t(-1.0925484305920792) * yz
    out[..., 6] = t(0.94617469575755997) * z2 - t(0.31539156525251999)
    out[..., 7] = t(-1.0925484305920792) * xz
    out[..., 8] = t(0.54627421529603959) * x2 - t(0.54627421529603959) * y2
    out[..., 9] = t(0.59004358992664352) * y * (t(-3.0) * x2 + y2)
    out[..., 10] = t(2.8906114426405538) * xy * z
    out[..., 11] = t(0.45704579946446572) * y * (t(1.0) - t(5.0) * z2)
    out[..., 12] = t(0.3731763325901154) * z * (t(5.0) * z2 - t(3.0))
    out[..., 13] = t(0.45704579946446572) * x * (t(1.0) - t(5.0) * z2)
    out[..., 14] = t(1.4453057213202769) * z * (x2 - y2)
    out[..., 15] = t(0.59004358992664352) * x * (-x2 + t(3.0) * y2)
    return out


def forward(enc: np.ndarray, dirs: np.ndarray, w: Dict[str, np.ndarray], dtype=np.float32):
    """Returns (drgb [S,4], cache) in `dtype`."""
    w = {k: np.asarray(v, dtype) for k, v in w.items()}
    enc = np.asarray(enc, dtype)
    a1 = enc @ w["W0"]
    h1 = np.maximum(a1, 0)
    x = h1 @ w["W1"]
    sigma = np.exp(x[:, :1])
    sh = sh4(np.asarray(dirs, dtype))
    c = np.concatenate([x, sh], axis=-1)
    a2 = c @ w["W2"]
    h2 = np.maximum(a2, 0)
    a3 = h2 @ w["W3"]
    h3 = np.maximum(a3, 0)
    a4 = h3 @ w["W4"]
    rgb = 1 / (1 + np.exp(-a4))
    drgb = np.concatenate([sigma, rgb], axis=-1).astype(dtype)
    cache = dict(enc=enc, a1=a1, h1=h1, x=x, c=c, a2=a2, h2=h2, a3=a3, h3=h3, rgb=rgb)
    return drgb, cache


def backward(dL_ddrgb: np.ndarray, cache, w: Dict[str, np.ndarray], dtype=np.float64):
    """Returns (dL_denc [S,32], dict of dL_dW)."""
    w = {k: np.asarray(v, dtype) for k, v in w.items()}
    c = {k: np.asarray(v, dtype) for k, v in cache.items()}
    g = np.asarray(dL_ddrgb, dtype)
    dx0 = g[:, 0] * np.exp(np.clip(c["x"][:, 0], -15, 15))
    rgb = c["rgb"]
    da4 = g[:, 1:] * rgb * (1 - rgb)
    grads = {"W4": c["h3"].T @ da4}
    da3 = (da4 @ w["W4"].T) * (c["a3"] > 0)
    grads["W3"] = c["h2"].T @ da3
    da2 = (da3 @ w["W3"].T) * (c["a2"] > 0)
    grads["W2"] = c["c"].T @ da2
    dc = da2 @ w["W2"].T
    dx = dc[:, :16].copy()
    dx[:, 0] += dx0
    grads["W1"] = c["h1"].T @ dx
    da1 = (dx @ w["W1"].T) * (c["a1"] > 0)
    grads["W0"] = c["enc"].T @ da1
    denc = da1 @ w["W0"].T
    return denc, grads


def kink_flip_tolerance(dL_ddrgb: np.ndarray, cache, w: Dict[str, np.ndarray], rel: float = 1e-6):
    """What ReLU decisions within rounding of a kink can move in the backward.  A pre-activation a
    with |a| <= rel * sum_k |x_k w_k| (x its layer input, w its weight column) may come out on either
    side of 0 in any float32-accurate evaluation of the layer; for every such entry the bound adds
    |backward of that one sample with the decision flipped - backward without| (FP64, one flip at a
    time; `cache` from forward(..., dtype=np.float64)).  Returns (dict of per-element bounds on
    dL/dW, per-element bounds on dL/denc [S, 32], number of such entries)."""
    w64 = {k: np.asarray(v, np.float64) for k, v in w.items()}
    g = np.asarray(dL_ddrgb, np.float64)
    tol_w = {k: np.zeros_like(v) for k, v in w64.items()}
    tol_enc = np.zeros((g.shape[0], w64["W0"].shape[0]))
    n_near = 0
    for a_key, x_key, w_key in (("a1", "enc", "W0"), ("a2", "c", "W2"), ("a3", "h2", "W3")):
        a = np.asarray(cache[a_key], np.float64)
        absum = np.abs(np.asarray(cache[x_key], np.float64)) @ np.abs(w64[w_key])
        for s, u in np.argwhere(np.abs(a) <= rel * absum):
            n_near += 1
            one = {k: np.array(v[s:s + 1], np.float64) for k, v in cache.items()}
            enc0, gw0 = backward(g[s:s + 1], one, w64)
            one[a_key][0, u] = -a[s, u] if a[s, u] != 0 else 1e-300
            enc1, gw1 = backward(g[s:s + 1], one, w64)
            for k in tol_w:
                tol_w[k] += np.abs(gw1[k] - gw0[k])
            tol_enc[s] += np.abs(enc1 - enc0)[0]
    return tol_w, tol_enc, n_near


def round_bf16(x) -> np.ndarray:
    """float32 values rounded to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def round_f16(x) -> np.ndarray:
    """float32 values rounded to IEEE half precision (nearest, ties to even; overflow to inf),
    returned as float32."""
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float32)


ROUNDERS = {"bf16": round_bf16, "fp16": round_f16}


def forward_half(enc: np.ndarray, dirs: np.ndarray, w: Dict[str, np.ndarray], operand: str = "bf16"):
    """The tensor-core forward restated for a 16-bit operand type: every MMA operand (weights,
    encodings, layer inputs) rounded to that type, products accumulated exactly (FP64 here, FP32
    on the GPU).  Returns (drgb [S,4] float64, cache)."""
    rnd = ROUNDERS[operand]

    def h(x):
        return rnd(np.asarray(x, np.float32)).astype(np.float64)

    wb = {k: h(v) for k, v in w.items()}
    enc_b = h(enc)
    a1 = enc_b @ wb["W0"]
    h1 = h(np.maximum(a1, 0))
    x = h1 @ wb["W1"]
    sigma = np.exp(x[:, :1])
    sh = sh4(np.asarray(dirs, np.float32)).astype(np.float64)
    c = h(np.concatenate([x, sh], axis=-1))
    a2 = c @ wb["W2"]
    h2 = h(np.maximum(a2, 0))
    a3 = h2 @ wb["W3"]
    h3 = h(np.maximum(a3, 0))
    a4 = h3 @ wb["W4"]
    rgb = 1 / (1 + np.exp(-a4))
    drgb = np.concatenate([sigma, rgb], axis=-1)
    return drgb, dict(enc=enc_b, h1=h1, x=x, c=c, h2=h2, h3=h3, rgb=rgb, wb=wb, operand=operand)


def backward_half(dL_ddrgb: np.ndarray, cache, grad_scale: float = 1.0):
    """The tensor-core backward restated: each layer's output gradient (times grad_scale, which
    includes any loss scale) is rounded to the operand type before it enters the data- and
    weight-gradient MMAs; relu masks come from the 16-bit layer inputs.  Returns (dL_denc [S,32],
    dict of dL_dW) in float64, both still multiplied by grad_scale."""
    rnd = ROUNDERS[cache["operand"]]

    def h(x):
        return rnd(np.asarray(x, np.float32)).astype(np.float64)

    c, wb = cache, cache["wb"]
    g = np.asarray(dL_ddrgb, np.float64) * grad_scale
    dx0 = g[:, 0] * np.exp(np.clip(c["x"][:, 0], -15, 15))
    rgb = c["rgb"]
    d4 = np.zeros((g.shape[0], 3))
    d4[:] = g[:, 1:] * rgb * (1 - rgb)
    d4 = h(d4)
    grads = {"W4": c["h3"].T @ d4}
    d3 = h((d4 @ wb["W4"].T) * (c["h3"] > 0))
    grads["W3"] = c["h2"].T @ d3
    d2 = h((d3 @ wb["W3"].T) * (c["h2"] > 0))
    grads["W2"] = c["c"].T @ d2
    dx = d2 @ wb["W2"][:16].T
    dx[:, 0] += dx0
    dx = h(dx)
    grads["W1"] = c["h1"].T @ dx
    d1 = h((dx @ wb["W1"].T) * (c["h1"] > 0))
    grads["W0"] = c["enc"].T @ d1
    denc = d1 @ wb["W0"].T
    return denc, grads


def forward_bf16(enc: np.ndarray, dirs: np.ndarray, w: Dict[str, np.ndarray]):
    """forward_half with BF16 operands."""
    return forward_half(enc, dirs, w, "bf16")


def backward_bf16(dL_ddrgb: np.ndarray, cache, grad_scale: float = 1.0):
    """backward_half of a forward_bf16 cache."""
    return backward_half(dL_ddrgb, cache, grad_scale)


def _fma32(a, b, c):
    """round_f32(a * b + c) with one rounding: the product of two float32 values is exact in
    float64, so only the sum rounds twice (float64, then float32), which differs from a fused
    multiply-add only when the float64 sum lands exactly halfway between two float32 values."""
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def _fma_chain(A: np.ndarray, W: np.ndarray) -> np.ndarray:
    """C[s][n] = sum_k A[s][k] W[k][n] as a float32 multiply-add chain in k order, from 0."""
    A64, W64 = np.asarray(A, np.float32).astype(np.float64), np.asarray(W, np.float32).astype(np.float64)
    acc = np.zeros((A64.shape[0], W64.shape[1]), np.float32)
    for k in range(A64.shape[1]):
        acc = (acc.astype(np.float64) + A64[:, k:k + 1] * W64[k][None, :]).astype(np.float32)
    return acc


def sh4_fma32(d: np.ndarray) -> np.ndarray:
    """sh4 in float32 with each a*b + c formed as one multiply-add, as a GPU compiler that
    contracts multiply-adds evaluates encoders.py:375-406's expressions."""
    d = np.asarray(d, np.float32)
    t = np.float32
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xy, xz, yz = x * y, x * z, y * z
    x2, y2, z2 = x * x, y * y, z * z
    out = np.empty((d.shape[0], 16), np.float32)
    out[:, 0] = t(0.28209479177387814)
    out[:, 1] = t(-0.48860251190291987) * y
    out[:, 2] = t(0.48860251190291987) * z
    out[:, 3] = t(-0.48860251190291987) * x
    out[:, 4] = t(1.0925484305920792) * xy
    out[:, 5] = t(-1.0925484305920792) * yz
    out[:, 6] = _fma32(t(0.94617469575755997), z2, -t(0.31539156525251999))
    out[:, 7] = t(-1.0925484305920792) * xz
    out[:, 8] = _fma32(t(0.54627421529603959), x2, -(t(0.54627421529603959) * y2))
    out[:, 9] = (t(0.59004358992664352) * y) * _fma32(t(-3.0), x2, y2)
    out[:, 10] = (t(2.8906114426405538) * xy) * z
    out[:, 11] = (t(0.45704579946446572) * y) * _fma32(t(-5.0), z2, t(1.0))
    out[:, 12] = (t(0.3731763325901154) * z) * _fma32(t(5.0), z2, t(-3.0))
    out[:, 13] = (t(0.45704579946446572) * x) * _fma32(t(-5.0), z2, t(1.0))
    out[:, 14] = (t(1.4453057213202769) * z) * (x2 - y2)
    out[:, 15] = (t(0.59004358992664352) * x) * _fma32(t(3.0), y2, -x2)
    return out


def forward_fma32(enc: np.ndarray, dirs: np.ndarray, w: Dict[str, np.ndarray]):
    """The field forward in float32 evaluated the way the FP32 SIMT kernel (mlp.cu) does: every
    layer output a multiply-add chain over its inputs in order, SH with contracted multiply-adds.
    Its pre-activations, and so its ReLU decisions, are the kernel's; a backward in float64 on
    this cache (`backward(..., cache)`) is the kernel's gradient without its rounding, which is how
    gradient parity is judged on whole batches where some pre-activations sit within float32
    rounding of a ReLU kink.  Returns (drgb [S,4] float32, cache)."""
    w = {k: np.asarray(v, np.float32) for k, v in w.items()}
    enc = np.asarray(enc, np.float32)
    a1 = _fma_chain(enc, w["W0"])
    h1 = np.maximum(a1, np.float32(0))
    x = _fma_chain(h1, w["W1"])
    c = np.concatenate([x, sh4_fma32(dirs)], axis=-1)
    a2 = _fma_chain(c, w["W2"])
    h2 = np.maximum(a2, np.float32(0))
    a3 = _fma_chain(h2, w["W3"])
    h3 = np.maximum(a3, np.float32(0))
    a4 = _fma_chain(h3, w["W4"])
    rgb = (np.float32(1) / (np.float32(1) + np.exp(-a4))).astype(np.float32)
    drgb = np.concatenate([np.exp(x[:, :1]), rgb], axis=-1).astype(np.float32)
    cache = dict(enc=enc, a1=a1, h1=h1, x=x, c=c, a2=a2, h2=h2, a3=a3, h3=h3, rgb=rgb)
    return drgb, cache


def density_only(enc: np.ndarray, w: Dict[str, np.ndarray], dtype=np.float32) -> np.ndarray:
    """NeRF.__call__ with dir=None (nerfs.py:71-72): sigma [S]."""
    w = {k: np.asarray(v, dtype) for k, v in w.items()}
    h1 = np.maximum(np.asarray(enc, dtype) @ w["W0"], 0)
    return np.exp((h1 @ w["W1"])[:, 0])


def kink_distance(enc: np.ndarray, dirs: np.ndarray, w: Dict[str, np.ndarray]) -> np.ndarray:
    """Per sample, the smallest |pre-activation| of the three ReLU layers relative to that layer's
    largest |pre-activation| over the batch (FP64).  Samples near 0 sit on a ReLU kink, where
    float32 evaluations may take either side and the gradient jumps; parity tests of gradients
    leave them out."""
    _, c = forward(enc, dirs, w, dtype=np.float64)
    out = np.full(np.asarray(enc).shape[0], np.inf)
    for k in ("a1", "a2", "a3"):
        a = np.abs(c[k])
        out = np.minimum(out, (a / a.max()).min(axis=1))
    return out


# ------------------------------------------------------------------ FP32 accuracy from BF16 pieces
#
# Restatement, as a checker, of the operand split the FP32 field kernels use on the tensor cores
# (jaxngp_gb300/csrc/mlp_tc.cu: split3, mma_kk_x6, mma_mn_x6): every matmul operand x becomes BF16
# pieces x1 = bf16(x), x2 = bf16(x - x1), x3 = bf16(x - x1 - x2), the differences taken in float32
# (exact there), and a matmul sums a chosen set of piece products.  Products are summed exactly
# (float64) and the result rounded once to float32, so these functions measure the error of the
# split itself, without the FP32 accumulator's own rounding.  No counterpart in the reference,
# whose MLP runs in FP32 (models/nerfs.py:39-128).

SPLIT_SCHEMES = {
    # name: (pieces per operand, (i, j) piece products, smallest first)
    "x6": (3, ((2, 0), (1, 1), (0, 2), (1, 0), (0, 1), (0, 0))),   # the kernels' scheme
    "x4": (2, ((1, 1), (1, 0), (0, 1), (0, 0))),
    "x3": (2, ((1, 0), (0, 1), (0, 0))),
}


def split_bf16(x, pieces: int = 3):
    """The BF16 pieces of float32 `x` (as float64 arrays), first piece first."""
    r = np.asarray(x, np.float32)
    out = []
    for _ in range(pieces):
        p = round_bf16(r)
        out.append(p.astype(np.float64))
        r = (r - p).astype(np.float32)
    return out


def matmul_split(A, B, scheme: str = "x6") -> np.ndarray:
    """A @ B from the scheme's products of BF16 pieces, summed exactly, rounded to float32."""
    n, prods = SPLIT_SCHEMES[scheme]
    a, b = split_bf16(A, n), split_bf16(B, n)
    return sum(a[i] @ b[j] for i, j in prods).astype(np.float32)


def forward_split(enc: np.ndarray, dirs: np.ndarray, w: Dict[str, np.ndarray], scheme: str = "x6"):
    """forward() with every matmul in split form and float32 in between (as the kernel: FP32
    layer outputs, ReLU, exp and sigmoid in float32).  Returns (drgb [S,4], cache)."""
    mm = lambda a, b: matmul_split(a, b, scheme)
    w = {k: np.asarray(v, np.float32) for k, v in w.items()}
    enc = np.asarray(enc, np.float32)
    a1 = mm(enc, w["W0"])
    h1 = np.maximum(a1, 0)
    x = mm(h1, w["W1"])
    sigma = np.exp(x[:, :1])
    c = np.concatenate([x, sh4(np.asarray(dirs, np.float32))], axis=-1)
    a2 = mm(c, w["W2"])
    h2 = np.maximum(a2, 0)
    a3 = mm(h2, w["W3"])
    h3 = np.maximum(a3, 0)
    a4 = mm(h3, w["W4"])
    rgb = (1 / (1 + np.exp(-a4))).astype(np.float32)
    drgb = np.concatenate([sigma, rgb], axis=-1).astype(np.float32)
    return drgb, dict(enc=enc, a1=a1, h1=h1, x=x, c=c, a2=a2, h2=h2, a3=a3, h3=h3, rgb=rgb)


def backward_split(dL_ddrgb: np.ndarray, cache, w: Dict[str, np.ndarray], scheme: str = "x6"):
    """backward() with every matmul (data and weight gradients) in split form, float32 in between;
    `cache` from forward_split.  Returns (dL_denc [S,32], dict of dL_dW)."""
    mm = lambda a, b: matmul_split(a, b, scheme)
    w = {k: np.asarray(v, np.float32) for k, v in w.items()}
    c = cache
    g = np.asarray(dL_ddrgb, np.float32)
    dx0 = (g[:, 0] * np.exp(np.clip(c["x"][:, 0], -15, 15))).astype(np.float32)
    rgb = c["rgb"]
    da4 = (g[:, 1:] * rgb * (1 - rgb)).astype(np.float32)
    grads = {"W4": mm(c["h3"].T, da4)}
    da3 = mm(da4, w["W4"].T) * (c["a3"] > 0)
    grads["W3"] = mm(c["h2"].T, da3)
    da2 = mm(da3, w["W3"].T) * (c["a2"] > 0)
    grads["W2"] = mm(c["c"].T, da2)
    dx = mm(da2, w["W2"][:16].T)
    dx[:, 0] += dx0
    grads["W1"] = mm(c["h1"].T, dx)
    da1 = mm(dx, w["W1"].T) * (c["a1"] > 0)
    grads["W0"] = mm(c["enc"].T, da1)
    return mm(da1, w["W0"].T), grads
