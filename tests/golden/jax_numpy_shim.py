"""A NumPy stand-in for the parts of jax / flax / chex that the reference's field code uses.

TEST INFRASTRUCTURE ONLY.  JAX is not installed where the golden fixtures are made, so
``make_golden.py`` runs the reference's own ``models/encoders.py`` and ``models/nerfs.py``
unmodified on top of this module.  It implements, with JAX's dtype rules (Python floats become
float32, Python ints int32, weak scalars keep the array dtype):

* ``jax.numpy``: the array functions those files call;
* ``jax.vmap`` and the reference's ``vmap_jaxfn_with`` by explicit mapping;
* ``Array.at[...].set`` and ``jax.custom_vjp`` (forward only);
* ``flax.linen``: ``Module`` (a keyword-only dataclass with an explicit parameter tree),
  ``compact``, ``Dense`` (no bias), ``relu``, ``sigmoid``; ``Module.param`` returns the
  parameter supplied in the tree.

"""
from __future__ import annotations

import dataclasses
import functools
import importlib.util
import sys
import types

import numpy as np


# ------------------------------------------------------------------------------ arrays / dtypes

class Array(np.ndarray):
    """ndarray with JAX's functional `.at[idx].set(v)` update, and JAX's gather rule for integer
    index arrays: an index past either end of axis 0 is clamped to it."""

    def __getitem__(self, idx):
        if isinstance(idx, np.ndarray) and idx.dtype.kind in "iu":
            idx = np.clip(idx.astype(np.int64), 0, self.shape[0] - 1)
        return super().__getitem__(idx)

    @property
    def at(self):
        arr = self

        class _At:
            def __getitem__(self, idx):
                class _Upd:
                    def set(self, v):
                        out = np.array(arr, copy=True).view(Array)
                        out[idx] = v
                        return out
                return _Upd()
        return _At()


def _canon(a: np.ndarray) -> np.ndarray:
    if a.dtype == np.float64:
        a = a.astype(np.float32)
    elif a.dtype == np.int64:
        a = a.astype(np.int32)
    return a


def _wrap(a):
    return np.asarray(a).view(Array)


def asarray(x, dtype=None):
    a = np.asarray(x, dtype=dtype)
    if dtype is None:
        a = _canon(a)
    return a.view(Array)


def empty(shape, dtype=np.float32):
    return np.zeros(shape, dtype=dtype).view(Array)


def _passthrough(fn):
    @functools.wraps(fn)
    def g(*a, **k):
        r = fn(*a, **k)
        if isinstance(r, (tuple, list)):
            return type(r)(_wrap(x) for x in r)
        return _wrap(r)
    return g


jnp = types.ModuleType("jax.numpy")
for _name in ["floor", "modf", "clip", "prod", "stack", "sum", "mod", "concatenate", "ones_like",
              "zeros_like", "square", "exp", "split", "broadcast_to", "where", "maximum",
              "minimum", "sqrt", "isfinite", "signbit", "log"]:
    setattr(jnp, _name, _passthrough(getattr(np, _name)))
jnp.asarray = asarray
jnp.array = asarray
jnp.empty = empty
jnp.zeros = lambda shape, dtype=np.float32: np.zeros(shape, dtype).view(Array)
jnp.ones = lambda shape, dtype=np.float32: np.ones(shape, dtype).view(Array)
jnp.uint32, jnp.int32, jnp.float32, jnp.float16, jnp.bfloat16 = (np.uint32, np.int32, np.float32,
                                                                  np.float16, np.float32)
jnp.bool_ = np.bool_
jnp.linalg = np.linalg
jnp.ndarray = np.ndarray


def vmap(fn=None, in_axes=0, **_):
    """Map `fn` over axis 0 of the arguments whose in_axes entry is 0 (None = broadcast)."""
    if fn is None:
        return lambda f: vmap(f, in_axes=in_axes)

    @functools.wraps(fn)
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = next(np.asarray(a).shape[0] for a, ax in zip(args, axes) if ax == 0)
        outs = []
        for i in range(n):
            call = [a[i] if ax == 0 else a for a, ax in zip(args, axes)]
            outs.append(fn(*call))
        if isinstance(outs[0], tuple):
            return tuple(_wrap(np.stack(o)) for o in zip(*outs))
        return _wrap(np.stack(outs))
    return mapped


class custom_vjp:
    """Forward-only stand-in for jax.custom_vjp."""

    def __init__(self, fn):
        self.fn = fn
        functools.update_wrapper(self, fn)

    def defvjp(self, fwd=None, bwd=None):
        return None

    def __call__(self, *a, **k):
        return self.fn(*a, **k)


# --------------------------------------------------------------------------------- flax.linen

_call_stack = []


class Module:
    """Keyword-only dataclass modules with an explicit parameter tree (bind())."""

    def __init_subclass__(cls, **kw):
        super().__init_subclass__(**kw)
        if "__annotations__" in cls.__dict__ or "__dataclass_fields__" not in cls.__dict__:
            dataclasses.dataclass(cls, kw_only=True, eq=False)

    def bind(self, params):
        object.__setattr__(self, "_params", params)
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, Module):
                v.bind(params.get(f.name, {}))
        return self

    def param(self, name, init_fn, shape, dtype=np.float32):
        p = np.asarray(self._params[name])
        if tuple(p.shape) != tuple(shape):
            raise ValueError(f"param {name}: expected shape {shape}, got {p.shape}")
        return p.view(Array)


def compact(method):
    @functools.wraps(method)
    def wrapped(self, *a, **k):
        object.__setattr__(self, "_counters", {})
        _call_stack.append(self)
        try:
            return method(self, *a, **k)
        finally:
            _call_stack.pop()
    return wrapped


class Dense:
    """flax.linen.Dense without bias: y = x @ kernel, kernel shape [in, out], named Dense_i."""

    def __init__(self, features, use_bias=True, kernel_init=None, **_):
        if use_bias:
            raise NotImplementedError("bias not needed by the reference's field")
        self.features = features
        parent = _call_stack[-1]
        i = parent._counters.get("Dense", 0)
        parent._counters["Dense"] = i + 1
        self.kernel = np.asarray(parent._params[f"Dense_{i}"]["kernel"])

    def __call__(self, x):
        assert self.kernel.shape == (x.shape[-1], self.features)
        return _wrap(np.asarray(x) @ self.kernel)


def _relu(x):
    return _wrap(np.maximum(x, 0).astype(np.asarray(x).dtype))


def _sigmoid(x):
    x = np.asarray(x)
    return _wrap((1.0 / (1.0 + np.exp(-x))).astype(x.dtype))


# ------------------------------------------------------------------------------ installation

def _module(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


def _next_multiple(value: int, step: int) -> int:
    return (value + step - 1) // step * step


def _empty_impl(clz):
    if "__dataclass_fields__" not in clz.__dict__:
        raise TypeError(f"class `{clz.__name__}` is not a dataclass")
    return clz


def install():
    """Register the stand-in modules in sys.modules."""
    jax = _module("jax", numpy=jnp, vmap=vmap, jit=lambda f=None, **k: f if f else (lambda g: g),
                  custom_vjp=custom_vjp, Array=np.ndarray, ShapedArray=object)
    sys.modules["jax.numpy"] = jnp
    jax.random = _module("jax.random", uniform=None, normal=None, PRNGKey=None, split=None,
                         KeyArray=object)
    inits = _module("jax.nn.initializers", Initializer=object)
    jax.nn = _module("jax.nn", initializers=inits)
    linen = _module("flax.linen", Module=Module, compact=compact, Dense=Dense, relu=_relu,
                    sigmoid=_sigmoid,
                    initializers=types.SimpleNamespace(glorot_uniform=lambda: None))
    _module("flax.linen.dtypes", Dtype=object)
    _module("flax", linen=linen)
    _module("chex", assert_axis_dimension=lambda *a, **k: None, assert_shape=lambda *a, **k: None)
    _module("jaxtcnn", HashGridMetadata=object, hashgrid_encode=None)
    _module("shjax", spherical_harmonics_encoding=None)
    utils = _module("utils")
    utils.__path__ = []
    utils.common = _module(
        "utils.common", next_multiple=_next_multiple, jit_jaxfn_with=lambda **k: (lambda f: f),
        vmap_jaxfn_with=lambda in_axes=0, **k: (lambda f: vmap(f, in_axes=in_axes)),
        mkValueError=lambda **k: ValueError(str(k)))
    utils.types = _module("utils.types", empty_impl=_empty_impl, ActivationType=str,
                          DirectionalEncodingType=str, PositionalEncodingType=str)
    models = _module("models")
    models.__path__ = []


def load_reference_module(name: str, path: str):
    """Execute a reference source file, unmodified, as module `name`."""
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod
