"""The XLA custom-call registration of INTEGRATION.md, up to the JAX call (JAX is not installed
here or on the GPU machine): every volrendjax target and shjax's is exported by the library, wraps
into the `xla._CUSTOM_CALL_TARGET` capsule that `xla_client.register_custom_call_target` takes,
and the capsule carries the function's own address.  No GPU needed."""
import ctypes
import os

import pytest

TARGETS = ["pack_density_into_bits", "march_rays", "march_rays_inference", "morton3d", "morton3d_invert",
           "integrate_rays", "integrate_rays_backward", "integrate_rays_inference",
           "spherical_harmonics_encoding_cuda_f32"]


def _lib():
    from jaxngp_gb300 import _lib as L
    if not os.path.exists(L.LIB_PATH):
        pytest.skip("the library is not built")
    return ctypes.CDLL(L.LIB_PATH)


def test_capsules_carry_the_targets():
    lib = _lib()
    new = ctypes.pythonapi.PyCapsule_New
    new.restype = ctypes.py_object
    new.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
    get = ctypes.pythonapi.PyCapsule_GetPointer
    get.restype = ctypes.c_void_p
    get.argtypes = [ctypes.py_object, ctypes.c_char_p]
    valid = ctypes.pythonapi.PyCapsule_IsValid
    valid.restype = ctypes.c_int
    valid.argtypes = [ctypes.py_object, ctypes.c_char_p]
    name = b"xla._CUSTOM_CALL_TARGET"
    for t in TARGETS:
        fn = ctypes.cast(getattr(lib, t), ctypes.c_void_p).value
        assert fn
        cap = new(fn, name, None)
        assert valid(cap, name) == 1
        assert get(cap, name) == fn
        # the status twin exists beside every target
        assert ctypes.cast(getattr(lib, t + "_status"), ctypes.c_void_p).value


def test_jax_absent_is_recorded():
    """The JAX side of the snippet needs jax; where it imports, register the targets for real."""
    try:
        from jax.lib import xla_client  # noqa: F401
    except ImportError:
        pytest.skip("jax is not installed (JAX registration exercised up to the capsule)")
    lib = _lib()
    new = ctypes.pythonapi.PyCapsule_New
    new.restype = ctypes.py_object
    new.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
    for t in TARGETS:
        fn = ctypes.cast(getattr(lib, t), ctypes.c_void_p).value
        xla_client.register_custom_call_target(t, new(fn, b"xla._CUSTOM_CALL_TARGET", None), platform="gpu")
