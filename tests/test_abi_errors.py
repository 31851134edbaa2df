"""Error statuses of the C ABI without a GPU: a wrong opaque length, out-of-contract descriptor
fields, missing required buffers and misaligned operands are rejected before any CUDA call, with
the status the header documents (NGP_ERR_OPAQUE_SIZE = 1, NGP_ERR_INVALID_ARGUMENT = 2), also
through the legacy void signature (ngp_last_status)."""
import ctypes

import pytest

OPAQUE_SIZE, INVALID = 1, 2


@pytest.fixture(scope="module")
def lib():
    import os
    from jaxngp_gb300 import _lib as L
    if not os.path.exists(L.LIB_PATH):
        from jaxngp_gb300 import build
        build.build()
    return ctypes.CDLL(L.LIB_PATH)


def call(lib, name, buffers, desc):
    """The `_status` entry with host-side pointers (never dereferenced on these error paths)."""
    arr = (ctypes.c_void_p * len(buffers))(*buffers)
    raw = bytes(desc) if not isinstance(desc, bytes) else desc
    f = getattr(lib, name + "_status")
    f.restype = ctypes.c_int
    return f(ctypes.c_void_p(0), arr, ctypes.c_char_p(raw), ctypes.c_size_t(len(raw)))


def tv_desc(**kw):
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.encoders import LevelTable
    d = L.NgpHashGridTVDescriptor(LevelTable(16, 1 << 14, 2, 16, 2048).descriptor(100, 1.0), 0.5, 1)
    for k, v in kw.items():
        setattr(d.grid if k in ("L", "F", "n_params") else d, k, v)
    return d


def test_hashgrid_tv_errors(lib):
    ok = [0x1000, 0x2000, 0, 0x3000, 0x4000, 0x5000]   # pos, latents, grad_scale, tv, grad, scratch
    assert call(lib, "ngp_hashgrid_tv", ok, b"short") == OPAQUE_SIZE
    assert call(lib, "ngp_hashgrid_tv", ok, tv_desc(L=0)) == INVALID          # no levels
    assert call(lib, "ngp_hashgrid_tv", ok, tv_desc(L=33)) == INVALID         # more than 32
    assert call(lib, "ngp_hashgrid_tv", ok, tv_desc(F=4)) == INVALID          # two features only
    assert call(lib, "ngp_hashgrid_tv", ok[:5] + [0], tv_desc()) == INVALID   # no scratch
    assert call(lib, "ngp_hashgrid_tv", [0x1000, 0x2004] + ok[2:], tv_desc()) == INVALID   # latents misaligned
    assert call(lib, "ngp_hashgrid_tv", ok[:5] + [0x5004], tv_desc()) == INVALID           # scratch misaligned


def test_integrate_rays_fp64_errors(lib):
    from jaxngp_gb300 import _lib as L
    d = L.IntegratingDescriptor(10, 100)
    ok = [0x1000, 0x2000, 0x3000, 0x4000, 0x5000, 0x6000, 0x7000, 0x8000, 0x9000]
    assert call(lib, "ngp_integrate_rays_fp64", ok, b"x" * 3) == OPAQUE_SIZE
    assert call(lib, "ngp_integrate_rays_fp64", ok[:5] + [0x6008] + ok[6:], d) == INVALID   # drgbs not 16-byte
    assert call(lib, "ngp_integrate_rays_fp64", ok[:6] + [0x7004] + ok[7:], d) == INVALID   # rgbd not 8-byte


def test_march_rays_fallback_errors(lib):
    from jaxngp_gb300 import _lib as L
    ok = [0x1000 * (i + 1) for i in range(19)]
    assert call(lib, "ngp_march_rays_fallback", ok, b"") == OPAQUE_SIZE
    assert call(lib, "ngp_march_rays_fallback", ok, L.MarchingDescriptor(8, 64, 1024, 0, 128, 1.0, 0.0)) == INVALID  # K = 0
    assert call(lib, "ngp_march_rays_fallback", ok, L.MarchingDescriptor(8, 64, 1024, 1, 96, 1.0, 0.0)) == INVALID  # G
    assert call(lib, "ngp_march_rays_fallback", ok, L.MarchingDescriptor(8, 64, 1024, 1, 2048, 1.0, 0.0)) == INVALID
    assert call(lib, "ngp_march_rays_fallback", ok[:16] + [0] + ok[17:],
                L.MarchingDescriptor(8, 64, 1024, 1, 128, 1.0, 0.0)) == INVALID   # no queue


def test_legacy_signature_records_the_status(lib):
    arr = (ctypes.c_void_p * 6)(0x1000, 0x2000, 0, 0x3000, 0x4000, 0x5000)
    lib.ngp_hashgrid_tv(ctypes.c_void_p(0), arr, ctypes.c_char_p(b"xy"), ctypes.c_size_t(2))
    lib.ngp_last_status.restype = ctypes.c_int
    assert lib.ngp_last_status() == OPAQUE_SIZE
    lib.ngp_last_status_message.restype = ctypes.c_char_p
    assert b"length" in lib.ngp_last_status_message()


def test_every_entry_rejects_missing_buffers_and_bad_descriptors(lib):
    """Every `_status` entry the header declares returns INVALID for a NULL buffer array; every
    entry that takes a descriptor returns OPAQUE_SIZE for an opaque of the wrong length; the one
    without a descriptor (ngp_march_count) returns INVALID for missing buffers -- all before any
    CUDA call."""
    import os
    import re
    header = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                               "ngp_gb300.h")).read()
    names = re.findall(r"int (\w+)_status\(cudaStream_t stream, void \*\*buffers, const char \*opaque, "
                       r"size_t opaque_len\);", header)
    assert len(names) >= 50
    nulls = (ctypes.c_void_p * 32)()
    for n in names:
        f = getattr(lib, n + "_status")
        f.restype = ctypes.c_int
        assert f(ctypes.c_void_p(0), None, ctypes.c_char_p(b"x"), ctypes.c_size_t(1)) == INVALID, n
        want = INVALID if n == "ngp_march_count" else OPAQUE_SIZE
        assert f(ctypes.c_void_p(0), nulls, ctypes.c_char_p(b"x"), ctypes.c_size_t(1)) == want, n
