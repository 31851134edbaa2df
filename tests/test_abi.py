"""The C-ABI library without a GPU: it loads, exports every function include/ngp_gb300.h declares,
and the ctypes descriptor structs have the header's sizes and field offsets (no compute calls)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ngp_gb300.h")
DECL = re.compile(r"^(?:const\s+)?(?:void|int|unsigned long long|size_t|char)\s*\**\s*(\w+)\s*\(", re.M)


def declared():
    return sorted(set(DECL.findall(open(HEADER).read())))


@pytest.fixture(scope="module")
def lib():
    from jaxngp_gb300 import _lib as L
    if not os.path.exists(L.LIB_PATH):
        from jaxngp_gb300 import build
        build.build()
    return ctypes.CDLL(L.LIB_PATH)


def test_header_declares_the_volrendjax_targets():
    names = declared()
    for t in ["pack_density_into_bits", "march_rays", "march_rays_inference", "morton3d", "morton3d_invert",
              "integrate_rays", "integrate_rays_backward", "integrate_rays_inference"]:
        assert t in names and t + "_status" in names
    assert len(names) > 40


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_queries_without_a_gpu(lib):
    assert lib.ngp_abi_version() == 1
    assert lib.ngp_last_status() == 0
    lib.ngp_kernel_launches.restype = ctypes.c_ulonglong
    assert lib.ngp_kernel_launches() >= 0
    lib.ngp_last_status_message.restype = ctypes.c_char_p
    assert isinstance(lib.ngp_last_status_message(), bytes)


def test_descriptor_layouts_match_header(tmp_path):
    """sizeof and offsetof of every descriptor, from a C program compiled against the header."""
    from jaxngp_gb300 import _lib as L
    cc = shutil.which("gcc")
    cuda_inc = "/usr/local/cuda/include"
    if cc is None or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime_api.h")):
        pytest.skip("gcc or the CUDA headers are not available")
    structs = {n: getattr(L, n) for n in dir(L)
               if isinstance(getattr(L, n), type) and issubclass(getattr(L, n), L._Desc) and getattr(L, n) is not L._Desc}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ngp_gb300.h"', "int main(void) {"]
    expect = []
    for name, cls in sorted(structs.items()):
        lines.append(f'printf("%zu\\n", sizeof({name}));')
        expect.append(ctypes.sizeof(cls))
        for fname, _ in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({name}, {fname}));')
            expect.append(getattr(cls, fname).offset)
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, str(src), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect
    assert len(structs) >= 14
