"""CPU tests of the C-ABI boundary: the library loads and exports every
entry point the public headers declare; context-free calls work without a GPU."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "rajzel_gb300")


def declared(header):
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:int|void|char|double|float)\s*\*?\s*(\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def built():
    from rajzel_gb300 import build as B
    B.build()
    return B


def test_headers_declare_entry_points():
    names = declared(os.path.join(ROOT, "include", "rajzel_gb300.h"))
    for n in ["rz_create", "rz_set_grid", "rz_set_slowness", "rz_set_receivers", "rz_forward", "rz_grad_obj",
              "rz_eikonal", "rz_eikonal_adj"]:
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(built.LIB)
    missing = [n for n in declared(os.path.join(ROOT, "include", "rajzel_gb300.h")) if not hasattr(lib, n)]
    assert not missing, missing


def test_compat_library_exports_reference_signatures(built):
    hdr = os.path.join(ROOT, "include", "rajzel_compat.h")
    if not os.path.exists(built.COMPAT):
        pytest.skip("compat shim not built")
    names = declared(hdr)
    assert {"eikonal", "eikonal_adj", "grad_obj", "forward"} <= set(names)
    out = os.popen(f"nm -D --defined-only {built.COMPAT}").read()
    missing = [n for n in names if f" T {n}" not in out]
    assert not missing, missing


def test_context_free_calls(built):
    lib = C.CDLL(built.LIB)
    lib.rz_abi_version.restype = C.c_int
    assert lib.rz_abi_version() == 1
    lib.rz_strerror.restype = C.c_char_p
    assert lib.rz_strerror(0) == b"ok"
    assert b"TTNORM" not in lib.rz_strerror(1)


def test_create_without_gpu_reports_error(built):
    """No GPU here: rz_create must fail with a status, not crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = C.CDLL(built.LIB)
    h = C.c_void_p()
    lib.rz_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    assert lib.rz_create(C.byref(h), 0) != 0
    assert not h.value


def test_python_mirror_fails_loudly_without_gpu(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import rajzel_gb300 as R
    with pytest.raises(R.RajzelError):
        R.Context(0)
