"""The C ABI library: builds, loads without a GPU, exports every symbol the
public header declares, and reports errors through status codes.  No compute
call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include"))) if h.endswith(".h")]


def declared_functions(path):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    # only the extern "C" C-ABI headers (estl_*.h) declare exported symbols
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(estl_[a-z0-9_]+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from estl_gb300 import build
    build.build()
    from estl_gb300 import _lib
    return _lib.lib()


def c_abi_headers():
    return [h for h in HEADERS if os.path.basename(h).startswith("estl_")]


def test_header_exports(lib):
    names = []
    for h in c_abi_headers():
        names += declared_functions(h)
    assert "estl_execute" in names and "estl_plan_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared in include/ but not exported: {missing}"


def test_binding_covers_header():
    from estl_gb300 import _lib
    names = []
    for h in c_abi_headers():
        names += declared_functions(h)
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_status_strings(lib):
    lib.estl_status_string.restype = ctypes.c_char_p
    assert lib.estl_status_string(0) == b"ESTL_OK"
    assert lib.estl_status_string(2) == b"ESTL_UNSUPPORTED_SIZE"


def test_calls_before_init_fail_cleanly(lib):
    from estl_gb300 import _lib
    L = _lib.lib()
    h = ctypes.c_void_p()
    st = L.estl_plan_create(4096, 1, -1, 0, ctypes.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert st == 7  # ESTL_NOT_INITIALIZED
        assert b"estl_init" in L.estl_last_error()
        st = L.estl_init(0, 0)
        assert st != 0 and L.estl_last_error()
    assert L.estl_max_batch(4096) >= 0


def test_product_does_not_use_the_oracle():
    """The shipped package never imports, links or loads the CPU oracle."""
    pkg = os.path.join(ROOT, "estl_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h", ".inc")):
                text = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"\bimport oracle\b|from oracle\b|liboracle|oracle/", text), f


def test_host_buffers_are_checked_before_the_call():
    """Host arrays go to the library as raw pointers, so the binding refuses a
    wrong dtype, a short, non-contiguous or read-only array first."""
    import numpy as np
    from estl_gb300 import EstlError, _check_host
    ok = np.zeros(16, np.complex64)
    _check_host(ok, "complex64", 16, "input")
    _check_host(ok, "complex64", 8, "output", writable=True)
    ro = ok.copy()
    ro.flags.writeable = False
    for bad, numel, writable in ((ok, 17, False), (ok.astype(np.complex128), 16, False), (ok[::2], 8, False),
                                 (ro, 16, True), (list(ok), 16, False)):
        with pytest.raises(EstlError):
            _check_host(bad, "complex64", numel, "buffer", writable=writable)
    _check_host(ro, "complex64", 16, "input")  # read-only is fine for an input
