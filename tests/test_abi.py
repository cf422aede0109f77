"""The C-ABI library: it loads without a GPU, exports every symbol that
include/r2d3c.h declares, and its host-only paths (randu, argument checks)
behave as documented.  No compute call is made here."""
import ctypes as C
import os
import re

import numpy as np

from oracle import rot2d3c_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "r2d3c.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(r2d3c_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    names = _declared()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name


def test_python_binding_covers_the_header(built_lib):
    from rot2d3c_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == _declared()


def test_randu_through_the_abi_matches_oracle(built_lib):
    import rot2d3c_gb300 as R
    s, so = [1], [1]
    for _ in range(100):
        assert np.float32(R.randu(s)) == np.float32(O.randu(so))
    assert s == so
    s, so = [2147483646], [2147483646]
    for _ in range(10):
        assert np.float32(R.randu(s)) == np.float32(O.randu(so))
    assert s == so


def test_argument_errors_are_status_codes(built_lib):
    import rot2d3c_gb300 as R
    from rot2d3c_gb300 import _lib
    lib = R.load()
    h = C.c_void_p()
    p = R.make_params(n=100)   # not a power of two
    assert lib.r2d3c_create(C.byref(p), 0, C.byref(h)) == _lib.R2D3C_EINVAL
    assert b"power of two" in lib.r2d3c_last_error()
    p = R.make_params(n=64, iflow=7)
    assert lib.r2d3c_create(C.byref(p), 0, C.byref(h)) == _lib.R2D3C_EINVAL
    assert lib.r2d3c_fft_plan_create(48, -1, 0, 0, C.byref(h)) == _lib.R2D3C_EINVAL
    assert lib.r2d3c_fft_plan_create(64, 3, 0, 0, C.byref(h)) == _lib.R2D3C_EINVAL
    assert lib.r2d3c_create(None, 0, C.byref(h)) == _lib.R2D3C_EINVAL
    assert lib.r2d3c_destroy(None) == 0
    assert lib.r2d3c_version().startswith(b"rot2d3c_gb300")
