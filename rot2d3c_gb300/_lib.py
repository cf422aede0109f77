"""ctypes binding of ``librot2d3c_gb300.so`` (declarations of include/r2d3c.h).

The library is the product: every compute call below goes to its CUDA
kernels.  There is no CPU fallback -- if the library is missing the import
of a compute entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librot2d3c_gb300.so")

R2D3C_OK = 0
R2D3C_EINVAL = -1
R2D3C_ECUDA = -2
R2D3C_ENOMEM = -3
R2D3C_ETIMEOUT = -4
R2D3C_EIO = -5
R2D3C_ESTATE = -6
FP64 = 0
FP32 = 1
R2C = -1
C2R = 1
DT_CFL = 0
DT_FIXED = 1
FIELD_PS, FIELD_VZ, FIELD_WW, FIELD_INVLAP_PSI = 0, 1, 2, 3

_STATUS_NAMES = {
    R2D3C_EINVAL: "EINVAL", R2D3C_ECUDA: "ECUDA", R2D3C_ENOMEM: "ENOMEM",
    R2D3C_ETIMEOUT: "ETIMEOUT", R2D3C_EIO: "EIO", R2D3C_ESTATE: "ESTATE",
}


class R2D3CError(RuntimeError):
    """A non-zero status returned by the C-ABI."""

    def __init__(self, code: int, where: str, text: str):
        super().__init__(f"{where}: {_STATUS_NAMES.get(code, code)} ({code}): {text}")
        self.code = code


class Params(C.Structure):
    """r2d3c_params: the 25 values of parameter.inp plus n."""
    _fields_ = [
        ("n", C.c_int), ("cfl", C.c_double), ("step", C.c_int), ("cstep", C.c_int),
        ("sstep", C.c_int), ("tstep", C.c_int), ("fp0", C.c_double), ("fz0", C.c_double),
        ("u0", C.c_double), ("v0", C.c_double), ("kdn", C.c_double), ("kup", C.c_double),
        ("nu", C.c_double), ("hnu", C.c_double), ("nn", C.c_int), ("mm", C.c_int),
        ("nuv", C.c_double), ("hnuv", C.c_double), ("nnv", C.c_int), ("mmv", C.c_int),
        ("omega", C.c_double), ("seed", C.c_int), ("iflow", C.c_int), ("prm1", C.c_double),
        ("prm2", C.c_double), ("dt_corr", C.c_double),
    ]


_lib = None

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)

# name -> (restype, argtypes); the list is checked against include/r2d3c.h by the tests
SIGNATURES = {
    "r2d3c_version": (C.c_char_p, []),
    "r2d3c_last_error": (C.c_char_p, []),
    "r2d3c_kernel_launches": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "r2d3c_fft_plan_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_P)]),
    "r2d3c_fft_plan_destroy": (C.c_int, [_P]),
    "r2d3c_fft_r2c": (C.c_int, [_P, _D, _D]),
    "r2d3c_fft_c2r": (C.c_int, [_P, _D, _D]),
    "r2d3c_fft_r2c_dev": (C.c_int, [_P, _P, _P, _P]),
    "r2d3c_fft_c2r_dev": (C.c_int, [_P, _P, _P, _P]),
    "r2d3c_fft_c2r_noalloc": (C.c_int, [C.c_int, _P, _P, _P]),
    "r2d3c_create": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(_P)]),
    "r2d3c_destroy": (C.c_int, [_P]),
    "r2d3c_device_bytes": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "r2d3c_set_state": (C.c_int, [_P, _D, _D]),
    "r2d3c_get_state": (C.c_int, [_P, _D, _D]),
    "r2d3c_set_state_physical": (C.c_int, [_P, _D, _D]),
    "r2d3c_set_forcing": (C.c_int, [_P, _D, _D]),
    "r2d3c_get_forcing": (C.c_int, [_P, _D, _D]),
    "r2d3c_initial_conditions": (C.c_int, [_P, _I]),
    "r2d3c_forcing_init": (C.c_int, [_P, _I, _I]),
    "r2d3c_cfl": (C.c_int, [_P, C.c_double, _D]),
    "r2d3c_force_random": (C.c_int, [_P, C.c_double, _I, _I]),
    "r2d3c_step": (C.c_int, [_P, C.c_double, _I, _I]),
    "r2d3c_advance": (C.c_int, [_P, C.c_int, C.c_int, C.c_double, _D, _D, _I, _I]),
    "r2d3c_set_time": (C.c_int, [_P, C.c_double]),
    "r2d3c_cond_check": (C.c_int, [_P, C.c_double, _D]),
    "r2d3c_spectrum": (C.c_int, [_P, _D, _D]),
    "r2d3c_transfers": (C.c_int, [_P, _D, _D, _D]),
    "r2d3c_get_field": (C.c_int, [_P, C.c_int, _D]),
    "r2d3c_ensemble_create": (C.c_int, [C.c_int, _I, _I, C.POINTER(Params), C.c_int, C.POINTER(_P)]),
    "r2d3c_ensemble_destroy": (C.c_int, [_P]),
    "r2d3c_ensemble_set_state": (C.c_int, [_P, C.c_int, _D, _D]),
    "r2d3c_ensemble_get_state": (C.c_int, [_P, C.c_int, _D, _D]),
    "r2d3c_ensemble_set_forcing": (C.c_int, [_P, C.c_int, _D, _D]),
    "r2d3c_ensemble_advance": (C.c_int, [_P, C.c_int, C.c_int, C.c_double, _D]),
    "r2d3c_ensemble_set_time": (C.c_int, [_P, C.c_int, C.c_double]),
    "r2d3c_ensemble_cond_check": (C.c_int, [_P, C.c_int, C.c_double, _D]),
    "r2d3c_ensemble_spectrum": (C.c_int, [_P, C.c_int, _D, _D]),
    "r2d3c_ensemble_kernel_launches": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "r2d3c_ensemble_plan_report": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "r2d3c_cnn_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_P)]),
    "r2d3c_cnn_destroy": (C.c_int, [_P]),
    "r2d3c_cnn_num_params": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "r2d3c_cnn_get_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "r2d3c_cnn_set_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "r2d3c_cnn_forward": (C.c_int, [_P, _P, C.c_int, _P]),
    "r2d3c_cnn_gradients": (C.c_int, [_P, _P, _P, C.c_int, C.POINTER(C.c_float), _D]),
    "r2d3c_cnn_train_step": (C.c_int, [_P, _P, _P, C.c_int, C.c_float, _D]),
    "r2d3c_cnn_backward": (C.c_int, [_P, _P, _P, C.c_int, _P, C.POINTER(C.c_float)]),
    "r2d3c_cnn_set_normalization": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                              C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "r2d3c_closure_inputs": (C.c_int, [_P, _P]),
    "r2d3c_closure_sample": (C.c_int, [_P, _P, _P, _P]),
    "r2d3c_closure_set_tendency": (C.c_int, [_P, _P]),
    "r2d3c_closure_set_band": (C.c_int, [_P, _P, C.c_int]),
    "r2d3c_closure_advance": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_double, _D, _D]),
    "r2d3c_closure_advance_every": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_double, _D, _D]),
    "r2d3c_closure_advance_overlapped": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_double, _D, _D]),
    "r2d3c_regrid_physical": (C.c_int, [C.c_int, C.c_int, _D, _D]),
    "r2d3c_regrid_physical_dev": (C.c_int, [C.c_int, C.c_int, _P, _P, _P]),
    "r2d3c_regrid_spectral": (C.c_int, [_P, _P]),
    "r2d3c_plan_report": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "r2d3c_derivk2": (C.c_int, [_P, _D, _D, C.c_int]),
    "r2d3c_laplak2": (C.c_int, [_P, _D, _D]),
    "r2d3c_inv_laplak2": (C.c_int, [_P, _D, _D]),
    "r2d3c_poisson": (C.c_int, [_P, _D, _D, _D]),
    "r2d3c_energy": (C.c_int, [_P, _D, C.c_int, _D]),
    "r2d3c_inerprod": (C.c_int, [_P, _D, _D, C.c_int, _D]),
    "r2d3c_randu": (C.c_float, [_I]),
    "r2d3c_profile_passes": (C.c_int, [_P, C.c_int, C.c_double, _D, C.POINTER(C.c_longlong)]),
    "r2d3c_fp64_fma_peak": (C.c_int, [_D]),
    "r2d3c_dev_ptr": (C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    "r2d3c_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "r2d3c_synchronize": (C.c_int, [_P]),
}


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, where: str) -> None:
    if code != R2D3C_OK:
        txt = load().r2d3c_last_error()
        raise R2D3CError(code, where, txt.decode() if txt else "")
