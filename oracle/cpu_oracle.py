"""ctypes wrapper of the C/OpenMP restatement (oracle/cpu/r2d3c_cpu.c).

TEST INFRASTRUCTURE ONLY: used by tests/ as a second check of the NumPy
oracle and by bench.py as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None
_D = C.POINTER(C.c_double)


def load():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        lib = C.CDLL(path)
        lib.r2d3c_cpu_run.restype = C.c_double
        lib.r2d3c_cpu_run.argtypes = [C.c_int, C.c_int, _D, _D, _D, _D, C.c_int, C.c_int, C.c_double,
                                      C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double,
                                      C.c_int, C.c_int, C.c_double]
        for f in (lib.r2d3c_cpu_r2c, lib.r2d3c_cpu_c2r):
            f.restype = C.c_int
            f.argtypes = [C.c_int, C.c_int, _D, _D]
        lib.r2d3c_cpu_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(_D)


def max_threads() -> int:
    return load().r2d3c_cpu_max_threads()


def run(p, ps, vz, fp, fz, nsteps: int, dt_or_cfl: float, cfl_mode: bool = False, threads: int = 0):
    """nsteps RK4 steps (in place on copies); returns (ps, vz, last dt)."""
    ps = np.ascontiguousarray(ps, np.complex128).copy()
    vz = np.ascontiguousarray(vz, np.complex128).copy()
    fp = np.ascontiguousarray(fp, np.complex128)
    fz = np.ascontiguousarray(fz, np.complex128)
    th = threads or max_threads()
    dt = load().r2d3c_cpu_run(p.n, th, _p(ps), _p(vz), _p(fp), _p(fz), nsteps, int(cfl_mode), dt_or_cfl,
                              p.nu, p.hnu, p.nn, p.mm, p.nuv, p.hnuv, p.nnv, p.mmv, p.omega)
    if dt < 0:
        raise MemoryError("C oracle allocation failed")
    return ps, vz, dt


def r2c(n: int, r, threads: int = 0):
    r = np.ascontiguousarray(r, np.float64)
    out = np.empty((n // 2 + 1, n), np.complex128)
    load().r2d3c_cpu_r2c(n, threads or max_threads(), _p(r), _p(out))
    return out


def c2r(n: int, c, threads: int = 0):
    c = np.ascontiguousarray(c, np.complex128)
    out = np.empty((n, n))
    load().r2d3c_cpu_c2r(n, threads or max_threads(), _p(c), _p(out))
    return out
