"""rot2d3c_gb300: GB300 (sm_103a) implementation of the Rot2D3C time-step hot path.

Python mirror of the reference's routine interface over the C-ABI of
``librot2d3c_gb300.so`` (include/r2d3c.h).  Names and argument meanings follow
the reference's Fortran subroutines:

* ``fftp2d_create_plan`` / ``fftp2d_real_to_complex`` /
  ``fftp2d_complex_to_real`` (src/fftp2D.f90:30-290);
* ``Context`` holds the main program's module state (Rot2D3C.para.f90:102-238)
  and exposes ``derivk2``, ``laplak2``, ``inv_laplak2``, ``poisson``,
  ``energy``, ``inerprod``, ``CFL_condition``, ``cond_check``, ``spectrum``,
  ``transfers``, ``rand_force``, the RK step and the field outputs
  (src/pseudospec2D_Rot2D3C.f90, src/Rot2D3C.para.f90:393-615);
* ``randu`` (src/pseudospec2D_mod.f90:52-71).

Array layouts are the reference's Fortran layouts seen from C:
spectral ``complex128[(n//2+1), n]`` indexed ``[kx][ky]`` and physical
``float64[n, n]`` indexed ``[y][x]``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (C2R, DT_CFL, DT_FIXED, FIELD_INVLAP_PSI, FIELD_PS, FIELD_VZ, FIELD_WW, FP32,
                   FP64, R2C, Params, R2D3CError, check, load)

__all__ = [
    "FP64", "FP32", "R2C", "C2R", "DT_CFL", "DT_FIXED", "FIELD_PS", "FIELD_VZ", "FIELD_WW",
    "FIELD_INVLAP_PSI", "Params", "R2D3CError", "FFTPlan", "Context", "randu", "load",
    "fftp2d_create_plan", "fftp2d_real_to_complex", "fftp2d_complex_to_real",
    "fftp2d_destroy_plan", "make_params", "Ensemble",
]

_DP = C.POINTER(C.c_double)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _spec_in(a, n):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.shape != (n // 2 + 1, n):
        raise ValueError(f"spectral array must have shape {(n // 2 + 1, n)}, got {a.shape}")
    return a


def _phys_in(a, n):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (n, n):
        raise ValueError(f"physical array must have shape {(n, n)}, got {a.shape}")
    return a


def randu(seed: list) -> float:
    """randu (pseudospec2D_mod.f90:52-71) through the C-ABI; ``seed`` is a
    one-element list updated in place like the Fortran INTEGER argument."""
    s = C.c_int(int(seed[0]))
    r = load().r2d3c_randu(C.byref(s))
    seed[0] = s.value
    return float(np.float32(r))


def regrid_physical(old: np.ndarray, m: int) -> np.ndarray:
    """The reference's slice regridder (regrid_slices.f90:95-104) on a whole
    n x n field (row-major [y][x]) onto m x m, n < m <= 2n."""
    old = np.ascontiguousarray(old, np.float64)
    n = old.shape[0]
    assert old.shape == (n, n)
    out = np.empty((m, m))
    check(load().r2d3c_regrid_physical(n, m, _dptr(old), _dptr(out)), "regrid_physical")
    return out


def regrid_spectral(src: "Context", dst: "Context") -> None:
    """dst's state = src's state zero-padded onto dst's finer grid."""
    check(load().r2d3c_regrid_spectral(src._h, dst._h), "regrid_spectral")


def fp64_fma_peak() -> float:
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    t = C.c_double()
    check(load().r2d3c_fp64_fma_peak(C.byref(t)), "fp64_fma_peak")
    return t.value


def make_params(**kw) -> Params:
    """r2d3c_params with the reference's parameter.inp defaults overridden by kw."""
    d = dict(n=64, cfl=0.5, step=1, cstep=100, sstep=1000, tstep=10000, fp0=1.0, fz0=1.0,
             u0=0.01, v0=0.01, kdn=12.0, kup=12.0, nu=0.001, hnu=1.0, nn=1, mm=2, nuv=0.001,
             hnuv=1.0, nnv=1, mmv=2, omega=0.0, seed=1, iflow=3, prm1=1.0, prm2=1.0, dt_corr=0.0)
    d.update(kw)
    p = Params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


class FFTPlan:
    """fftp2d plan (fftp2D.f90:30-63).  ``dir`` = R2C (-1) or C2R (+1)."""

    def __init__(self, n: int, dir: int, precision: int = FP64, flags: int = 0):
        self.n, self.dir, self.precision = n, dir, precision
        h = C.c_void_p()
        check(load().r2d3c_fft_plan_create(n, dir, flags, precision, C.byref(h)), "fft_plan_create")
        self._h = h

    def r2c(self, r: np.ndarray) -> np.ndarray:
        """fftp2d_real_to_complex (fftp2D.f90:133-211)."""
        r = _phys_in(r, self.n)
        out = np.empty((self.n // 2 + 1, self.n), dtype=np.complex128)
        check(load().r2d3c_fft_r2c(self._h, _dptr(r), _dptr(out)), "fft_r2c")
        return out

    def c2r(self, c: np.ndarray) -> np.ndarray:
        """fftp2d_complex_to_real (fftp2D.f90:214-290)."""
        c = _spec_in(c, self.n)
        out = np.empty((self.n, self.n), dtype=np.float64)
        check(load().r2d3c_fft_c2r(self._h, _dptr(c), _dptr(out)), "fft_c2r")
        return out

    def r2c_dev(self, d_in: int, d_out: int, stream: int = 0) -> None:
        check(load().r2d3c_fft_r2c_dev(self._h, C.c_void_p(d_in), C.c_void_p(d_out),
                                       C.c_void_p(stream or None)), "fft_r2c_dev")

    def c2r_dev(self, d_in: int, d_out: int, stream: int = 0) -> None:
        check(load().r2d3c_fft_c2r_dev(self._h, C.c_void_p(d_in), C.c_void_p(d_out),
                                       C.c_void_p(stream or None)), "fft_c2r_dev")

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            load().r2d3c_fft_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def fftp2d_create_plan(n: int, fftdir: int, flags: int = 0, precision: int = FP64) -> FFTPlan:
    return FFTPlan(n, fftdir, precision, flags)


def fftp2d_destroy_plan(plan: FFTPlan) -> None:
    plan.destroy()


def fftp2d_real_to_complex(plan: FFTPlan, r: np.ndarray) -> np.ndarray:
    return plan.r2c(r)


def fftp2d_complex_to_real(plan: FFTPlan, c: np.ndarray) -> np.ndarray:
    return plan.c2r(c)


class Context:
    """One Rot2D3C run on the current CUDA device (the module state of the
    reference main program, Rot2D3C.para.f90:102-238)."""

    def __init__(self, params: Params, precision: int = FP64):
        self.params = params
        self.n = params.n
        self.precision = precision
        h = C.c_void_p()
        check(load().r2d3c_create(C.byref(params), precision, C.byref(h)), "create")
        self._h = h

    # ---------------------------------------------------------------- state
    def _spec_pair_out(self):
        sh = (self.n // 2 + 1, self.n)
        return np.empty(sh, np.complex128), np.empty(sh, np.complex128)

    def set_state(self, ps: np.ndarray, vz: np.ndarray) -> None:
        a, b = _spec_in(ps, self.n), _spec_in(vz, self.n)
        check(load().r2d3c_set_state(self._h, _dptr(a), _dptr(b)), "set_state")

    def get_state(self):
        a, b = self._spec_pair_out()
        check(load().r2d3c_get_state(self._h, _dptr(a), _dptr(b)), "get_state")
        return a, b

    def set_state_physical(self, ps: np.ndarray, vz: np.ndarray) -> None:
        a, b = _phys_in(ps, self.n), _phys_in(vz, self.n)
        check(load().r2d3c_set_state_physical(self._h, _dptr(a), _dptr(b)), "set_state_physical")

    def set_forcing(self, fp: np.ndarray, fz: np.ndarray) -> None:
        a, b = _spec_in(fp, self.n), _spec_in(fz, self.n)
        check(load().r2d3c_set_forcing(self._h, _dptr(a), _dptr(b)), "set_forcing")

    def get_forcing(self):
        a, b = self._spec_pair_out()
        check(load().r2d3c_get_forcing(self._h, _dptr(a), _dptr(b)), "get_forcing")
        return a, b

    def initial_conditions(self, seed: list) -> None:
        s = C.c_int(int(seed[0]))
        check(load().r2d3c_initial_conditions(self._h, C.byref(s)), "initial_conditions")
        seed[0] = s.value

    def forcing_init(self, seed: list, seed1: list) -> None:
        s, s1 = C.c_int(int(seed[0])), C.c_int(int(seed1[0]))
        check(load().r2d3c_forcing_init(self._h, C.byref(s), C.byref(s1)), "forcing_init")
        seed[0], seed1[0] = s.value, s1.value

    # ------------------------------------------------------------ hot path
    def CFL_condition(self, cfl: float) -> float:
        dt = C.c_double()
        check(load().r2d3c_cfl(self._h, cfl, C.byref(dt)), "cfl")
        return dt.value

    def rand_force(self, dt: float, seed: list, seed1: list) -> None:
        s, s1 = C.c_int(int(seed[0])), C.c_int(int(seed1[0]))
        check(load().r2d3c_force_random(self._h, dt, C.byref(s), C.byref(s1)), "force_random")
        seed[0], seed1[0] = s.value, s1.value

    def step(self, dt: float, seed: list | None = None, seed1: list | None = None) -> None:
        s = C.c_int(int(seed[0]) if seed else 0)
        s1 = C.c_int(int(seed1[0]) if seed1 else 0)
        check(load().r2d3c_step(self._h, dt, C.byref(s), C.byref(s1)), "step")
        if seed is not None:
            seed[0] = s.value
        if seed1 is not None:
            seed1[0] = s1.value

    def advance(self, nsteps: int, dt_mode: int, cfl_or_dt: float,
                seed: list | None = None, seed1: list | None = None):
        """Returns (time, dt of the last step)."""
        t, dtl = C.c_double(), C.c_double()
        s = C.c_int(int(seed[0]) if seed else 0)
        s1 = C.c_int(int(seed1[0]) if seed1 else 0)
        check(load().r2d3c_advance(self._h, nsteps, dt_mode, cfl_or_dt, C.byref(t), C.byref(dtl),
                                   C.byref(s), C.byref(s1)), "advance")
        if seed is not None:
            seed[0] = s.value
        if seed1 is not None:
            seed1[0] = s1.value
        return t.value, dtl.value

    def set_time(self, t: float) -> None:
        check(load().r2d3c_set_time(self._h, t), "set_time")

    # ---------------------------------------------------------- diagnostics
    def cond_check(self, time: float) -> np.ndarray:
        out = np.empty(30)
        check(load().r2d3c_cond_check(self._h, time, _dptr(out)), "cond_check")
        return out

    def spectrum(self):
        nb = self.n // 2 + 1
        ek, ezk = np.empty(nb), np.empty(nb)
        check(load().r2d3c_spectrum(self._h, _dptr(ek), _dptr(ezk)), "spectrum")
        return ek, ezk

    def transfers(self):
        nb = self.n // 2 + 1
        f0, f1, f2 = np.empty(nb), np.empty(nb), np.empty(nb)
        check(load().r2d3c_transfers(self._h, _dptr(f0), _dptr(f1), _dptr(f2)), "transfers")
        return f0, f1, f2

    def get_field(self, which: int) -> np.ndarray:
        out = np.empty((self.n, self.n))
        check(load().r2d3c_get_field(self._h, which, _dptr(out)), "get_field")
        return out

    # ------------------------------------------------------------ operators
    def derivk2(self, a: np.ndarray, dir: int) -> np.ndarray:
        a = _spec_in(a, self.n)
        b = np.empty_like(a)
        check(load().r2d3c_derivk2(self._h, _dptr(a), _dptr(b), dir), "derivk2")
        return b

    def laplak2(self, a: np.ndarray) -> np.ndarray:
        a = _spec_in(a, self.n)
        b = np.empty_like(a)
        check(load().r2d3c_laplak2(self._h, _dptr(a), _dptr(b)), "laplak2")
        return b

    def inv_laplak2(self, a: np.ndarray) -> np.ndarray:
        a = _spec_in(a, self.n)
        b = np.empty_like(a)
        check(load().r2d3c_inv_laplak2(self._h, _dptr(a), _dptr(b)), "inv_laplak2")
        return b

    def poisson(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a, b = _spec_in(a, self.n), _spec_in(b, self.n)
        c = np.empty_like(a)
        check(load().r2d3c_poisson(self._h, _dptr(a), _dptr(b), _dptr(c)), "poisson")
        return c

    def energy(self, a: np.ndarray, kin: int) -> float:
        a = _spec_in(a, self.n)
        r = C.c_double()
        check(load().r2d3c_energy(self._h, _dptr(a), kin, C.byref(r)), "energy")
        return r.value

    def inerprod(self, a: np.ndarray, b: np.ndarray, kin: int) -> float:
        a, b = _spec_in(a, self.n), _spec_in(b, self.n)
        r = C.c_double()
        check(load().r2d3c_inerprod(self._h, _dptr(a), _dptr(b), kin, C.byref(r)), "inerprod")
        return r.value

    # ---------------------------------------------------------------- misc
    def profile_passes(self, nsteps: int, dt: float):
        """(ms per launch [A, B, C, other], launches [A, B, C, other])."""
        ms = (C.c_double * 4)()
        cnt = (C.c_longlong * 4)()
        check(load().r2d3c_profile_passes(self._h, nsteps, dt, ms, cnt), "profile_passes")
        return list(ms), list(cnt)

    def kernel_launches(self) -> int:
        c = C.c_longlong()
        check(load().r2d3c_kernel_launches(self._h, C.byref(c)), "kernel_launches")
        return c.value

    def plan_report(self) -> dict:
        """The launch-schedule autotuner's timings and choice (r2d3c_plan_report)."""
        import json
        buf = C.create_string_buffer(16384)
        check(load().r2d3c_plan_report(self._h, buf, len(buf)), "plan_report")
        return json.loads(buf.value.decode())

    def device_bytes(self) -> int:
        c = C.c_longlong()
        check(load().r2d3c_device_bytes(self._h, C.byref(c)), "device_bytes")
        return c.value

    def dev_ptr(self, which: int) -> int:
        p = C.c_void_p()
        check(load().r2d3c_dev_ptr(self._h, which, C.byref(p)), "dev_ptr")
        return p.value or 0

    def stream(self) -> int:
        p = C.c_void_p()
        check(load().r2d3c_stream(self._h, C.byref(p)), "stream")
        return p.value or 0

    def synchronize(self) -> None:
        check(load().r2d3c_synchronize(self._h), "synchronize")

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            load().r2d3c_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Ensemble:
    """Independent runs advanced together (r2d3c_ensemble_*): runs of equal n
    share kernel launches, and one CUDA graph holds one step of every size
    group.  ``groups`` is a list of (n, [Params, ...]); runs are numbered
    group by group."""

    def __init__(self, groups, precision: int = FP64):
        ns = [int(n) for n, _ in groups]
        runs = [len(ps) for _, ps in groups]
        allp = [p for _, ps in groups for p in ps]
        self.ns = [n for n, ps in groups for _ in ps]
        arr = (Params * len(allp))(*allp)
        h = C.c_void_p()
        check(load().r2d3c_ensemble_create(len(groups), (C.c_int * len(ns))(*ns), (C.c_int * len(runs))(*runs),
                                           arr, precision, C.byref(h)), "ensemble_create")
        self._h = h
        self.nruns = len(allp)

    def set_state(self, run: int, ps, vz) -> None:
        n = self.ns[run]
        a, b = _spec_in(ps, n), _spec_in(vz, n)
        check(load().r2d3c_ensemble_set_state(self._h, run, _dptr(a), _dptr(b)), "ensemble_set_state")

    def get_state(self, run: int):
        n = self.ns[run]
        a = np.empty((n // 2 + 1, n), np.complex128)
        b = np.empty_like(a)
        check(load().r2d3c_ensemble_get_state(self._h, run, _dptr(a), _dptr(b)), "ensemble_get_state")
        return a, b

    def set_forcing(self, run: int, fp, fz) -> None:
        n = self.ns[run]
        a, b = _spec_in(fp, n), _spec_in(fz, n)
        check(load().r2d3c_ensemble_set_forcing(self._h, run, _dptr(a), _dptr(b)), "ensemble_set_forcing")

    def set_time(self, run: int, t: float) -> None:
        check(load().r2d3c_ensemble_set_time(self._h, run, t), "ensemble_set_time")

    def advance(self, nsteps: int, dt_mode: int, cfl_or_dt: float) -> np.ndarray:
        t = np.empty(self.nruns)
        check(load().r2d3c_ensemble_advance(self._h, nsteps, dt_mode, cfl_or_dt, _dptr(t)), "ensemble_advance")
        return t

    def cond_check(self, run: int, time: float) -> np.ndarray:
        out = np.empty(30)
        check(load().r2d3c_ensemble_cond_check(self._h, run, time, _dptr(out)), "ensemble_cond_check")
        return out

    def spectrum(self, run: int):
        nb = self.ns[run] // 2 + 1
        ek, ezk = np.empty(nb), np.empty(nb)
        check(load().r2d3c_ensemble_spectrum(self._h, run, _dptr(ek), _dptr(ezk)), "ensemble_spectrum")
        return ek, ezk

    def kernel_launches(self) -> int:
        c = C.c_longlong()
        check(load().r2d3c_ensemble_kernel_launches(self._h, C.byref(c)), "ensemble_kernel_launches")
        return c.value

    def plan_report(self) -> list:
        """The plan autotuner's timings and choices of every size group."""
        import json
        buf = C.create_string_buffer(65536)
        check(load().r2d3c_ensemble_plan_report(self._h, buf, len(buf)), "ensemble_plan_report")
        return json.loads(buf.value.decode())

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            load().r2d3c_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
