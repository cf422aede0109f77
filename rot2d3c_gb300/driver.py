"""Main program of a run on one GPU: the control flow of PROGRAM Rot2D3C
(src/Rot2D3C.para.f90:2-639) over the C-ABI.

It reads ``parameter.inp`` and ``status.inp`` from the working directory,
builds the initial condition (stat == 0, :245-299) or reads the binary fields
of output ``stat`` from ``idir`` (:300-338), sets up the forcing (:343-381),
and runs the main loop (:393-615) with the reference's output cadence:
cond_check every ``cstep`` steps, spectrum/transfers every ``sstep`` steps,
binary fields every ``tstep`` steps, with the reference's file names and
formats (rot2d3c_gb300.io).  Between output steps whole stretches of steps
go to ``r2d3c_advance`` (CFL time step, rand_force and the RK step, replayed
from one CUDA graph), which is equivalent to the reference's per-step order
because the diagnostics neither read dt nor touch the random seeds.

    python -m rot2d3c_gb300.driver --n 256 [--dir RUNDIR] [--fp32] [--max-steps K]

The grid size is a run-time value here (module grid, pseudospec2D_mod.f90:7-14,
fixes it at compile time in the reference).
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import FP32, FP64, Context, make_params
from . import io as fio


def _digits3(v: int):
    """Character counters c//d//u of a 3-digit output index (:91-97, :315-320)."""
    f = np.float32(v)
    ic = 48 + int(f / np.float32(100))
    id_ = 48 + int(f / np.float32(10)) - int(f / np.float32(100)) * 10
    iu = 48 + int(v) - int(f / np.float32(10)) * 10
    return ic, id_, iu


class Run:
    """State of one run: counters, seeds and the device context."""

    def __init__(self, n: int, workdir: str = ".", precision: int = FP64):
        self.n = n
        self.dir = workdir
        self.stat, self.time = fio.read_status_inp(os.path.join(workdir, "status.inp"))
        prm = fio.read_parameter_inp(os.path.join(workdir, "parameter.inp"))
        self.idir = os.path.join(workdir, prm.pop("idir"))
        self.odir = os.path.join(workdir, prm.pop("odir"))
        self.prm = prm
        self.ctx = Context(make_params(n=n, **prm), precision)
        self.seed = [prm["seed"]]
        self.seed1 = [0]
        self.node = "000"  # one rank (:91-97)

    def _read_field(self, name: str, ext: str):
        return fio.read_field(os.path.join(self.idir, f"{name}.{self.node}.{ext}.out"), self.n)

    def setup(self):
        p = self.prm
        self.ic = self.id = self.iu = 48
        self.jt = self.jc = self.jd = self.ju = 48
        if self.stat == 0:  # :245-299
            self.ini = 1
            self.timet, self.timec, self.times = p["tstep"], p["cstep"], p["sstep"]
            self.ctx.initial_conditions(self.seed)
        else:  # :300-338
            self.ini = int((self.stat - 1) * p["tstep"])
            dump = float(self.ini) / float(p["sstep"]) + 1
            self.timet = self.timec = self.times = 0
            self.jt = 48 + int(dump / 1000)
            self.jc = 48 + int(dump / 100) - int(dump / 1000) * 10
            self.jd = 48 + int(dump / 10) - int(dump / 100) * 10
            self.ju = 48 + int(dump) - int(dump / 10) * 10
            self.ic, self.id, self.iu = _digits3(self.stat)
            ext = chr(self.ic) + chr(self.id) + chr(self.iu)
            self.ctx.set_state_physical(self._read_field("ps", ext), self._read_field("vz", ext))
        self.ctx.forcing_init(self.seed, self.seed1)  # :343-381
        self.ctx.set_time(self.time)

    # ------------------------------------------------------------ outputs
    def _cond_check(self):
        fio.append_cond_check(self.dir, self.ctx.cond_check(self.time))

    def _spectra(self):  # :428-457
        self.ju += 1
        if self.ju == 58:
            self.ju = 48
            self.jd += 1
        if self.jd == 58:
            self.jd = 48
            self.jc += 1
        if self.jc == 58:
            self.jc = 48
            self.jt += 1
        ext4 = chr(self.jt) + chr(self.jc) + chr(self.jd) + chr(self.ju)
        ek, ezk = self.ctx.spectrum()
        fio.write_spectrum(self.odir, ext4, ek, ezk)
        fl = self.ctx.transfers()
        fio.write_transfers(self.odir, ext4, *fl)
        fio.append_time_line(os.path.join(self.dir, "time_spec.txt"), ext4, self.time)

    def _fields(self):  # :461-530
        self.iu += 1
        if self.iu == 58:
            self.iu = 48
            self.id += 1
        if self.id == 58:
            self.id = 48
            self.ic += 1
        ext = chr(self.ic) + chr(self.id) + chr(self.iu)
        for which, name in ((0, "ps"), (1, "vz"), (2, "ww"), (3, "invlap_psi")):
            fio.write_field(os.path.join(self.odir, f"{name}.{self.node}.{ext}.out"),
                            self.ctx.get_field(which))
        fio.append_time_line(os.path.join(self.dir, "time_field.txt"), ext, self.time)

    # ------------------------------------------------------------ loop
    def loop(self, max_steps: int | None = None):
        p = self.prm
        last = p["step"] if max_steps is None else min(p["step"], self.ini + max_steps - 1)
        t = self.ini
        while t <= last:
            due = (self.timec == p["cstep"], self.times == p["sstep"], self.timet == p["tstep"])
            if any(due):
                if due[0]:
                    self.timec = 0
                    self._cond_check()
                if due[1]:
                    self.times = 0
                    self._spectra()
                if due[2]:
                    self.timet = 0
                    self._fields()
                k = 1
            else:
                # steps until the next output (counters only grow between them)
                gaps = [c - x for c, x in ((p["cstep"], self.timec), (p["sstep"], self.times),
                                           (p["tstep"], self.timet)) if c - x > 0]
                k = max(1, min(gaps + [last - t + 1]))
            self.time, _ = self.ctx.advance(k, 0, p["cfl"], self.seed, self.seed1)
            self.timet += k
            self.times += k
            self.timec += k
            t += k
        return self.time


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, required=True)
    ap.add_argument("--dir", default=".")
    ap.add_argument("--fp32", action="store_true")
    ap.add_argument("--max-steps", type=int, default=None)
    a = ap.parse_args(argv)
    r = Run(a.n, a.dir, FP32 if a.fp32 else FP64)
    r.setup()
    t = r.loop(a.max_steps)
    print(f"done: time = {t!r}")


if __name__ == "__main__":
    main()
