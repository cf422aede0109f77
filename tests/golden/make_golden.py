"""Generate the golden fixtures of the test-suite from the oracle.

The reference ships no golden vectors and cannot be built here (no Fortran
compiler, MPI or FFTW 2), so these fixtures pin the oracle restatement (and,
through the GPU tests, the CUDA path) to fixed, reviewed numbers: a regression
anchor, not a reference-run output.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import rot2d3c_oracle as O  # noqa: E402


def main():
    out = {}
    # randu stream from seed 1 (pseudospec2D_mod.f90:52-71)
    s = [1]
    out["randu_seed1"] = np.array([O.randu(s) for _ in range(8)], dtype=np.float32)
    out["randu_seed1_final"] = np.array([s[0]])

    # seeded end-to-end run at n = 32: fixed dt, synthetic forcing
    n = 32
    p = O.Params(n=n, omega=1.0, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, nn=1, mm=2, iflow=0)
    g = O.Grid(n)
    rng = np.random.default_rng(2024)
    ps = O.random_phase_field(g, 1.0, 10.0, -2.0, rng) * 20.0
    vz = O.random_phase_field(g, 1.0, 10.0, -1.0, rng) * 20.0
    fp = O.random_phase_field(g, 4.0, 6.0, 0.0, rng)
    fz = O.random_phase_field(g, 4.0, 6.0, 0.0, rng)
    out.update(ps0=ps, vz0=vz, fp=fp, fz=fz)
    dt = 1e-3
    a, b = ps, vz
    for k in range(10):
        a, b, _, _ = O.rk_step(g, p, a, b, fp, fz, dt)
        if k == 0:
            out.update(ps1=a, vz1=b)
    out.update(ps10=a, vz10=b)
    out["cond_check10"] = O.cond_check(g, p, a, b, fp, fz, 10 * dt)
    ek, ezk = O.spectrum(g, a, b)
    f0, f1, f2 = O.transfers(g, a, b)
    out.update(ek10=ek, ezk10=ezk, fl0_10=f0, fl1_10=f1, fl2_10=f2)
    out["params"] = np.array([n, p.omega, p.nu, p.hnu, p.nuv, p.hnuv, p.nn, p.mm, p.nnv, p.mmv, dt])

    # seeded initial condition (stat == 0 branch), n = 32, kup = 3
    pi = O.Params(n=n, kup=3.0, u0=0.3, v0=0.2)
    s = [5]
    ips, ivz = O.initial_conditions(g, pi, s)
    out.update(ic_ps=ips, ic_vz=ivz, ic_seed_final=np.array([s[0]]))
    np.savez_compressed(os.path.join(HERE, "golden_n32.npz"), **out)
    print("wrote", os.path.join(HERE, "golden_n32.npz"))


if __name__ == "__main__":
    main()
