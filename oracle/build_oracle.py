"""Build recipe of the oracle's C restatement (test infrastructure only).

Compiles oracle/cpu/r2d3c_cpu.c with gcc/OpenMP into oracle/_build/libr2d3c_cpu.so.
The reference itself (Fortran + MPI + FFTW 2) cannot be compiled here, so
there is no oracle/_ref build.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu", "r2d3c_cpu.c")
OUT = os.path.join(HERE, "_build", "libr2d3c_cpu.so")


def build(force: bool = False) -> str | None:
    if not os.path.exists(SRC):
        return None
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", SRC, "-o", OUT, "-lm"]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
