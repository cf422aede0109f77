"""Build recipe of the CUDA library ``librot2d3c_gb300.so`` (sm_103a only)
and of the main-program executable ``bin/rot2d3c_gpu`` linked against it.

The translation units (C-ABI, FP64 engine, FP32 engine, allocation-free
transform, closure CNN) are compiled in parallel with nvcc and linked into
one shared library next to this file; the C++ main program (``app/``) is
compiled with the host C++ compiler.  The build is incremental: nothing is
recompiled when the outputs are newer than every source and header.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librot2d3c_gb300.so")
APP_SRC = os.path.join(HERE, "app", "rot2d3c_gpu.cpp")
APP = os.path.join(HERE, "bin", "rot2d3c_gpu")
SOURCES = [
    "r2d3c_api.cu", "r2d3c_engine_f64.cu", "r2d3c_engine_f32.cu", "r2d3c_noalloc.cu", "r2d3c_cnn.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rot2d3c_gb300")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(APP):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(APP))
    return all(os.path.getmtime(f) <= t for f in _deps() + [APP_SRC])


def build_app() -> str:
    """The main program, linked against the library (found next to bin/)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no host C++ compiler for the main program")
    os.makedirs(os.path.dirname(APP), exist_ok=True)
    tmp = APP + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, APP_SRC, "-o", tmp, "-L", HERE, "-lrot2d3c_gb300",
           "-Wl,-rpath,$ORIGIN/.."]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("main program build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, APP)
    return APP


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library; return its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()
    procs = []
    for src in SOURCES:
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        log = os.path.join(OBJDIR, src.replace(".cu", ".ptxas.log"))
        cmd = [cc, *ARCH, *CFLAGS, "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
        fh = open(log, "w")
        procs.append((subprocess.Popen(cmd, stdout=fh, stderr=subprocess.STDOUT), fh, log, obj))
    objs = []
    failed = []
    for p, fh, log, obj in procs:
        rc = p.wait()
        fh.close()
        if rc != 0:
            failed.append(log)
        objs.append(obj)
    if failed:
        msg = "".join(open(f).read()[-4000:] for f in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    build_app()
    if verbose:
        print("built", LIB, "and", APP, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
