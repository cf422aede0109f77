"""The C++ main program (bin/rot2d3c_gpu, the host side of the run over the
C-ABI) against the Python driver, which is checked against the oracle main
loop: every output file byte for byte, for a fresh run and a restart."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from rot2d3c_gb300 import io as fio

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _tree(d):
    out = {}
    for root, _, files in os.walk(d):
        for f in files:
            p = os.path.join(root, f)
            out[os.path.relpath(p, d)] = open(p, "rb").read()
    return out


def _prepare(d, restart):
    os.makedirs(d / "ins")
    os.makedirs(d / "outs")
    lines = open(os.path.join(GOLD, "parameter_small.inp")).read().splitlines()
    if restart:
        lines[1] = "  9                   % 2  step"
        (d / "parameter.inp").write_text("\n".join(lines) + "\n")
        fio.write_status_inp(str(d / "status.inp"), 2, 0.5)
        rng = np.random.default_rng(3)
        g = O.Grid(32)
        fio.write_field(str(d / "ins" / "ps.000.002.out"), O.c2r(g, O.random_phase_field(g, 1, 6, -2.0, rng)) * 1e-3)
        fio.write_field(str(d / "ins" / "vz.000.002.out"), O.c2r(g, O.random_phase_field(g, 1, 6, -1.0, rng)) * 1e-3)
    else:
        shutil.copy(os.path.join(GOLD, "parameter_small.inp"), d / "parameter.inp")
        shutil.copy(os.path.join(GOLD, "status_small.inp"), d / "status.inp")


@pytest.mark.parametrize("restart", [False, True])
def test_app_outputs_equal_the_python_driver(gpu, tmp_path, restart):
    from rot2d3c_gb300 import build as B
    from rot2d3c_gb300.driver import Run
    B.build()
    a, b = tmp_path / "py", tmp_path / "cpp"
    for d in (a, b):
        os.makedirs(d)
        _prepare(d, restart)
    r = Run(32, str(a))
    r.setup()
    r.loop()
    res = subprocess.run([B.APP, "--n", "32", "--dir", str(b)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    ta, tb = _tree(a), _tree(b)
    assert sorted(ta) == sorted(tb)
    assert len([k for k in ta if k.endswith(".out")]) >= 4
    for k in ta:
        assert ta[k] == tb[k], k
