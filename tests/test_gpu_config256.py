"""The 256^2 FP64 configuration of the reference workload (seeded shell 1-10
IC with |u| ~ k^-1, time-constant random-phase forcing in shell 4-6,
Omega = 1, nu = 1e-3, hypoviscosity 0.1 with mm = 2, dt = 1e-3): the GPU
state after 1, 10 and 100 steps against the oracle, FP64 and FP32, and the
spectrum after 1000 FP64 steps."""
import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import params, random_forcing, random_state, rel_l2

pytestmark = pytest.mark.gpu

N, DT = 256, 1e-3


def _setup(prec):
    import rot2d3c_gb300 as gpu
    p, cp = params(N, omega=1.0, nu=1e-3, nuv=1e-3, hnu=0.1, hnuv=0.1, nn=1, mm=2, nnv=1, mmv=2, iflow=0)
    g, ps, vz = random_state(N, 1, kmin=1.0, kmax_shell=10.0, slope=-1.0)
    # energy(ps, 1) = energy(vz, 0) = 0.5 (u0 = v0 = sqrt(0.5))
    ps = ps * np.sqrt(0.5 / O.energy(g, ps, 1))
    vz = vz * np.sqrt(0.5 / O.energy(g, vz, 0))
    fp, fz = random_forcing(g, 2, 4.0, 6.0)
    fp = fp * np.sqrt(1.0 / O.energy(g, fp, 1))
    fz = fz * np.sqrt(1.0 / O.energy(g, fz, 0))
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.set_time(0.0)
    return g, p, c, ps, vz, fp, fz


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_256_steps_1_10_100(gpu, prec, tol):
    g, p, c, ps, vz, fp, fz = _setup(prec)
    done = 0
    for k in (1, 10, 100):
        c.advance(k - done, gpu.DT_FIXED, DT)
        for _ in range(k - done):
            ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, DT)
        done = k
        a, b = c.get_state()
        assert rel_l2(a, ps) < tol and rel_l2(b, vz) < tol, (k, rel_l2(a, ps), rel_l2(b, vz))


def test_256_fp64_1000_steps_spectrum(gpu):
    g, p, c, ps, vz, fp, fz = _setup(0)
    c.advance(1000, gpu.DT_FIXED, DT)
    for _ in range(1000):
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, DT)
    a, b = c.get_state()
    assert rel_l2(a, ps) < 1e-10 and rel_l2(b, vz) < 1e-10
    ek, ezk = c.spectrum()
    oek, oezk = O.spectrum(g, ps, vz)
    live = oek > 1e-14 * oek.max()
    assert np.max(np.abs(ek[live] - oek[live]) / oek[live]) < 1e-9
