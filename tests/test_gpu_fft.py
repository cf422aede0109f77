"""Level-1 transforms (fftp2D.f90:133-290) on the GPU against the oracle."""
import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu

SMALL = [16, 32, 64, 128, 256, 512]
TOL = {0: 1e-13, 1: 3e-6}  # FP64, FP32 relative L2


@pytest.mark.parametrize("n", SMALL)
@pytest.mark.parametrize("prec", [0, 1])
def test_r2c_matches_oracle(gpu, n, prec):
    g = O.Grid(n)
    r = np.random.default_rng(n).standard_normal((n, n))
    out = gpu.FFTPlan(n, gpu.R2C, prec).r2c(r)
    assert rel_l2(out, O.r2c(g, r)) < TOL[prec]
    # exact zeros of the real transform: Im at kx = 0, ky = 0 and at the Nyquists
    if prec == 0:
        assert out[0, 0].imag == 0.0 and out[n // 2, 0].imag == 0.0


@pytest.mark.parametrize("n", SMALL)
@pytest.mark.parametrize("prec", [0, 1])
def test_c2r_matches_oracle_and_ignores_imag_of_dc_and_nyquist(gpu, n, prec):
    g = O.Grid(n)
    rng = np.random.default_rng(100 + n)
    c = rng.standard_normal((n // 2 + 1, n)) + 1j * rng.standard_normal((n // 2 + 1, n))
    out = gpu.FFTPlan(n, gpu.C2R, prec).c2r(c)
    assert rel_l2(out, O.c2r(g, c)) < TOL[prec]


@pytest.mark.parametrize("n", [16, 64, 1024, 2048, 4096, 8192])
@pytest.mark.parametrize("prec", [0, 1])
def test_roundtrip_is_n2_times_identity(gpu, n, prec):
    r = np.random.default_rng(7).standard_normal((n, n))
    c = gpu.FFTPlan(n, gpu.R2C, prec).r2c(r)
    back = gpu.FFTPlan(n, gpu.C2R, prec).c2r(c)
    tol = {0: 2e-15, 1: 1e-6}[prec] * np.log2(n)
    assert rel_l2(back / float(n) ** 2, r) < tol


def test_single_mode_known_answer(gpu):
    """cos(3x + 2y) transforms to n^2/2 at (kx,ky) = (3,2) and nothing else."""
    n = 32
    x = np.arange(n)
    xx, yy = np.meshgrid(x, x)  # [y][x]
    r = np.cos(2 * np.pi * (3 * xx + 2 * yy) / n)
    c = gpu.FFTPlan(n, gpu.R2C, 0).r2c(r)
    expect = np.zeros((n // 2 + 1, n), complex)
    expect[3, 2] = n * n / 2
    assert np.abs(c - expect).max() < 1e-11


def test_dev_pointer_variants(gpu):
    import torch
    n = 64
    g = O.Grid(n)
    r = np.random.default_rng(3).standard_normal((n, n))
    d_in = torch.from_numpy(r).cuda()
    d_spec = torch.empty((n // 2 + 1, n, 2), dtype=torch.float64, device="cuda")
    d_back = torch.empty((n, n), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    gpu.FFTPlan(n, gpu.R2C, 0).r2c_dev(d_in.data_ptr(), d_spec.data_ptr(), s)
    gpu.FFTPlan(n, gpu.C2R, 0).c2r_dev(d_spec.data_ptr(), d_back.data_ptr(), s)
    torch.cuda.synchronize()
    spec = d_spec.cpu().numpy()
    assert rel_l2(spec[..., 0] + 1j * spec[..., 1], O.r2c(g, r)) < 1e-13
    assert rel_l2(d_back.cpu().numpy() / n**2, r) < 1e-14
