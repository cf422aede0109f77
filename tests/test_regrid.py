"""Regridding: the reference's slice regridder (regrid_slices.f90) restated
as one gather, against the literal slice loops; the GPU gather and the
spectral zero-padding."""
import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import params, random_state, rel_l2


def _global_map(old, m):
    n = old.shape[0]
    src = (np.arange(m) + 2) * n // m - 1
    return old[np.ix_(src, src)]


@pytest.mark.parametrize("n,m,nn,mn", [(8, 16, 2, 4), (16, 32, 4, 8), (12, 18, 3, 3), (16, 24, 2, 4), (32, 64, 1, 1)])
def test_slice_loops_are_one_global_gather(n, m, nn, mn):
    """The per-slice loops of the reference equal out[y][x] = in[(y+2)n/m-1][(x+2)n/m-1]
    (0-based) whatever the slicing, which is what the GPU kernel computes."""
    rng = np.random.default_rng(n * m + nn)
    old = rng.standard_normal((n, n))
    np.testing.assert_array_equal(O.regrid_slices(old, n, m, nn, mn), _global_map(old, m))


@pytest.mark.gpu
@pytest.mark.parametrize("n,m", [(64, 128), (96, 160), (256, 512)])
def test_gpu_regrid_physical_matches_reference_loops(gpu, n, m):
    rng = np.random.default_rng(n + m)
    old = rng.standard_normal((n, n))
    new = gpu.regrid_physical(old, m)
    np.testing.assert_array_equal(new, O.regrid_slices(old, n, m, 1, 1))


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_spectral_regrid_keeps_the_field(gpu, prec, tol):
    """Zero-padding 64^2 -> 128^2: the physical fields agree on the common
    grid points, and filtering back (the closure's sharp cutoff) returns the
    original retained modes."""
    import torch
    from rot2d3c_gb300.closure import closure_sample
    nc, nf = 64, 128
    g, ps, vz = random_state(nc, 17, amp=3.0)
    _, cpc = params(nc, iflow=0)
    _, cpf = params(nf, iflow=0)
    c, f = gpu.Context(cpc, prec), gpu.Context(cpf, prec)
    c.set_state(ps, vz)
    gpu.regrid_spectral(c, f)
    pc, pf = c.get_field(0), f.get_field(0)
    assert rel_l2(pf[::2, ::2], pc) < tol
    back = gpu.Context(cpc, prec)
    x = torch.zeros((nc, nc, 8), dtype=torch.float32, device="cuda")
    y = torch.zeros((nc, nc, 2), dtype=torch.float32, device="cuda")
    closure_sample(f, back, x, y)
    a, b = back.get_state()
    assert rel_l2(a, ps) < tol and rel_l2(b, vz) < tol
