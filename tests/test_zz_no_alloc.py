"""The allocation-free C2R entry point (r2d3c_fft_c2r_noalloc).

Callers whose device memory is owned by another allocator, or that may not
pay the implicit synchronisation of cudaMalloc/cudaFree, use this variant:
it keeps its scratch in a fixed file-scope device array instead of
allocating.  This test calls it through the C-ABI on device buffers and
checks it against the plan-based entry point (r2d3c_fft_c2r_dev) on two
calls in a row, and that sizes above its limit are refused.  The file name
sorts last so that a run stopping at the first failure has run every other
test before it.
"""
import ctypes as C

import numpy as np
import pytest

from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [16, 64, 256, 512])
def test_noalloc_c2r_matches_plan_entry_point(gpu, n):
    import torch
    lib = gpu.load()
    rng = np.random.default_rng(1000 + n)
    plan = gpu.FFTPlan(n, gpu.C2R, gpu.FP64)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # the second call reuses the scratch left by the first
        spec = rng.standard_normal((n // 2 + 1, n, 2))
        d_spec = torch.from_numpy(spec).cuda()
        d_na = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        d_ref = torch.empty((n, n), dtype=torch.float64, device="cuda")
        rc = lib.r2d3c_fft_c2r_noalloc(n, C.c_void_p(d_spec.data_ptr()), C.c_void_p(d_na.data_ptr()),
                                       C.c_void_p(stream))
        assert rc == 0, lib.r2d3c_last_error()
        plan.c2r_dev(d_spec.data_ptr(), d_ref.data_ptr(), stream)
        torch.cuda.synchronize()
        a, b = d_na.cpu().numpy(), d_ref.cpu().numpy()
        assert np.isfinite(a).all()
        assert rel_l2(a, b) < 1e-13, (call, rel_l2(a, b))


def test_noalloc_rejects_sizes_above_its_limit(gpu):
    import torch
    lib = gpu.load()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.r2d3c_fft_c2r_noalloc(1024, C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert rc == -1
    assert b"512" in lib.r2d3c_last_error()
