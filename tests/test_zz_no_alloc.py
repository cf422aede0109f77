"""The allocation-free C2R entry point (r2d3c_fft_c2r_noalloc).

Callers whose device memory is owned by another allocator, or that may not
pay the implicit synchronisation of cudaMalloc/cudaFree, use this variant:
it keeps its scratch in a fixed file-scope device array instead of
allocating.  This test calls it through the C-ABI on device buffers and
checks it against the plan-based entry point (r2d3c_fft_c2r_dev) on two
calls in a row, against the oracle's C2R (including a nonzero imaginary
part at kx = 0 and kx = n/2, which the transform ignores), with its first
call of a fresh process made on a non-blocking stream, and that sizes above
its limit are refused.  The file name sorts last so that a run stopping at
the first failure has run every other test before it.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512])
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


@pytest.mark.parametrize("n", [32, 512])
def test_noalloc_c2r_matches_oracle(gpu, n):
    import torch
    lib = gpu.load()
    g = O.Grid(n)
    rng = np.random.default_rng(2000 + n)
    spec = rng.standard_normal((n // 2 + 1, n)) + 1j * rng.standard_normal((n // 2 + 1, n))
    # the imaginary parts at kx = 0 and kx = n/2 are nonzero here and must be ignored
    assert np.abs(spec[0].imag).min() > 0 and np.abs(spec[n // 2].imag).min() > 0
    want = O.c2r(g, spec)
    d_spec = torch.from_numpy(np.ascontiguousarray(spec.view(np.float64))).cuda()
    d_out = torch.empty((n, n), dtype=torch.float64, device="cuda")
    for call in range(2):
        d_out.fill_(float("nan"))
        rc = lib.r2d3c_fft_c2r_noalloc(n, C.c_void_p(d_spec.data_ptr()), C.c_void_p(d_out.data_ptr()), None)
        assert rc == 0, lib.r2d3c_last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert rel_l2(got, want) < 1e-13, (call, rel_l2(got, want))


_FRESH = r"""
import ctypes as C, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
import rot2d3c_gb300 as R
from oracle import rot2d3c_oracle as O
lib = R.load()
n = 256
s = torch.cuda.Stream()  # torch's pool streams are created non-blocking
rng = np.random.default_rng(7)
spec = rng.standard_normal((n // 2 + 1, n)) + 1j * rng.standard_normal((n // 2 + 1, n))
want = O.c2r(O.Grid(n), spec)
with torch.cuda.stream(s):
    d_spec = torch.from_numpy(np.ascontiguousarray(spec.view(np.float64))).to("cuda", non_blocking=False)
    d_out = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
s.synchronize()
for call in range(2):
    rc = lib.r2d3c_fft_c2r_noalloc(n, C.c_void_p(d_spec.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                   C.c_void_p(s.cuda_stream))
    assert rc == 0, lib.r2d3c_last_error()
    s.synchronize()
    got = d_out.cpu().numpy()
    err = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    assert err < 1e-13, (call, err)
print("fresh-process first call ok")
"""


def test_noalloc_first_call_of_a_fresh_process_on_a_nonblocking_stream(gpu):
    """The set-up of the first call (twiddle upload) must be complete before
    kernels on a stream that does not wait for the legacy default stream
    read it; a fresh process makes that call the very first one."""
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh-process first call ok" in r.stdout


def test_noalloc_rejects_sizes_above_its_limit(gpu):
    import torch
    lib = gpu.load()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.r2d3c_fft_c2r_noalloc(1024, C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert rc == -1
    assert b"512" in lib.r2d3c_last_error()
