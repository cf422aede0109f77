"""The 4096^2 workload of the benchmark (RK4, fixed dt = 1e-4, nu = 1e-5,
hypoviscosity 0.1 with mm = 2, Omega = 10, seeded k^-3 initial spectrum on
1 <= |k| <= 100, forcing shell 20-22) after 100 steps: the FP64 drop-in path
against the C/OpenMP oracle (relative L2 <= 1e-12 for psi, vz and omega =
k^2 psi) and the FP32 path against the same oracle state (<= 1e-5).

At this size the GPU runs its large-grid kernel variants (the launch shapes
the plan autotuner picks at 4096, the persistent cp.async-staged pass B of
the FP32 path), which the smaller parity cases do not reach.  The oracle's
100 steps take about a minute on 16 host threads; the result is shared by
both precisions.
"""
import numpy as np
import pytest

from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu

N, DT, STEPS = 4096, 1e-4, 100


@pytest.fixture(scope="module")
def oracle_state():
    import bench
    from oracle import cpu_oracle as CO
    from oracle import rot2d3c_oracle as O
    ps, vz, fp, fz, ka2 = bench.workload_inputs(N)
    w = bench.WORKLOAD
    p = O.Params(n=N, nu=w["nu"], hnu=w["hnu"], nn=w["nn"], mm=w["mm"], nuv=w["nu"], hnuv=w["hnu"],
                 nnv=w["nn"], mmv=w["mm"], omega=w["omega"], iflow=0)
    a, b, _ = CO.run(p, ps, vz, fp, fz, STEPS, DT, False)
    return (ps, vz, fp, fz, ka2), (a, b)


def _gpu_state(gpu, prec, inputs):
    import bench
    ps, vz, fp, fz, _ = inputs
    c = gpu.Context(bench.make_cparams(N), prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.set_time(0.0)
    t, _ = c.advance(STEPS, gpu.DT_FIXED, DT)
    a, b = c.get_state()
    c.destroy()
    assert abs(t - STEPS * DT) < 1e-12
    return a, b


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_4096_100_steps_against_oracle(gpu, oracle_state, prec, tol):
    inputs, (oa, ob) = oracle_state
    ka2 = inputs[4]
    a, b = _gpu_state(gpu, prec, inputs)
    e_ps, e_vz, e_w = rel_l2(a, oa), rel_l2(b, ob), rel_l2(ka2 * a, ka2 * oa)
    print(f"4096^2 {'FP64' if prec == 0 else 'FP32'} after {STEPS} steps vs oracle: "
          f"psi {e_ps:.2e} vz {e_vz:.2e} omega {e_w:.2e}")
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert e_ps <= tol and e_vz <= tol and e_w <= tol, (e_ps, e_vz, e_w)
