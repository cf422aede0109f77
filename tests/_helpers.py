"""Shared helpers of the test-suite (seeded synthetic inputs, error norms)."""
import numpy as np

from oracle import rot2d3c_oracle as O


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def random_state(n: int, seed: int, kmin=1.0, kmax_shell=None, slope=-1.0, amp=1.0):
    """Truncated random-phase spectral pair (ps, vz) on an n-grid."""
    g = O.Grid(n)
    rng = np.random.default_rng(seed)
    km = kmax_shell if kmax_shell is not None else n / 3.0
    ps = O.random_phase_field(g, kmin, km, slope - 1.0, rng) * amp
    vz = O.random_phase_field(g, kmin, km, slope, rng) * amp
    return g, ps, vz


def random_forcing(g, seed: int, kmin=4.0, kmax_shell=6.0):
    rng = np.random.default_rng(seed)
    fp = O.random_phase_field(g, kmin, kmax_shell, 0.0, rng)
    fz = O.random_phase_field(g, kmin, kmax_shell, 0.0, rng)
    return fp, fz


def params(n, **kw):
    """Oracle Params and the matching C-ABI params."""
    import rot2d3c_gb300 as R
    p = O.Params(n=n, **kw)
    fields = {k: getattr(p, k) for k in p.__dataclass_fields__ if k not in ("idir", "odir")}
    return p, R.make_params(**fields)
