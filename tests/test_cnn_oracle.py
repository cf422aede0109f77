"""The float64 CNN reference (CPU): its hand-derived backward pass agrees with
central finite differences, and bfloat16 rounding is round-to-nearest-even."""
import numpy as np

from oracle import cnn_oracle as CO


def test_reference_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n = sum(9 * a * b + b for a, b in zip(CO.CIN, CO.COUT))
    p = rng.uniform(-0.2, 0.2, n)
    x = rng.standard_normal((1, 4, 4, 8))
    t = rng.standard_normal((1, 4, 4, 2))
    _, g = CO.loss_and_grads(p, x, t, emulate=False)
    for idx in [0, 100, 2303, 2309, 12000, n - 1, n - 3, n - 70]:
        e = np.zeros(n)
        e[idx] = 1e-6
        fd = (CO.loss_and_grads(p + e, x, t, False)[0] - CO.loss_and_grads(p - e, x, t, False)[0]) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx]))


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159])
    r = CO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-12
