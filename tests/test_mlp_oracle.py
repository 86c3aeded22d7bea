"""CPU checks of the warm-start network's oracle (oracle/mlp_oracle.py): its
analytic gradient against central finite differences, and the BF16 rounding
used to mirror the engine's weights."""
import numpy as np

import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in, h1, h2 = 6, 5, 4
    p = rng.normal(0, 0.5, h1 * n_in + h1 + h2 * h1 + h2 + h2 + 1)
    x = rng.normal(0, 1, (17, n_in))
    y = rng.normal(0, 1, 17)
    # the calculus of the gradient, without the BF16 operand rounding (piecewise constant)
    _, g = M.loss_and_grad(p, x, y, n_in, h1, h2, exact=True)
    eps = 1e-6
    fd = np.zeros_like(p)
    for k in range(len(p)):
        a, b = p.copy(), p.copy()
        a[k] += eps
        b[k] -= eps
        fd[k] = (M.loss_and_grad(a, x, y, n_in, h1, h2, exact=True)[0] -
                 M.loss_and_grad(b, x, y, n_in, h1, h2, exact=True)[0]) / (2 * eps)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-8)


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 1e-3], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # a tie rounds to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - v[3]) <= 2 ** -7 * abs(v[3])
    assert abs(r[4] - v[4]) <= 2 ** -8 * abs(v[4])
