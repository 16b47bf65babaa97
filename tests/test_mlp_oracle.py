"""The MLP oracle itself: its backward pass against central finite
differences of its loss (FP64 copies of the weights, no BF16 rounding), and
its BF16 rounding against the bit-level definition."""
import numpy as np


def test_bf16_rounding_ties_to_even():
    import mlp_oracle as M
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e38], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even mantissa
    assert r[2] == np.float32(1.0 + 2 ** -6)  # tie -> even (rounds up)
    assert r[3] == -2.5


def test_backward_matches_finite_differences():
    import mlp_oracle as M
    rng = np.random.default_rng(7)
    p = M.init_params(3)
    x = rng.normal(size=(32, M.N_FEAT)).astype(np.float32)
    y = (rng.random(32) < 0.3).astype(np.float32)

    def loss_of(pp):
        logit, _ = M.forward(pp, x, exact=True)
        return M.loss_and_dlogit(logit, y, 2.0)[0]

    logit, cache = M.forward(p, x, exact=True)
    _, dl = M.loss_and_dlogit(logit, y, 2.0)
    g = M.backward(p, cache, dl)
    for key, idx in [("W1", (5, 7)), ("W2", (3, 100)), ("W3", (127, 0)), ("b2", (17,)), ("w4", (9,)), ("b4", (0,))]:
        eps = 1e-2
        pp = {k: v.copy() for k, v in p.items()}
        pp[key][idx] += eps
        lp = loss_of(pp)
        pp[key][idx] -= 2 * eps
        lm = loss_of(pp)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[key][idx]) <= 2e-3 * max(1.0, abs(fd)) + 2e-5, (key, idx, fd, g[key][idx])
