"""The learned filter's tcgen05 kernels against the numpy oracle
(oracle/mlp_oracle.py) on the same weights and inputs.

Tolerances: forward probabilities within 2e-3 absolute; each gradient tensor
within 2e-2 relative (L2 norm of the difference over the norm of the
oracle's), which covers FP32 summation order and the occasional BF16 rounding
of an activation landing on the other side of a tie."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, seed=5):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 40)).astype(np.float32)
    y = (x[:, 0] + 0.5 * x[:, 1] - 0.25 * x[:, 2] ** 2 + 0.3 * rng.normal(size=n) > 0).astype(np.float32)
    return x, y


def test_forward_matches_oracle():
    import mlp_oracle as M
    from rabbitvar_gb300 import mlp
    m = mlp.Mlp(batch=512, seed=11)
    x, _ = _data(1000)
    probs = m.predict(x)
    p = mlp.unpack(m.params())
    logit, _ = M.forward(p, x)
    ref = 1.0 / (1.0 + np.exp(-logit))
    assert np.max(np.abs(probs - ref)) < 2e-3
    m.close()


@pytest.mark.parametrize("n,pos_weight", [(512, 1.0), (384, 3.0), (2048, 1.0)])
def test_gradients_match_oracle(n, pos_weight):
    import mlp_oracle as M
    from rabbitvar_gb300 import mlp
    m = mlp.Mlp(batch=2048 if n > 512 else 512, seed=12)
    x, y = _data(n, seed=n)
    g, loss = m.gradients(x, y, pos_weight)
    p = mlp.unpack(m.params())
    logit, cache = M.forward(p, x)
    ref_loss, dl = M.loss_and_dlogit(logit, y, pos_weight)
    gr = M.backward(p, cache, dl)
    assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss))
    gg = mlp.unpack(g)
    for k in gr:
        num = np.linalg.norm(gg[k] - gr[k])
        den = np.linalg.norm(gr[k]) + 1e-12
        assert num / den < 2e-2, (k, num / den)
    m.close()


def test_training_reduces_loss_and_fits():
    from rabbitvar_gb300 import mlp
    m = mlp.Mlp(batch=1024, seed=13)
    x, y = _data(20000, seed=1)
    losses = m.train(x, y, epochs=6, lr=2e-3)
    assert losses[-1] < 0.6 * losses[0]
    xt, yt = _data(4000, seed=2)
    acc = np.mean((m.predict(xt) > 0.5) == (yt > 0.5))
    assert acc > 0.85  # the labels carry noise (a 0.3-sigma term): ~0.9 is the best reachable
    m.close()
