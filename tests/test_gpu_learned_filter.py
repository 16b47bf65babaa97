"""The learned filter against the hard filter on held-out synthetic deep
panels (planted truth): at the hard filter's recall the learned filter's
F1 must be at least the hard filter's, and at the hard filter's precision
its recall must be at least the hard filter's."""
import pytest

pytestmark = pytest.mark.gpu


def test_learned_filter_f1_at_equal_recall():
    from rabbitvar_gb300 import learn, mlp
    xtr, ytr, _ = learn.dataset([101, 102, 103, 104], n_regions=6)
    xte, yte, hte = learn.dataset([201, 202], n_regions=6)
    assert ytr.sum() > 200 and yte.sum() > 50
    m = mlp.Mlp(batch=4096, seed=3)
    losses = m.train(xtr, ytr, epochs=20, lr=1e-3)
    assert losses[-1] < losses[0]
    res = learn.compare(m.predict(xte), yte, hte)
    m.close()
    assert res["learned"]["recall"] >= res["hard"]["recall"] - 1e-9
    assert res["learned"]["f1"] >= res["hard"]["f1"], res
    eq = res["learned_at_hard_precision"]
    assert eq["precision"] >= res["hard"]["precision"] - 1e-12
    assert eq["recall"] >= res["hard"]["recall"], res
