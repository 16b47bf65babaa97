"""FP64 Fisher restatement against scipy.stats.fisher_exact (two-sided).

htslib's kt_fisher_exact is not available here, so parity with htslib's own
p-values is unpinned; the restatement is pinned to scipy instead."""
import numpy as np
import pytest


def test_fisher_vs_scipy():
    stats = pytest.importorskip("scipy.stats")
    import oracle as O
    rng = np.random.default_rng(1)
    tabs = rng.integers(0, 40, size=(300, 4)).tolist()
    tabs += rng.integers(0, 600, size=(40, 4)).tolist()
    tabs += [[0, 0, 0, 0], [10, 0, 0, 10], [3, 3, 3, 3], [200, 1, 1, 200], [0, 5, 5, 0]]
    for a, b, c, d in tabs:
        _, _, two = O.fisher(a, b, c, d)
        ref = stats.fisher_exact([[a, b], [c, d]], alternative="two-sided")[1]
        assert abs(two - ref) <= 1e-9 * max(ref, 1e-300) or abs(two - ref) < 1e-12, (a, b, c, d, two, ref)


def test_fisher_tails():
    import oracle as O
    left, right, two = O.fisher(12, 5, 29, 2)
    assert 0 <= left <= 1 and 0 <= right <= 1 and two >= min(left, right) - 1e-15
