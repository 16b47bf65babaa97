"""The learned-vs-hard evaluation (learn.compare) on hand-made scores: equal
recall, equal precision and best-F1 operating points (CPU only)."""
import numpy as np


def test_compare_operating_points():
    from rabbitvar_gb300 import learn
    # 10 candidates: 4 true.  Hard filter calls 3 (2 true): precision 2/3, recall 1/2.
    y = np.array([1, 1, 1, 1, 0, 0, 0, 0, 0, 0], np.float32)
    hard = np.array([1, 1, 0, 0, 1, 0, 0, 0, 0, 0], np.float32)
    # scores rank three true candidates first, then a false one, then the last true one
    s = np.array([0.9, 0.8, 0.7, 0.3, 0.6, 0.2, 0.1, 0.05, 0.04, 0.01], np.float32)
    r = learn.compare(s, y, hard)
    assert r["hard"]["called"] == 3 and abs(r["hard"]["precision"] - 2 / 3) < 1e-12
    assert abs(r["hard"]["recall"] - 0.5) < 1e-12
    # equal recall (2 true kept): the two top scores, precision 1
    assert r["learned"]["called"] == 2 and r["learned"]["precision"] == 1.0
    # at precision >= 2/3 the learned filter keeps 3 true of 4 (3 called) -> recall 0.75
    # (4 true needs 5 calls: precision 0.8 >= 2/3, recall 1.0)
    eq = r["learned_at_hard_precision"]
    assert eq["recall"] == 1.0 and eq["called"] == 5 and eq["precision"] >= 2 / 3
    assert abs(r["learned_best_f1"]["f1"] - max(2 * 1 * 0.75 / 1.75, 2 * 0.8 / 1.8)) < 1e-9


def test_compare_ties_are_one_threshold():
    from rabbitvar_gb300 import learn
    y = np.array([1, 0, 1, 0], np.float32)
    hard = np.array([1, 0, 0, 0], np.float32)
    s = np.array([0.5, 0.5, 0.5, 0.1], np.float32)  # a threshold cannot split the tie
    r = learn.compare(s, y, hard)
    assert r["learned_at_hard_precision"]["called"] in (0, 3) or r["learned_at_hard_precision"]["precision"] >= 1.0
    assert r["learned_best_f1"]["called"] in (3, 4)
