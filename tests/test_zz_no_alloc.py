"""The allocation-free Fisher entry point (rv_fisher_batch_static).

Callers that cannot allocate device memory (processes whose device memory
belongs to another allocator or a fixed budget, plugin hosts that forbid
hidden allocations) pass their own device buffers; the function's only extra
memory is a file-scope device array.  This test calls it through the C ABI
twice in a row (the second call with a larger table total, so the scratch
table is refilled) and checks both results against the FP64 oracle and
against rv_fisher_batch, within the Fisher tolerance (1e-9 relative); it
also runs a call on a non-default stream and checks that tables the scratch
cannot hold (a total above its limit, a negative count) are rejected with
the outputs untouched.  It is collected last so a failure here cannot stop
the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-9


def _static_fn():
    from rabbitvar_gb300 import api
    L = api.lib()
    f = L.rv_fisher_batch_static
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    f.restype = C.c_int
    return api, f


def _run_static(f, tabs, stream=None):
    torch = pytest.importorskip("torch")
    t = torch.tensor(np.ascontiguousarray(tabs, dtype=np.int32), device="cuda")
    p = torch.full((tabs.shape[0],), -1.0, dtype=torch.float64, device="cuda")
    r = torch.full((tabs.shape[0],), -1.0, dtype=torch.float64, device="cuda")
    err = C.create_string_buffer(256)
    torch.cuda.synchronize()
    handle = stream.cuda_stream if stream is not None else None
    st = f(t.data_ptr(), tabs.shape[0], p.data_ptr(), r.data_ptr(), handle, err, 256)
    torch.cuda.synchronize()
    return st, p.cpu().numpy(), r.cpu().numpy(), err.value.decode()


def _oracle(tabs):
    import oracle as O
    p = np.array([O.fisher(*map(int, t))[2] for t in tabs])
    ad = tabs[:, 0].astype(float) * tabs[:, 3]
    bc = tabs[:, 1].astype(float) * tabs[:, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where((ad != 0) & (bc != 0), np.maximum(ad / bc, bc / ad), 0.0)
    return p, ratio


def _close(a, b):
    return np.all(np.abs(a - b) <= REL * np.maximum(np.abs(b), 1e-300))


def test_static_fisher_matches_oracle_and_allocating_entry_point():
    api, f = _static_fn()
    ctx = api.Context(api.default_params(local_realign=0))
    rng = np.random.default_rng(5)
    first = rng.integers(0, 80, size=(500, 4)).astype(np.int32)
    first[0] = [0, 0, 0, 0]
    second = rng.integers(0, 2500, size=(300, 4)).astype(np.int32)
    second[1] = [9000, 3, 2, 7000]
    for tabs in (first, second):
        st, p, r, msg = _run_static(f, tabs)
        assert st == 0, msg
        p_ora, r_ora = _oracle(tabs)
        assert _close(p, p_ora)
        assert _close(r, r_ora)
        p_ref, r_ref = ctx.fisher(tabs)
        assert _close(p, p_ref)
        assert np.array_equal(r, r_ref)
    ctx.close()


def test_static_fisher_on_a_side_stream():
    torch = pytest.importorskip("torch")
    _, f = _static_fn()
    rng = np.random.default_rng(9)
    tabs = rng.integers(0, 300, size=(1000, 4)).astype(np.int32)
    side = torch.cuda.Stream()
    st, p, r, msg = _run_static(f, tabs, stream=side)
    assert st == 0, msg
    p_ora, r_ora = _oracle(tabs)
    assert _close(p, p_ora)
    assert _close(r, r_ora)


@pytest.mark.parametrize("bad", [[200000, 70000, 1, 1], [5, -1, 3, 2]])
def test_static_fisher_rejects_tables_it_cannot_hold(bad):
    _, f = _static_fn()
    tabs = np.array([[3, 4, 5, 6], bad], dtype=np.int32)
    st, p, r, msg = _run_static(f, tabs)
    assert st == -1 and "262143" in msg
    assert np.all(p == -1.0) and np.all(r == -1.0)  # outputs untouched
