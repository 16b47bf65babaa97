"""The allocation-free Fisher entry point (rv_fisher_batch_static).

Callers that cannot allocate device memory (graph-capture code that must not
allocate, processes whose device memory belongs to another allocator or a
fixed budget, plugin hosts) pass their own device buffers; the function's
only extra memory is a file-scope device array.  This test calls it through
the C ABI twice in a row (the second call with a larger table total, so the
scratch table is refilled) and checks both results against rv_fisher_batch
within the Fisher tolerance (1e-9 relative).  It is collected last so a
failure here cannot stop the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_fn():
    from rabbitvar_gb300 import api
    L = api.lib()
    f = L.rv_fisher_batch_static
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    f.restype = C.c_int
    return api, f


def _run_static(f, tabs):
    torch = pytest.importorskip("torch")
    t = torch.tensor(np.ascontiguousarray(tabs, dtype=np.int32), device="cuda")
    p = torch.full((tabs.shape[0],), -1.0, dtype=torch.float64, device="cuda")
    r = torch.full((tabs.shape[0],), -1.0, dtype=torch.float64, device="cuda")
    err = C.create_string_buffer(256)
    st = f(t.data_ptr(), tabs.shape[0], p.data_ptr(), r.data_ptr(), None, err, 256)
    torch.cuda.synchronize()
    return st, p.cpu().numpy(), r.cpu().numpy(), err.value.decode()


def test_static_fisher_matches_allocating_entry_point():
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
        p_ref, r_ref = ctx.fisher(tabs)
        assert np.all(np.abs(p - p_ref) <= 1e-9 * np.maximum(np.abs(p_ref), 1e-300))
        assert np.array_equal(r, r_ref)


def test_static_fisher_rejects_oversized_tables():
    api, f = _static_fn()
    tabs = np.array([[200000, 70000, 1, 1]], dtype=np.int32)
    st, p, r, msg = _run_static(f, tabs)
    assert st == -1 and "262143" in msg
    assert p[0] == -1.0  # outputs untouched
