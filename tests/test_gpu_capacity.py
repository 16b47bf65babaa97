"""Device tables that overflow grow, and the pileup runs again.

The hash table of string-keyed alleles, the key-text arena, the list of
deferred reference-base subtractions and the list of map entries whose
pstd/qstd are replayed in read order are forced far below what the read set
needs (rv_set_capacities).  The kernels set an error bit and drop what does
not fit; rv_pileup grows the tables to what the run needed and runs the
pileup again.  The records must then equal the reference's golden records,
with at least one re-run counted."""
import json
import os

import pytest

from cmp import diff_records, flag_params, widened

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))


def _make_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


@pytest.mark.parametrize("name,caps", [
    ("germline_dense_k1", dict(hash_slots=64)),
    ("germline_dense_k1", dict(arena_bytes=64)),
    ("dense_multi_k1", dict(deferred=1)),
    ("paths_q0", dict(order_fix=1)),
    ("dense_multi_k1", dict(hash_slots=16, arena_bytes=16, deferred=1, order_fix=1)),
])
def test_tables_grow_and_pileup_reruns(name, caps):
    from rabbitvar_gb300 import api, synth
    mg = _make_golden()
    cases = dict(mg.CASES)
    cases.update(mg.RECORDS_ONLY)
    g, rs, (a, b), flags = cases[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"]
    ctx = api.Context(api.default_params(**flag_params(flags)))
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    ctx.set_capacities(**caps)
    text = ctx.call(api.Batch.from_readset(rs), [widened(a, b, flags)], "S", rs.contig)
    stats = ctx.capacity_stats()
    # a second batch on the grown tables needs no re-run
    text2 = ctx.call(api.Batch.from_readset(rs), [widened(a, b, flags)], "S", rs.contig)
    stats2 = ctx.capacity_stats()
    ctx.close()
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    assert diff_records(recs, text.splitlines()) == []
    assert text2 == text
    assert stats["retries"] >= 1
    assert stats2["retries"] == stats["retries"]
