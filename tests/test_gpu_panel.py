"""Batched amplicon panel (-t -u): all regions in one submit and one
persistent pileup launch give the oracle's records, and the same records as
one call per region."""
import pytest

from cmp import diff_records

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [0, 1])
def test_batched_panel_matches_oracle_and_per_region(k):
    import numpy as np
    import oracle as O
    from rabbitvar_gb300 import api, synth
    g, _, rs, regions = synth.amplicon_panel(seed=0x5EED0002, n_regions=24, genome_len=24 * 5000,
                                             median_depth=150.0)
    params = dict(local_realign=k, dedup=1, unique_fwd=1)
    ctx = api.Context(api.default_params(**params))
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    batched = ctx.call(api.Batch.from_readset(rs), regions, "S", rs.contig).splitlines()
    n, ora = O.run_regions(rs, g, regions, params=O.default_params(**params))
    assert n > 20
    assert diff_records(ora.splitlines(), batched) == []
    if k:
        # -k 1's noPassingReads reads every record of the batch, so one call
        # per region on a subset of the reads is not the same computation
        ctx.close()
        return
    per = []
    span = rs.pos.astype(np.int64) + 150
    for a, b in regions:
        idx = np.nonzero((rs.pos < b) & (span > a - 1 - 200))[0]
        per += ctx.call(api.Batch.from_readset(synth.take(rs, idx)), [(a, b)], "S", rs.contig).splitlines()
    assert sorted(per) == sorted(batched)
    ctx.close()
