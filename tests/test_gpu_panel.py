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


@pytest.mark.parametrize("k", [0, 1])
def test_panel_pileup_graph_matches_direct_launches(k):
    """rv_pileup under a CUDA graph (rv_set_pileup_graph) gives the records of
    direct launches on every call: the autotuner's trial calls (direct), the
    first graph and its replays.  With -k 0, one call per region (a different
    batch geometry on every call, so the graph is updated between calls) gives
    the batched records too."""
    import numpy as np
    from rabbitvar_gb300 import api, synth
    g, _, rs, regions = synth.amplicon_panel(seed=0x5EED0002, n_regions=24, genome_len=24 * 5000,
                                             median_depth=150.0)
    params = dict(local_realign=k, dedup=1, unique_fwd=1)
    genome = synth.genome_str(g).encode()
    batch = api.Batch.from_readset(rs)
    direct = api.Context(api.default_params(**params))
    direct.upload_reference(rs.contig, genome)
    want = sorted(direct.call(batch, regions, "S", rs.contig).splitlines())
    direct.close()
    assert len(want) > 20
    ctx = api.Context(api.default_params(**params))
    ctx.upload_reference(rs.contig, genome)
    ctx.set_pileup_graph(True)
    for _ in range(6):
        assert sorted(ctx.call(batch, regions, "S", rs.contig).splitlines()) == want
    launches, inst = ctx.pileup_graph_stats()
    assert launches >= 3 and 1 <= inst <= launches
    if k == 0:
        per = []
        span = rs.pos.astype(np.int64) + 150
        for a, b in regions:
            idx = np.nonzero((rs.pos < b) & (span > a - 1 - 200))[0]
            per += ctx.call(api.Batch.from_readset(synth.take(rs, idx)), [(a, b)], "S", rs.contig).splitlines()
        assert sorted(per) == want
        assert ctx.pileup_graph_stats()[0] == launches + len(regions)
    ctx.close()
