"""Somatic mode (tumor/normal pair) on the GPU against the oracle, which is
pinned to the reference binary's own records (tests/golden/somatic_*.txt).

Records must match one for one: the same alleles with the same label,
integer and string columns equal, %f columns within 2e-6 relative (the
Fisher p-values are FP64 on both sides)."""
import pytest

from cmp import diff_records, diff_vcf

pytestmark = pytest.mark.gpu


def _pair(**kw):
    from rabbitvar_gb300 import api
    return api, api.SomaticPair(api.default_params(local_realign=0, **kw))


def _run(g, t, n, regions, **kw):
    from rabbitvar_gb300 import synth
    api, pair = _pair(**kw)
    pair.upload_reference(t.contig, synth.genome_str(g).encode())
    text = pair.call(api.Batch.from_readset(t), api.Batch.from_readset(n), regions, "T", t.contig)
    pair.close()
    return text.splitlines()


@pytest.mark.parametrize("seed,fisher", [(0x5EED0051, 1), (0x5EED0052, 0), (0x5EED0053, 1)])
def test_somatic_whole_contig(seed, fisher):
    import oracle as O
    from rabbitvar_gb300 import synth
    g, _, t, n = synth.somatic_mix(seed)
    mine = _run(g, t, n, [(1, g.shape[0])], fisher=fisher)
    ora = O.run_somatic(t, n, g, 1, g.shape[0], "O", "T", O.default_params(local_realign=0, fisher=fisher))
    ora = ora.splitlines()
    assert len(ora) > 100
    assert len(mine) == len(ora)
    assert diff_records(ora, mine, somatic=True) == []
    labels = {r.split("\t")[-11 if fisher else -7] for r in mine}
    assert {"StrongSomatic", "Germline", "LikelyLOH", "StrongLOH", "SampleSpecific"} <= labels


def test_somatic_tiles_match_golden():
    """BED-style tiles over the golden pair: the union of per-region records
    equals the oracle's per-region runs, and the whole-contig run equals the
    reference's golden records."""
    import os
    import oracle as O
    from rabbitvar_gb300 import synth
    g, _, t, n = synth.somatic_mix(0x5EED0051)
    gold = open(os.path.join(os.path.dirname(__file__), "golden", "somatic_mix.records.txt")).read().splitlines()
    mine = _run(g, t, n, [(1, g.shape[0])], fisher=1)
    assert diff_records(gold, mine, somatic=True) == []
    # and through the VCF writer: the reference writer's VCF of its own records
    from rabbitvar_gb300 import vcf
    want = open(os.path.join(os.path.dirname(__file__), "golden", "somatic_mix.vcf")).read()
    assert diff_vcf(want, vcf.write("\n".join(mine) + "\n", "TUMOR")) == []
    tiles = [(1 + 3000 * i, 3000 * (i + 1)) for i in range(10)]
    mine_t = _run(g, t, n, tiles, fisher=1)
    _, ora_t = O.run_somatic_regions(t, n, g, tiles, "T", O.default_params(local_realign=0, fisher=1))
    ora_t = ora_t.splitlines()
    assert len(mine_t) == len(ora_t) > 100
    assert diff_records(ora_t, mine_t, somatic=True) == []


def test_somatic_stream_matches_calls():
    """rv_call_somatic_stream over five batches (two context pairs, records
    formatted on a host thread while the next batch is piled up, a batch's
    reads uploaded while the batch before it on the same pair is realigned;
    batches of different sizes, so an early upload replaces a larger or
    smaller batch) gives the records of one call per batch, in order."""
    from rabbitvar_gb300 import api, synth
    g, _, t, n = synth.somatic_mix(0x5EED0051)
    regions = [[(1, g.shape[0])], [(1, 3000), (3001, 9000), (9001, g.shape[0])], [(8001, 20000)]]
    params = dict(local_realign=1, fisher=1)
    pair = api.SomaticPair(api.default_params(**params))
    pair.upload_reference(t.contig, synth.genome_str(g).encode())
    bt, bn = api.Batch.from_readset(t), api.Batch.from_readset(n)
    # the first half of each sample's reads as a second batch
    ht = api.Batch.from_readset(synth.read_range(t, 0, t.n // 2))
    hn = api.Batch.from_readset(synth.read_range(n, 0, n.n // 2))
    jobs = [(bt, bn, regions[0]), (bt, bn, regions[1]), (ht, hn, regions[0]), (bt, bn, regions[2]),
            (bt, bn, regions[0])]
    want = [pair.call(a, b, rg, "T", t.contig) for a, b, rg in jobs]
    pair.close()
    stream = api.SomaticStream(api.default_params(**params))
    stream.upload_reference(t.contig, synth.genome_str(g).encode())
    got = stream.run(jobs, "T", t.contig)
    stream.close()
    assert got == want
    assert all(len(w.splitlines()) > 10 for w in want)
    assert want[2] != want[0]
