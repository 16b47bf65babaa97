"""-k 1 (the reference's default) through the GPU path: the device CIGAR
rewrite and pileup, the host realigner (adjustMNP and the indel passes
realigndel / realignins / realignlgins30) over the device-built maps with its
changes patched back, and the device scoring.

The maps after the realigner (R stage) must equal the reference's own dump
(golden) and the oracle's; the records must equal the reference's golden
records.  Counts and keys are exact; fractional sums (the realigner's
adjRefCnt / adjRefFactor factors, the GPU's quality sums) within 1e-9
relative."""
import gzip
import json
import os

import pytest

from cmp import diff_dump, diff_records

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
R_TAGS = ["RN", "RI", "RC"]


def _make_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def _run(g, rs, regions, **kw):
    from rabbitvar_gb300 import api, synth
    ctx = api.Context(api.default_params(local_realign=1, **kw))
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    ctx.submit(api.Batch.from_readset(rs), regions)
    ctx.pileup()
    ctx.realign()
    r_dumps = [ctx.export_maps(i, "R") for i in range(len(regions))]
    ctx.score()
    text, _ = ctx.format_records("S", rs.contig)
    ctx.close()
    return r_dumps, text.splitlines()


def test_k1_maps_and_records_match_reference_golden():
    """germline_dense_k1: R-stage maps against the reference's own dump,
    records against its records."""
    mg = _make_golden()
    g, rs, (a, b), flags = mg.CASES["germline_dense_k1"]()
    assert mg.readset_fingerprint(rs) == META["germline_dense_k1"]["fingerprint"]
    gold = gzip.open(os.path.join(GOLD, "germline_dense_k1.dump.txt.gz"), "rt").read()
    r, mine = _run(g, rs, [(a, b)])
    assert diff_dump(gold, r[0], R_TAGS, rel=1e-9) == []
    recs = open(os.path.join(GOLD, "germline_dense_k1.records.txt")).read().splitlines()
    assert len(recs) > 5
    assert diff_records(recs, mine) == []


@pytest.mark.parametrize("name", ["contig_end_k1", "dense_multi_k1"])
def test_k1_records_match_reference_golden(name):
    mg = _make_golden()
    g, rs, (a, b), flags = mg.RECORDS_ONLY[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"]
    _, mine = _run(g, rs, [(a, b)], fisher=1 if "--fisher" in flags else 0)
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    assert len(recs) == META[name]["records"] > 5
    assert diff_records(recs, mine) == []


@pytest.mark.parametrize("case", ["germline", "tiles"])
def test_k1_maps_match_oracle(case, germline_small):
    """R-stage maps of every region against the oracle (one region of 100 kb;
    ten 6-kb regions in one batch), and the records of the whole batch."""
    import oracle as O
    from rabbitvar_gb300 import synth
    if case == "germline":
        g, _, rs = germline_small
        regions = [(1, 100000)]
    else:
        g, _, rs = synth.dense_multi()
        regions = [(1 + 6000 * i, 6000 * (i + 1)) for i in range(10)]
    r, mine = _run(g, rs, regions)
    prm = O.default_params(local_realign=1)
    for i in range(len(regions)) if len(regions) < 4 else (0, 3, 6, 9):
        ora = O.run_region(rs, g, regions[i][0], regions[i][1], stages="R", params=prm)
        assert diff_dump(ora, r[i], R_TAGS, rel=1e-9) == [], f"region {i}"
    n, ora_text = O.run_regions(rs, g, regions, params=prm)
    assert n > 50
    assert diff_records(ora_text.splitlines(), mine) == []


def test_k1_somatic_matches_reference_golden():
    """Somatic pair with -k 1 --fisher: the 63-column records against the
    reference's golden records."""
    from rabbitvar_gb300 import api, synth
    g, _, t, n = synth.somatic_mix(0x5EED0051)
    pair = api.SomaticPair(api.default_params(local_realign=1, fisher=1))
    pair.upload_reference(t.contig, synth.genome_str(g).encode())
    mine = pair.call(api.Batch.from_readset(t), api.Batch.from_readset(n), [(1, g.shape[0])], "T", t.contig)
    pair.close()
    gold = open(os.path.join(GOLD, "somatic_mix_k1.records.txt")).read().splitlines()
    assert len(gold) > 50
    assert diff_records(gold, mine.splitlines(), somatic=True) == []
