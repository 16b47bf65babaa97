"""One locus per pileup code path through the GPU path, against the
reference's own output on the same reads.

The `paths_k0` / `paths_k1` golden cases (tests/golden/make_golden.py,
`_path_reads`) are hand-written reads: MNV growth and its quality stop,
deletions with unequal flank qualities, an insertion shifted 3' in a
homopolymer and one after a leading soft clip, reference-matching and
foreign soft clips with low-quality stops, mismatches beside indels, the
record filters (unmapped/secondary/duplicate/supplementary flags, a one-base
read, too many mismatches, both ends clipped), MAPQ 0, hard clips, N bases,
low base qualities, and CIGAR shapes the -k 1 rewrite changes (leading and
trailing insertions, close indels, a short block before a clip);
`paths_cigar_k1` hits each rule of the -k 1 CIGAR rewrite in turn;
`paths_q0` puts zero-quality bases before, between and after nonzero ones in
read order (the reference's order-dependent qstd rule).  `options_k0` /
`options_k1` run read sets with non-default values of every option the path
reads, and the remaining single-sample golden cases (dense germline sets
with -k 0 and -k 1, a contig end, -u --fisher, -t) run their own flags.  The
maps after the CIGAR walk (P) and after the realigner (R) must equal the
reference's dump, and the records its records: counts and keys exact,
fractional sums within 1e-9 relative.  The somatic golden cases (including
`somatic_options`, non-default somatic options) must give the reference's
63-column records."""
import gzip
import json
import os

import pytest

from cmp import diff_dump, diff_records, flag_params, widened

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
SINGLE = sorted(k for k, v in META.items() if not v.get("somatic") and not v.get("records_only"))
RECORDS_ONLY = sorted(k for k, v in META.items() if v.get("records_only"))
SOMATIC = sorted(k for k, v in META.items() if v.get("somatic"))
P_TAGS = ["P_ML", "PN", "PI", "PC", "PS5", "PS3", "PCI", "PCD", "PMN"]
R_TAGS = ["RN", "RI", "RC"]


def _make_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


@pytest.mark.parametrize("name", SINGLE)
def test_single_sample_golden_cases_match_reference(name):
    from rabbitvar_gb300 import api, synth
    mg = _make_golden()
    g, rs, (a, b), flags = mg.CASES[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"]
    ctx = api.Context(api.default_params(**flag_params(flags)))
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    ctx.submit(api.Batch.from_readset(rs), [widened(a, b, flags)])
    ctx.pileup()
    p_dump = ctx.export_maps(0, "P")
    ctx.realign()
    r_dump = ctx.export_maps(0, "R")
    ctx.score()
    mine = ctx.format_records("S", rs.contig)[0].splitlines()
    ctx.close()
    gold = gzip.open(os.path.join(GOLD, f"{name}.dump.txt.gz"), "rt").read()
    assert diff_dump(gold, p_dump, P_TAGS, rel=1e-9) == []
    assert diff_dump(gold, r_dump, R_TAGS, rel=1e-9) == []
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    assert len(recs) == META[name]["records"] > 5
    assert diff_records(recs, mine) == []


@pytest.mark.parametrize("name", RECORDS_ONLY)
def test_records_only_golden_cases_match_reference(name):
    """Records against the reference's: -k 1 at a contig end and on a dense
    multi-variant set, and pileup mode (-p: every covered position printed,
    alleles failing isGoodVar kept) with -k 0 and with -k 1 --fisher."""
    from rabbitvar_gb300 import api, synth
    mg = _make_golden()
    g, rs, (a, b), flags = mg.RECORDS_ONLY[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"]
    ctx = api.Context(api.default_params(**flag_params(flags)))
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    mine = ctx.call(api.Batch.from_readset(rs), [widened(a, b, flags)], "S", rs.contig).splitlines()
    ctx.close()
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    assert len(recs) == META[name]["records"] > 5
    assert diff_records(recs, mine) == []


@pytest.mark.parametrize("name", SOMATIC)
def test_somatic_golden_cases_match_reference(name):
    from rabbitvar_gb300 import api, synth
    mg = _make_golden()
    g, t, n, (a, b), flags = mg.SOMATIC[name]()
    assert [mg.readset_fingerprint(t), mg.readset_fingerprint(n)] == META[name]["fingerprint"]
    pair = api.SomaticPair(api.default_params(**flag_params(flags)))
    pair.upload_reference(t.contig, synth.genome_str(g).encode())
    mine = pair.call(api.Batch.from_readset(t), api.Batch.from_readset(n), [widened(a, b, flags)], "T", t.contig)
    pair.close()
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    assert len(recs) == META[name]["records"] > 50
    assert diff_records(recs, mine.splitlines(), somatic=True) == []
