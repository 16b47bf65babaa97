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
`paths_cigar_k1` hits each rule of the -k 1 CIGAR rewrite in turn.  The maps
after the CIGAR walk (P) and after the realigner (R) must equal the
reference's dump, and the records its records: counts and keys exact,
fractional sums within 1e-9 relative."""
import gzip
import json
import os

import pytest

from cmp import diff_dump, diff_records

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
P_TAGS = ["P_ML", "PN", "PI", "PC", "PS5", "PS3", "PCI", "PCD", "PMN"]
R_TAGS = ["RN", "RI", "RC"]


def _make_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


@pytest.mark.parametrize("name", ["paths_k0", "paths_k1", "paths_cigar_k1"])
def test_path_cases_match_reference_golden(name):
    from rabbitvar_gb300 import api, synth
    mg = _make_golden()
    g, rs, (a, b), flags = mg.CASES[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"]
    k = int(flags[flags.index("-k") + 1])
    ctx = api.Context(api.default_params(local_realign=k, fisher=1 if "--fisher" in flags else 0))
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    ctx.submit(api.Batch.from_readset(rs), [(a, b)])
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
