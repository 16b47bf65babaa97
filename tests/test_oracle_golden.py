"""The oracle (CPU restatement) against golden outputs of the reference.

The golden files under tests/golden/ were produced by the reference itself
(its unmodified sources built here against the project's htslib-API shim;
tests/golden/make_golden.py).  The oracle must reproduce every map entry
after the CIGAR walk (P), after the realigner (R), every per-site variant (V)
and every emitted record, exactly (doubles to 1e-12 relative).
"""
import gzip
import json
import os

import pytest

from cmp import diff_dump, diff_records, flag_params, widened

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
SINGLE = sorted(k for k, v in META.items() if not v.get("somatic") and not v.get("records_only"))
RECORDS_ONLY = sorted(k for k, v in META.items() if v.get("records_only"))
SOMATIC = sorted(k for k, v in META.items() if v.get("somatic"))

P_TAGS = ["P_ML", "PN", "PI", "PC", "PS5", "PS3", "PCI", "PCD", "PMN"]
R_TAGS = ["RN", "RI", "RC"]


def _params(flags):
    import oracle as O
    return O.default_params(**flag_params(flags))


_widened = widened


def _make_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


@pytest.mark.parametrize("name", SINGLE)
def test_oracle_matches_reference_golden(name):
    import oracle as O
    mg = _make_golden()
    g, rs, (a, b), flags = mg.CASES[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"], "synthetic generator drifted: rerun make_golden.py"
    gold = gzip.open(os.path.join(GOLD, f"{name}.dump.txt.gz"), "rt").read()
    ora = O.run_region(rs, g, *_widened(a, b, flags), stages="PRVO", params=_params(flags))
    # pp/pq (last-seen read position/quality) are compared too: the oracle is sequential
    assert diff_dump(gold, ora, P_TAGS, skip=(), rel=1e-12) == []
    assert diff_dump(gold, ora, R_TAGS, skip=(), rel=1e-12) == []
    assert diff_dump(gold, ora, ["V"], skip=(), rel=1e-12, key_cols=3) == []
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    mine = [l for l in ora.splitlines() if l.startswith("S\t")]
    assert len(recs) == META[name]["records"] > 5
    assert diff_records(recs, mine, rel=0) == []


def test_oracle_matches_reference_binary_config0(tmp_path):
    """Against the reference binary itself when it was built here (the
    reference tree is not present on GPU hosts)."""
    import oracle as O
    if not O.have_reference():
        pytest.skip("reference binaries not built (reference tree absent)")
    from rabbitvar_gb300 import synth
    g, vs, rs = synth.germline_small()
    bam, fa = str(tmp_path / "s.bam"), str(tmp_path / "ref.fa")
    synth.write_bam(bam, rs)
    synth.write_fasta(fa, rs.contig, g)
    ref = O.reference_dump(fa, bam, "ctg:1-100000", ["-k", "0"], stages="PV")
    ora = O.run_region(rs, g, 1, 100000, stages="PVO", params=O.default_params(local_realign=0))
    assert diff_dump(ref, ora, P_TAGS, skip=(), rel=1e-12) == []
    assert diff_dump(ref, ora, ["V"], skip=(), rel=1e-12, key_cols=3) == []
    recs = O.reference_records(fa, bam, "ctg:1-100000", str(tmp_path / "o.txt"), ["-k", "0"])
    assert diff_records(recs, [l for l in ora.splitlines() if l.startswith("S\t")], rel=0) == []


@pytest.mark.parametrize("name", SOMATIC)
def test_oracle_somatic_matches_reference_golden(name):
    """Somatic mode: every one of the 63-column records (labels StrongSomatic,
    LikelySomatic, Germline, AFDiff, LikelyLOH, StrongLOH, SampleSpecific),
    byte for byte."""
    import oracle as O
    mg = _make_golden()
    g, t, n, (a, b), flags = mg.SOMATIC[name]()
    assert [mg.readset_fingerprint(t), mg.readset_fingerprint(n)] == META[name]["fingerprint"], \
        "synthetic generator drifted: rerun make_golden.py"
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    mine = O.run_somatic(t, n, g, a, b, "O", "T", _params(flags)).splitlines()
    assert len(recs) == META[name]["records"] > 50
    assert sorted(mine) == sorted(recs)
    if name == "somatic_mix":
        labels = {r.split("\t")[53] for r in recs}
        assert labels >= {"StrongSomatic", "LikelySomatic", "Germline", "AFDiff", "LikelyLOH", "StrongLOH",
                          "SampleSpecific"}


@pytest.mark.parametrize("name", RECORDS_ONLY)
def test_oracle_records_match_reference_golden(name):
    import oracle as O
    mg = _make_golden()
    g, rs, (a, b), flags = mg.RECORDS_ONLY[name]()
    assert mg.readset_fingerprint(rs) == META[name]["fingerprint"], "synthetic generator drifted: rerun make_golden.py"
    recs = open(os.path.join(GOLD, f"{name}.records.txt")).read().splitlines()
    ora = O.run_region(rs, g, *_widened(a, b, flags), stages="O", params=_params(flags))
    assert len(recs) == META[name]["records"] > 5
    assert diff_records(recs, ora.splitlines(), rel=0) == []


def test_oracle_somatic_matches_reference_binary_bench_shape(tmp_path):
    """The somatic pair at the bench workload's depths (tumor 200x, normal
    100x, 2x150) on a 100 kb contig, -k 1 --fisher: the oracle's records equal
    the reference binary's, byte for byte.  The bench's CPU baseline times the
    oracle, so this pins it on that shape."""
    import oracle as O
    if not O.have_reference():
        pytest.skip("reference binaries not built (reference tree absent)")
    from rabbitvar_gb300 import synth
    g, _, t, n = synth.somatic_pair(length=100_000)
    tb, nb, fa = str(tmp_path / "T.bam"), str(tmp_path / "N.bam"), str(tmp_path / "ref.fa")
    synth.write_bam(tb, t)
    synth.write_bam(nb, n)
    synth.write_fasta(fa, t.contig, g)
    recs = O.reference_records(fa, f"{tb}|{nb}", f"{t.contig}:1-100000", str(tmp_path / "o.txt"),
                               ["-k", "1", "--fisher"], sample="T|N")
    mine = O.run_somatic(t, n, g, 1, 100_000, "O", "T", O.default_params(local_realign=1, fisher=1)).splitlines()
    assert len(recs) > 100
    assert sorted(mine) == sorted(recs)


def test_oracle_somatic_matches_reference_binary_deep_panel(tmp_path):
    """One region of the deep targeted panel (5 kb, tumor 5000x + normal
    1000x, low-VAF somatic variants, C>A artifacts at Q20), -k 1 --fisher:
    the oracle's records equal the reference binary's byte for byte, so the
    oracle is pinned on the panel the GPU parity test and the bench use."""
    import oracle as O
    if not O.have_reference():
        pytest.skip("reference binaries not built (reference tree absent)")
    from rabbitvar_gb300 import synth
    g, _, t, n, regions = synth.deep_somatic_panel(only=[137])
    t, n = synth.unpacked(t), synth.unpacked(n)
    a, b = regions[137]
    tb, nb, fa = str(tmp_path / "T.bam"), str(tmp_path / "N.bam"), str(tmp_path / "ref.fa")
    synth.write_bam(tb, t)
    synth.write_bam(nb, n)
    synth.write_fasta(fa, t.contig, g)
    recs = O.reference_records(fa, f"{tb}|{nb}", f"{t.contig}:{a}-{b}", str(tmp_path / "o.txt"),
                               ["-k", "1", "--fisher"], sample="T|N")
    mine = O.run_somatic(t, n, g, a, b, "O", "T", O.default_params(local_realign=1, fisher=1)).splitlines()
    assert len(recs) >= 3
    assert sorted(mine) == sorted(recs)
