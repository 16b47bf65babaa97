"""Regenerate the golden fixtures from the reference itself.

Requires oracle/_ref/ (the unmodified reference sources built against the
project's htslib-API shim by oracle/Makefile; needs the reference tree).
For each case: seeded synthetic reads -> BAM + FASTA in a temporary folder ->
the reference's per-region dump (rvref_dump: maps after CigarParser and
VariationRealigner, variants after ToVarsBuilder) and its emitted records
(the RabbitVar binary) -> gzipped text files next to this script, plus a
fingerprint of the generated reads so a change of the generator is reported
as such rather than as a parity failure.  The somatic cases (a tumor/normal
pair run in the reference's somatic mode) keep the emitted records only.

    python tests/golden/make_golden.py             # every case
    python tests/golden/make_golden.py paths_k0    # only the named cases
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

from rabbitvar_gb300 import synth  # noqa: E402


def case_germline_dense():
    rng = np.random.default_rng(0x60D0)
    g = synth.make_genome(6_000, rng, homopolymer_rate=0.02)
    vs = synth.plant_variants(g, rng, 5e-3, 1.5e-3, lambda r: r.choice([0.3, 0.5, 1.0]), mnv_frac=0.25,
                              margin=100, spacing=10)
    rs = synth.simulate(g, vs, 45.0, rng, softclip_frac=0.06, n_rate=1e-3, tail_margin=250)
    return g, rs, (1, 6_000), ["-k", "0"]


def case_contig_end():
    rng = np.random.default_rng(0x60D1)
    g = synth.make_genome(3_000, rng)
    vs = synth.plant_variants(g, rng, 6e-3, 1e-3, lambda r: 0.5, mnv_frac=0.3, margin=20, spacing=8)
    rs = synth.simulate(g, vs, 70.0, rng, softclip_frac=0.05)
    return g, rs, (1, 3_000), ["-k", "0"]


def case_unique_fisher():
    rng = np.random.default_rng(0x60D2)
    g = synth.make_genome(6_000, rng)
    vs = synth.plant_variants(g, rng, 4e-3, 1e-3, lambda r: r.uniform(0.1, 1.0), mnv_frac=0.2, margin=100)
    rs = synth.simulate(g, vs, 60.0, rng, softclip_frac=0.04, tail_margin=250)
    return g, rs, (1_501, 4_500), ["-k", "0", "-u", "--fisher"]


def case_dedup():
    # reads starting in 2000..4000 get mate position 4 (so -t considers them)
    # and two exact copies each
    g, _, rs = synth.dense_multi(seed=0x5EED00D2, length=8_000)
    idx = []
    for i in range(rs.n):
        idx.append(i)
        if 2000 <= rs.pos[i] < 4000:
            idx += [i, i]
    rs2 = synth.take(rs, np.array(idx))
    rs2.mpos[(rs2.pos >= 2000) & (rs2.pos < 4000)] = 4
    return g, rs2, (1_801, 4_200), ["-k", "0", "-t"]


def case_germline_dense_k1():
    # local realignment (-k 1, the reference's default): CIGAR rewrite and indel realigner
    g, rs, region, _ = case_germline_dense()
    return g, rs, region, ["-k", "1"]


def _path_reads():
    """Hand-written reads over an 8 kb contig, one locus per pileup code path,
    on a background of reference reads (depth ~12, both strands).  Every read
    set below would change the maps or records if its path were handled
    differently: MNV growth and its quality stop (parseCigar.cpp:711-767),
    deletions and their flank-quality rule (:1525-1727), insertions shifted
    3' in a homopolymer and after a leading soft clip (:1303-1523), soft
    clips that match the reference and ones with low-quality stops
    (:1112-1301), mismatches next to indels (complex tails, :779-882),
    record filters (recordPreprocessor.cpp:101-180; parseCigar.cpp:517-606),
    hard clips, N bases and low base/mapping qualities."""
    rng = np.random.default_rng(0x60D7)
    g = synth.make_genome(8_000, rng)
    g[1_500:1_508] = 0  # an A homopolymer for the insertion shift
    other = lambda p: "ACGT"[(int(g[p]) + 1) % 4]  # noqa: E731
    reads = [{"pos": p, "segs": [("M", 150)], "rev": (p // 12) % 2 == 1} for p in range(0, 8_000 - 150, 12)]

    def add(starts, segs_of, **kw):
        for j, p in enumerate(starts):
            reads.append(dict(pos=p, segs=segs_of(p), rev=j % 2 == 1, **kw))

    # MNV: two adjacent mismatches, a gap of one matching base, a low-quality second base
    add([440, 455, 470, 480], lambda p: [("M", 150, {500 - p: other(500), 501 - p: other(501)})])
    add([540, 560, 575], lambda p: [("M", 150, {600 - p: other(600), 602 - p: other(602)})])
    for p in (640, 655, 670):
        reads.append({"pos": p, "segs": [("M", 150, {700 - p: other(700), 701 - p: other(701)})],
                      "qual_at": {701 - p: 14}})
    # deletion with unequal flank qualities; a longer deletion
    for j, p in enumerate((940, 950, 965, 975)):
        reads.append({"pos": p, "segs": [("M", 1000 - p), ("D", 3), ("M", 150 - (1000 - p))],
                      "qual_at": {1000 - p - 1: 20 + 5 * j}, "rev": j % 2 == 0})
    add([1040, 1062], lambda p: [("M", 1100 - p), ("D", 9), ("M", 150 - (1100 - p))])
    # insertion inside the homopolymer (shifted 3'); insertion after a leading soft clip
    add([1440, 1452, 1466], lambda p: [("M", 1503 - p), ("I", "A"), ("M", 149 - (1503 - p))])
    add([1700, 1700], lambda p: [("S", 5), ("I", "GT"), ("M", 143)])
    # soft clips: matching the reference (3' and 5'), foreign bases with low-quality stops
    add([1900, 1910, 1920], lambda p: [("M", 2000 - p), ("S", 150 - (2000 - p))])
    add([2050, 2060], lambda p: [("S", 25), ("M", 125)])
    for p in (2150, 2160, 2170):
        clip = "".join(other(2250 + k) for k in range(30))
        reads.append({"pos": p, "segs": [("M", 2250 - p), ("S", clip)],
                      "qual_at": {2250 - p + 4: 11, 2250 - p + 9: 8}})
    # mismatch two bases before a deletion; mismatch just after an insertion
    add([2440, 2455, 2470], lambda p: [("M", 2500 - p, {2498 - p: other(2498)}), ("D", 2),
                                       ("M", 148 - (2500 - p))])
    add([2640, 2652, 2664], lambda p: [("M", 2700 - p), ("I", "GT"),
                                       ("M", 148 - (2700 - p), {1: other(2701)})])
    # record filters: flags 0x4/0x100/0x400/0x800, a one-base read, too many mismatches,
    # both ends clipped >= 10; each would add an SNV at 3000 if it were counted
    snv = lambda p: {3000 - p: other(3000)}  # noqa: E731
    for f in (0x4 | 0x1, 0x100 | 0x1, 0x400 | 0x1, 0x800 | 0x1):
        reads.append({"pos": 2950, "segs": [("M", 150, snv(2950))], "flag": f})
    reads.append({"pos": 2999, "segs": [("M", 1)]})
    reads.append({"pos": 2940, "segs": [("M", 150, {**snv(2940), **{k: other(2940 + k) for k in range(20, 29)}})]})
    reads.append({"pos": 2930, "segs": [("S", 12), ("M", 126, snv(2930 + 12)), ("S", 12)]})
    # counted: MAPQ 0, a hard clip, an N base, low base quality (below goodq)
    add([3140, 3150], lambda p: [("M", 150, {3200 - p: other(3200)})], mapq=0)
    add([3160, 3170], lambda p: [("H", 10), ("M", 140, {3200 - p: other(3200)})])
    add([3340, 3350, 3360], lambda p: [("M", 150, {3400 - p: "N"})])
    for p in (3540, 3550, 3560):
        reads.append({"pos": p, "segs": [("M", 150, {3600 - p: other(3600)})], "qual_at": {3600 - p: 15}})
    # CIGAR shapes the -k 1 rewrite acts on: leading/trailing insertion, close indels,
    # a short match block before a soft clip
    add([3800, 3810], lambda p: [("I", "TT"), ("M", 148)])
    add([3900, 3910], lambda p: [("M", 148), ("I", "CC")])
    add([4040, 4052, 4064], lambda p: [("M", 4100 - p), ("D", 2), ("M", 4), ("I", "GA"), ("M", 144 - (4100 - p))])
    add([4240, 4250], lambda p: [("M", 4300 - p), ("D", 1), ("M", 3), ("S", 150 - (4300 - p) - 3)])
    return g, synth.explicit_reads("ctg", g, reads)


def case_paths_k0():
    g, rs = _path_reads()
    return g, rs, (1, 8_000), ["-k", "0", "--fisher"]


def case_paths_k1():
    g, rs = _path_reads()
    return g, rs, (1, 8_000), ["-k", "1"]


def _cigar_rule_reads():
    """Hand-written reads whose CIGARs hit each rule of the -k 1 CIGAR rewrite
    (cigarModifier.cpp:219-380, patterns include/patterns.h:52-122), three
    copies per shape (two strands) on a background of reference reads: a clip
    followed by an indel at either end, a short match block between a clip and
    an indel, a 1-9 base match block before/after an indel at either end, three
    close deletions, three close indels, insertion-match-deletion, adjacent
    deletions, adjacent insertions, and mismatches next to a clip or at the
    read ends (the rules applied after the loop)."""
    rng = np.random.default_rng(0x60D8)
    g = synth.make_genome(8_000, rng)
    other = lambda p: "ACGT"[(int(g[p]) + 1) % 4]  # noqa: E731
    reads = [{"pos": p, "segs": [("M", 150)], "rev": (p // 12) % 2 == 1} for p in range(0, 8_000 - 150, 12)]
    shapes = [
        lambda p: [("S", 10), ("I", "GTA"), ("M", 137)],
        lambda p: [("S", 10), ("D", 3), ("M", 140)],
        lambda p: [("M", 137), ("I", "CAG"), ("S", 10)],
        lambda p: [("M", 140), ("D", 3), ("S", 10)],
        lambda p: [("S", 10), ("M", 8), ("I", "TG"), ("M", 130)],
        lambda p: [("S", 10), ("M", 8), ("D", 2), ("M", 132)],
        lambda p: [("M", 130), ("I", "TG"), ("M", 8), ("S", 10)],
        lambda p: [("M", 5), ("D", 2), ("M", 145)],
        lambda p: [("M", 5), ("I", "AC"), ("M", 143)],
        lambda p: [("M", 143), ("I", "AC"), ("M", 5)],
        lambda p: [("M", 145), ("D", 2), ("M", 5)],
        lambda p: [("M", 50), ("D", 2), ("M", 3), ("D", 2), ("M", 3), ("D", 2), ("M", 94)],
        lambda p: [("M", 50), ("D", 2), ("M", 3), ("I", "TT"), ("M", 3), ("D", 1), ("M", 92)],
        lambda p: [("M", 60), ("I", "GG"), ("M", 4), ("D", 3), ("M", 84)],
        lambda p: [("M", 60), ("D", 2), ("D", 3), ("M", 90)],
        lambda p: [("M", 60), ("I", "AC"), ("I", "GTA"), ("M", 85)],
        lambda p: [("M", 140, {137: other(p + 137), 138: other(p + 138)}), ("S", 10)],
        lambda p: [("S", 10), ("M", 140, {2: other(p + 2), 3: other(p + 3)})],
        lambda p: [("M", 150, {1: other(p + 1), 2: other(p + 2)})],
        lambda p: [("M", 150, {146: other(p + 146), 148: other(p + 148)})],
    ]
    for k, shape in enumerate(shapes):
        base = 200 + 370 * k
        for j in range(3):
            reads.append({"pos": base, "segs": shape(base), "rev": j == 1})
    return g, synth.explicit_reads("ctg", g, reads)


def case_paths_cigar_k1():
    g, rs = _cigar_rule_reads()
    return g, rs, (1, 8_000), ["-k", "1"]


def case_paths_q0():
    """Zero-quality bases at variant sites (the order-dependent pstd/qstd rule,
    parseCigar.cpp:902-914): three carrying reads per site with base
    qualities, in read order, 37/0/37, 0/37/37, 37/37/0, 0/0/37, 0/37/0 and
    0/0/0.  The oracle replays the
    rule in read order; the GPU path's order-free form differs where a Q0
    base follows a nonzero one (not used by the GPU tests)."""
    rng = np.random.default_rng(0x60D9)
    g = synth.make_genome(3_000, rng)
    other = lambda p: "ACGT"[(int(g[p]) + 1) % 4]  # noqa: E731
    reads = [{"pos": p, "segs": [("M", 150)], "rev": (p // 12) % 2 == 1} for p in range(0, 3_000 - 150, 12)]
    sites = ((400, (37, 0, 37)), (800, (0, 37, 37)), (1200, (37, 37, 0)), (1600, (0, 0, 37)), (2000, (0, 37, 0)),
             (2400, (0, 0, 0)))
    for site, quals in sites:
        for j, q in enumerate(quals):  # read order = j
            p = site - 80 + 10 * j
            reads.append({"pos": p, "segs": [("M", 150, {site - p: other(site)})], "qual_at": {site - p: q},
                          "rev": j == 1})
    rs = synth.explicit_reads("ctg", g, reads)
    return g, rs, (1, 3_000), ["-k", "0", "-q", "0", "-P", "0"]


def case_options_k0():
    # non-default values of the options the path reads (-x widens the -R region on both sides)
    g, rs, region, _ = case_unique_fisher()
    return g, rs, region, ["-k", "0", "-x", "30", "-T", "120", "-P", "10", "-3", "-O", "20", "-B", "4", "-o", "2",
                           "-q", "25", "-m", "6", "-r", "3", "-X", "3", "--fisher"]


def case_options_k1():
    g, rs, region, _ = case_germline_dense()
    return g, rs, region, ["-k", "1", "--UN", "-M", "20", "-Q", "10", "-Y", "600", "-f", "0.05"]


CASES = {"germline_dense": case_germline_dense, "contig_end": case_contig_end, "unique_fisher": case_unique_fisher,
         "dedup": case_dedup, "germline_dense_k1": case_germline_dense_k1, "paths_k0": case_paths_k0,
         "paths_k1": case_paths_k1, "paths_cigar_k1": case_paths_cigar_k1, "paths_q0": case_paths_q0, "options_k0": case_options_k0,
         "options_k1": case_options_k1}


# records only
def case_contig_end_k1():
    g, rs, region, _ = case_contig_end()
    return g, rs, region, ["-k", "1"]


def case_dense_multi_k1():
    g, _, rs = synth.dense_multi()
    return g, rs, (1, 30_000), ["-k", "1", "--fisher"]


def case_pileup_k0():
    # pileup mode (-p): every covered position printed, failing variants kept
    g, rs, _, _ = case_germline_dense()
    return g, rs, (1_001, 2_500), ["-k", "0", "-p"]


def case_pileup_k1():
    g, _, rs = synth.dense_multi()
    return g, rs, (2_001, 4_000), ["-k", "1", "-p", "--fisher"]


RECORDS_ONLY = {"contig_end_k1": case_contig_end_k1, "dense_multi_k1": case_dense_multi_k1,
                "pileup_k0": case_pileup_k0, "pileup_k1": case_pileup_k1}


# somatic mode (`-b 'T.bam|N.bam' -N 'T|N'`): records only
def case_somatic_mix():
    g, _, t, n = synth.somatic_mix(0x5EED0051)
    return g, t, n, (1, g.shape[0]), ["-k", "0", "--fisher"]


def case_somatic_sub():
    g, _, t, n = synth.somatic_mix(0x5EED0052)
    return g, t, n, (8_001, 20_000), ["-k", "0"]


def case_somatic_mix_k1():
    g, _, t, n = synth.somatic_mix(0x5EED0051)
    return g, t, n, (1, g.shape[0]), ["-k", "1", "--fisher"]


def case_somatic_options():
    # somatic mode with non-default thresholds, -V (lofreq) included
    g, _, t, n = synth.somatic_mix(0x5EED0053)
    return g, t, n, (1, g.shape[0]), ["-k", "0", "--fisher", "-V", "0.1", "-f", "0.02", "-r", "3", "-q", "25",
                                      "-B", "3", "-o", "2", "-P", "8", "-O", "10", "-3"]


SOMATIC = {"somatic_mix": case_somatic_mix, "somatic_options": case_somatic_options, "somatic_sub": case_somatic_sub, "somatic_mix_k1": case_somatic_mix_k1}


def readset_fingerprint(rs) -> str:
    h = hashlib.sha256()
    for a in (rs.pos, rs.flag, rs.mapq, rs.mpos, rs.nm, rs.n_cigar, rs.cigar, rs.l_qseq, rs.seq4, rs.qual):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main(only=()):
    """Regenerate every case, or only the named ones (their golden.json
    entries are replaced, the others kept)."""
    import oracle as O
    if not O.have_reference():
        raise SystemExit("oracle/_ref is not built (needs the reference tree): make -C oracle ref")
    meta = {}
    if only:
        with open(os.path.join(HERE, "golden.json")) as f:
            meta = json.load(f)
    pick = lambda d: {k: v for k, v in d.items() if not only or k in only}  # noqa: E731
    for name, fn in pick(CASES).items():
        g, rs, (a, b), flags = fn()
        with tempfile.TemporaryDirectory() as td:
            bam = os.path.join(td, "s.bam")
            fa = os.path.join(td, "ref.fa")
            synth.write_bam(bam, rs)
            synth.write_fasta(fa, rs.contig, g)
            region = f"{rs.contig}:{a}-{b}"
            dump_flags = [f for f in flags if f != "--fisher"]
            dump = O.reference_dump(fa, bam, region, dump_flags, stages="PRV")
            recs = O.reference_records(fa, bam, region, os.path.join(td, "out.txt"), flags)
        # mtime 0: the same dump gives the same bytes
        with gzip.GzipFile(os.path.join(HERE, f"{name}.dump.txt.gz"), "wb", mtime=0) as f:
            f.write(dump.encode())
        with open(os.path.join(HERE, f"{name}.records.txt"), "w") as f:
            f.write("\n".join(sorted(recs)) + "\n")
        meta[name] = {"region": [a, b], "flags": flags, "reads": rs.n, "fingerprint": readset_fingerprint(rs),
                      "records": len(recs)}
        print(name, rs.n, "reads", len(recs), "records")
    for name, fn in pick(RECORDS_ONLY).items():
        g, rs, (a, b), flags = fn()
        with tempfile.TemporaryDirectory() as td:
            bam = os.path.join(td, "s.bam")
            fa = os.path.join(td, "ref.fa")
            synth.write_bam(bam, rs)
            synth.write_fasta(fa, rs.contig, g)
            recs = O.reference_records(fa, bam, f"{rs.contig}:{a}-{b}", os.path.join(td, "out.txt"), flags)
        with open(os.path.join(HERE, f"{name}.records.txt"), "w") as f:
            f.write("\n".join(sorted(recs)) + "\n")
        meta[name] = {"records_only": True, "region": [a, b], "flags": flags, "reads": rs.n,
                      "fingerprint": readset_fingerprint(rs), "records": len(recs)}
        print(name, rs.n, "reads", len(recs), "records")
    for name, fn in pick(SOMATIC).items():
        g, t, n, (a, b), flags = fn()
        with tempfile.TemporaryDirectory() as td:
            tb, nb, fa = (os.path.join(td, x) for x in ("T.bam", "N.bam", "ref.fa"))
            synth.write_bam(tb, t)
            synth.write_bam(nb, n)
            synth.write_fasta(fa, t.contig, g)
            recs = O.reference_records(fa, f"{tb}|{nb}", f"{t.contig}:{a}-{b}", os.path.join(td, "out.txt"), flags,
                                       sample="T|N")
        with open(os.path.join(HERE, f"{name}.records.txt"), "w") as f:
            f.write("\n".join(sorted(recs)) + "\n")
        meta[name] = {"somatic": True, "region": [a, b], "flags": flags, "reads": [t.n, n.n],
                      "fingerprint": [readset_fingerprint(t), readset_fingerprint(n)], "records": len(recs)}
        print(name, t.n, n.n, "reads", len(recs), "records")
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
