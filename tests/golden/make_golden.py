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

    python tests/golden/make_golden.py
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


CASES = {"germline_dense": case_germline_dense, "contig_end": case_contig_end, "unique_fisher": case_unique_fisher,
         "dedup": case_dedup, "germline_dense_k1": case_germline_dense_k1}


# records only
def case_contig_end_k1():
    g, rs, region, _ = case_contig_end()
    return g, rs, region, ["-k", "1"]


def case_dense_multi_k1():
    g, _, rs = synth.dense_multi()
    return g, rs, (1, 30_000), ["-k", "1", "--fisher"]


RECORDS_ONLY = {"contig_end_k1": case_contig_end_k1, "dense_multi_k1": case_dense_multi_k1}


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


SOMATIC = {"somatic_mix": case_somatic_mix, "somatic_sub": case_somatic_sub, "somatic_mix_k1": case_somatic_mix_k1}


def readset_fingerprint(rs) -> str:
    h = hashlib.sha256()
    for a in (rs.pos, rs.flag, rs.mapq, rs.mpos, rs.nm, rs.n_cigar, rs.cigar, rs.l_qseq, rs.seq4, rs.qual):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    import oracle as O
    if not O.have_reference():
        raise SystemExit("oracle/_ref is not built (needs the reference tree): make -C oracle ref")
    meta = {}
    for name, fn in CASES.items():
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
    for name, fn in RECORDS_ONLY.items():
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
    for name, fn in SOMATIC.items():
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
    main()
