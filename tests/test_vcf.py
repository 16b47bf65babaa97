"""Somatic records to VCF (rabbitvar_gb300/vcf.py) against the reference's
own VCF writer run on the reference's golden somatic records
(tests/golden/somatic_mix.vcf, made by tests/golden/make_vcf_golden.py)."""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_vcf_matches_reference_writer():
    from rabbitvar_gb300 import vcf
    text = open(os.path.join(GOLD, "somatic_mix.records.txt")).read()
    want = open(os.path.join(GOLD, "somatic_mix.vcf")).read()
    got = vcf.write(text, "TUMOR")
    assert got == want
    assert sum(1 for l in got.splitlines() if not l.startswith("#")) == 55


def test_vcf_learned_scores_and_threshold():
    from rabbitvar_gb300 import vcf
    text = open(os.path.join(GOLD, "somatic_mix.records.txt")).read()
    n = len([l for l in text.splitlines() if l])
    scores = list(np.linspace(0.0, 1.0, n))
    got = vcf.write(text, "TUMOR", scores=scores, threshold=0.5)
    body = [l for l in got.splitlines() if not l.startswith("#")]
    assert 0 < len(body) < 55
    assert all(";RFV=" in l for l in body)
    assert all(float(l.split("RFV=")[1].split("\t")[0]) >= 0.5 for l in body)


def test_diff_vcf_tolerates_last_digit_only():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from cmp import diff_vcf
    want = open(os.path.join(GOLD, "somatic_mix.vcf")).read()
    lines = want.splitlines()
    i = next(j for j, l in enumerate(lines) if not l.startswith("#"))
    f = lines[i].split("\t")
    assert diff_vcf(want, want) == []
    # one unit in the sixth decimal of AF is tolerated, a changed depth is not
    af = f[7].split("AF=")[1].split(";")[0]
    near = lines[:i] + [lines[i].replace(f"AF={af}", f"AF={float(af) + 1e-6:.6f}", 1)] + lines[i + 1:]
    assert diff_vcf(want, "\n".join(near)) == []
    dp = f[7].split("DP=")[1].split(";")[0]
    far = lines[:i] + [lines[i].replace(f"DP={dp}", f"DP={int(dp) + 1}", 1)] + lines[i + 1:]
    assert diff_vcf(want, "\n".join(far)) != []
