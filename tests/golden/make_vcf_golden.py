"""Golden VCF for the somatic post-processing (rabbitvar_gb300/vcf.py).

Runs the reference's own VCF writer (utils/vcf_writer.py: write_header,
format_record) on the reference's golden somatic records
(tests/golden/somatic_mix.records.txt), typed as the reference's pandas
reader hands them to the writer (float32 columns as Python floats of float32
values, integer columns as Python ints, empty fields as NaN), after the hard
filter of utils/datautil.py:148-155 and the (Chr, Start) sort of
run_rabbitvar.py:239.  Needs the reference tree (this machine only); writes
tests/golden/somatic_mix.vcf.

    python tests/golden/make_vcf_golden.py
"""
import io
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = "/root/reference/utils"


class Row(list):
    """A record the way format_record indexes it: by position, and 'pred'."""

    def __init__(self, values, pred=None):
        super().__init__(values)
        self.pred = pred

    def __getitem__(self, k):
        if k == "pred":
            return self.pred
        return list.__getitem__(self, k)


def main():
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.dirname(HERE))
    import numpy as np
    import vcf_writer as W  # the reference's writer
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from rabbitvar_gb300 import vcf as V  # only for the column names and types
    text = open(os.path.join(HERE, "somatic_mix.records.txt")).read()
    rows = []
    for line in text.splitlines():
        f = line.split("\t")
        vals = []
        for i, c in enumerate(V.COLUMNS):
            t = f[i] if i < len(f) else ""
            if c in V._STR:
                vals.append(t if t != "" else math.nan)
            elif c in V._INT:
                vals.append(int(t) if t != "" else math.nan)
            else:
                vals.append(float(np.float32(float(t))) if t != "" else math.nan)
        rows.append(vals)
    ci = {c: i for i, c in enumerate(V.COLUMNS)}
    labels = {"Germline": 0, "StrongLOH": 1, "LikelyLOH": 2, "StrongSomatic": 3, "LikelySomatic": 4, "AFDiff": 5,
              "SampleSpecific": 6}
    types = {"SNV": 0, "Deletion": 1, "Insertion": 2, "Complex": 3, "MNV": 3}
    kept = []
    for i, r in enumerate(rows):
        af, qm, nm, lab = r[ci["Var1AF"]], r[ci["Var1QMean"]], r[ci["Var1NM"]], labels.get(r[ci["VarLabel"]])
        if af < 0.01 or qm <= 20 or nm >= 6 or nm < 0 or lab not in (3, 4, 5):
            continue
        r = list(r)
        r[ci["VarLabel"]] = lab
        r[ci["VarType"]] = types[r[ci["VarType"]]]
        kept.append((r[ci["Chr"]], r[ci["Start"]], i, r))
    kept.sort(key=lambda x: (x[0], x[1], x[2]))
    out = io.StringIO()
    W.write_header(out)
    out.write("\t".join(["#CHROM", "POS", "ID", "REF", "ALT", "QUAL", "FILTER", "INFO", "FORMAT", "TUMOR"]) + "\n")
    for _, _, _, r in kept:
        out.write(W.format_record(Row(r), True) + "\n")
    open(os.path.join(HERE, "somatic_mix.vcf"), "w").write(out.getvalue())
    print(f"{len(kept)} of {len(rows)} records written")


if __name__ == "__main__":
    main()
