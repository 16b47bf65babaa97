"""VCF output of somatic records: the reference's post-processing of its
63-column somatic text (run_rabbitvar.py:110-166 rf_filter, whose hard
filter is utils/datautil.py:148-155; utils/vcf_writer.py write_header and
format_record; run_rabbitvar.py:228-249, which sorts by contig and start and
writes), with the learned filter's probability in place of the random
forest's (the RFV field).

The reference reads the text with pandas and these column types
(utils/datautil.py:109-126): float32 columns reach the formatter as Python
floats holding float32-rounded values, integer columns as Python ints; the
same conversions are applied here.
"""
from __future__ import annotations

import math
import re

import numpy as np

# the 63 columns of a somatic record, and the reader's types
COLUMNS = (
    "Sample Gene Chr Start End Ref Alt "
    "Var1Depth Var1AltDepth Var1RefFwdReads Var1RefRevReads Var1AltFwdReads Var1AltRevReads Var1Genotype Var1AF "
    "Var1Bias Var1PMean Var1PStd Var1QMean Var1QStd Var1MQ Var1Sig_Noise Var1HiAF Var1ExtraAF Var1NM Var1Pvalue "
    "Var1Oddr Var2Depth Var2AltDepth Var2RefFwdReads Var2RefRevReads Var2AltFwdReads Var2AltRevReads Var2Genotype "
    "Var2AF Var2Bias Var2PMean Var2PStd Var2QMean Var2QStd Var2MQ Var2Sig_Noise Var2HiAF Var2ExtraAF Var2NM "
    "Var2Pvalue Var2Oddr shift3 MSI MSI_NT 5pFlankSeq 3pFlankSeq Seg VarLabel VarType Duprate1 SV_info1 Duprate2 "
    "SV_info2 Pvalue Oddratio TumorNormalAllelLogOdds TumorNormalindelAltLogOdd").split()
_STR = {"Sample", "Gene", "Chr", "Ref", "Alt", "Var1Genotype", "Var1Bias", "Var2Genotype", "Var2Bias", "5pFlankSeq",
        "3pFlankSeq", "Seg", "VarLabel", "VarType"}
_INT = {"Start", "End", "Var1Depth", "Var1AltDepth", "Var1RefFwdReads", "Var1RefRevReads", "Var1AltFwdReads",
        "Var1AltRevReads", "Var1PStd", "Var1QStd", "Var2Depth", "Var2AltDepth", "Var2RefFwdReads", "Var2RefRevReads",
        "Var2AltFwdReads", "Var2AltRevReads", "Var2PStd", "Var2QStd", "shift3", "MSI_NT", "SV_info1", "SV_info2"}

# status labels and variant types (run_rabbitvar.py:26-30, utils/Global.py:9-24)
LABELS = ("Germline", "StrongLOH", "LikelyLOH", "StrongSomatic", "LikelySomatic", "AFDiff", "SampleSpecific")
TYPE_NAMES = {"SNV": "SNV", "Deletion": "Deletion", "Insertion": "Insertion", "Complex": "Complex", "MNV": "Complex"}

FORMAT_KEYS = "GT:DP:VD:ALD:RD:AD:AF:BIAS:PMEAN:PSTD:QUAL:QSTD:SBF:ODDRATIO:MQ:SN:HIAF:ADJAF:NM"

_HEADER_INFO = [
    ("SAMPLE", "1", "String", "Sample name (with whitespace translated to underscores)"),
    ("TYPE", "1", "String", "Variant Type: SNV Insertion Deletion Complex"),
    ("DP", "1", "Integer", "Total Depth"),
    ("END", "1", "Integer", "Chr End Position"),
    ("VD", "1", "Integer", "Variant Depth"),
    ("AF", "A", "Float", "Allele Frequency"),
    ("BIAS", "1", "String", "Strand Bias Info"),
    ("REFBIAS", "1", "String", "Reference depth by strand"),
    ("VARBIAS", "1", "String", "Variant depth by strand"),
    ("PMEAN", "1", "Float", "Mean position in reads"),
    ("PSTD", "1", "Float", "Position STD in reads"),
    ("QUAL", "1", "Float", "Mean quality score in reads"),
    ("QSTD", "1", "Float", "Quality score STD in reads"),
    ("SBF", "1", "Float", "Strand Bias Fisher p-value"),
    ("ODDRATIO", "1", "Float", "Strand Bias Odds ratio"),
    ("MQ", "1", "Float", "Mean Mapping Quality"),
    ("SN", "1", "Float", "Signal to noise"),
    ("HIAF", "1", "Float", "Allele frequency using only high quality bases"),
    ("ADJAF", "1", "Float", "Adjusted AF for indels due to local realignment"),
    ("SHIFT3", "1", "Integer", "No. of bases to be shifted to 3 prime for deletions due to alternative alignment"),
    ("MSI", "1", "Float", "MicroSatellite. > 1 indicates MSI"),
    ("MSILEN", "1", "Float", "MicroSatellite unit length in bp"),
    ("NM", "1", "Float", "Mean mismatches in reads"),
    ("LSEQ", "1", "String", "5' flanking seq"),
    ("RSEQ", "1", "String", "3' flanking seq"),
    ("GDAMP", "1", "Integer", "No. of amplicons supporting variant"),
    ("TLAMP", "1", "Integer", "Total of amplicons covering variant"),
    ("NCAMP", "1", "Integer", "No. of amplicons don't work"),
    ("AMPFLAG", "1", "Integer", "Top variant in amplicons don't match"),
    ("HICNT", "1", "Integer", "High quality variant reads"),
    ("HICOV", "1", "Integer", "High quality total reads"),
    ("SPLITREAD", "1", "Integer", "No. of split reads supporting SV"),
    ("SPANPAIR", "1", "Integer", "No. of pairs supporting SV"),
    ("DUPRATE", "1", "Float", "Duplication rate in fraction"),
]
_HEADER_FORMAT = [
    ("GT", "1", "String", "Genotype"),
    ("DP", "1", "Integer", "Total Depth"),
    ("VD", "1", "Integer", "Variant Depth"),
    ("AD", "R", "Integer", "Allelic depths for the ref and alt alleles in the order listed"),
    ("AF", "A", "Float", "Allele Frequency"),
    ("RD", "2", "Integer", "Reference forward, reverse reads"),
    ("ALD", "2", "Integer", "Variant forward, reverse reads"),
]


def header(sample_name: str) -> str:
    """The meta lines and the column line (utils/vcf_writer.py:8-57 and
    run_rabbitvar.py:241-244)."""
    out = ["##fileformat=VCFv4.3"]
    out += [f'##INFO=<ID={i},Number={n},Type={t},Description="{d}">' for i, n, t, d in _HEADER_INFO]
    out.append('##FILTER=<ID=Bias,Description="Strand Bias">')
    out += [f'##FORMAT=<ID={i},Number={n},Type={t},Description="{d}">' for i, n, t, d in _HEADER_FORMAT]
    out.append("\t".join(["#CHROM", "POS", "ID", "REF", "ALT", "QUAL", "FILTER", "INFO", "FORMAT", sample_name]))
    return "\n".join(out) + "\n"


def _value(name: str, text: str):
    if name in _STR:
        return text if text != "" else math.nan  # the reader's na_values = ['']
    if text == "":
        return None
    if name in _INT:
        return int(text)
    return float(np.float32(float(text)))


def parse(text: str) -> list[dict]:
    """Typed records of the somatic text (one dict per line)."""
    out = []
    for line in text.splitlines():
        if not line:
            continue
        f = line.split("\t")
        out.append({c: _value(c, f[i] if i < len(f) else "") for i, c in enumerate(COLUMNS)})
    return out


def hard_filter(records: list[dict]) -> list[dict]:
    """Kept records: AF >= 0.01, mean quality > 20, 0 <= NM < 6 and a somatic
    label (utils/datautil.py:148-155)."""
    keep = []
    for r in records:
        af, qm, nm = r["Var1AF"], r["Var1QMean"], r["Var1NM"]
        if af is None or qm is None or nm is None:
            continue
        if af < 0.01 or qm <= 20 or nm >= 6 or nm < 0:
            continue
        if r["VarLabel"] not in ("StrongSomatic", "LikelySomatic", "AFDiff"):
            continue
        keep.append(r)
    return keep


def _genotype(af: float) -> str:
    return "1/1" if 1 - af < 0.2 else ("1/0" if af >= 0.5 else ("0/1" if af >= 0.02 else "0/0"))


def _bias(b) -> str:
    b = str(b).replace(";", ",")
    return "0,0" if b == "0" else b


def _sample_fields(r: dict, s: str) -> str:
    af = r[f"Var{s}AF"]
    rd = r[f"Var{s}RefFwdReads"] + r[f"Var{s}RefRevReads"]
    vd = r[f"Var{s}AltDepth"]
    return ":".join([
        _genotype(af), str(r[f"Var{s}Depth"]), str(vd),
        f"{r[f'Var{s}AltFwdReads']},{r[f'Var{s}AltRevReads']}",
        f"{r[f'Var{s}RefFwdReads']},{r[f'Var{s}RefRevReads']}",
        f"{rd},{vd}", f"{af:.6f}", _bias(r[f"Var{s}Bias"]), str(r[f"Var{s}PMean"]), str(r[f"Var{s}PStd"]),
        str(r[f"Var{s}QMean"]), str(r[f"Var{s}QStd"]), str(r[f"Var{s}Pvalue"]), str(r[f"Var{s}Oddr"]),
        f"{r[f'Var{s}MQ']:.0}", str(r[f"Var{s}Sig_Noise"]), f"{r[f'Var{s}HiAF']:.6f}",
        f"{r[f'Var{s}ExtraAF']:.6f}", str(r[f"Var{s}NM"])])


def format_record(r: dict, score: float | None = None) -> str:
    """One VCF line (utils/vcf_writer.py:104-146); `score` is the learned
    filter's probability (the RFV field), None for the hard filter alone."""
    if r["VarLabel"] not in LABELS:
        raise ValueError(f"record with label {r['VarLabel']!r} cannot be written")
    if r["VarType"] not in TYPE_NAMES:
        raise ValueError(f"record with variant type {r['VarType']!r} cannot be written")
    vd1, vd2 = r["Var1AltDepth"], r["Var2AltDepth"]
    qual = (int(math.log(vd1) / math.log(2) * r["Var1QMean"]) if vd1 > vd2
            else int(math.log(vd2) / math.log(2) * r["Var2QMean"]))
    head = "\t".join([str(r["Chr"]), str(r["Start"]), ".", r["Ref"], r["Alt"], str(qual)])
    sample = re.sub(r"\s", "_", str(r["Sample"]))
    info = (f"STATUS={r['VarLabel']};SAMPLE={sample};TYPE={TYPE_NAMES[r['VarType']]};DP={r['Var1Depth']};"
            f"VD={vd1};AF={r['Var1AF']:.6f};SHIFT3={r['shift3']};MSI={r['MSI']};MSILEN={r['MSI_NT']};"
            f"SSF={r['Pvalue']};SOR={r['Oddratio']};LSEQ={r['5pFlankSeq']};RSEQ={r['3pFlankSeq']}")
    if score is not None:
        info += f";RFV={score}"
    return "\t".join([head, "PASS", info, FORMAT_KEYS, _sample_fields(r, "1"), _sample_fields(r, "2")])


def write(text: str, sample_name: str, scores: list[float] | None = None, threshold: float | None = None) -> str:
    """The VCF of somatic record text: hard filter, then (with per-record
    learned scores and a threshold) the learned filter, sorted by contig and
    start (a stable sort: ties keep the text's order)."""
    recs = parse(text)
    if scores is not None:
        if len(scores) != len(recs):
            raise ValueError("one score per record")
        for r, s in zip(recs, scores):
            r["_score"] = s
    recs = hard_filter(recs)
    if scores is not None and threshold is not None:
        recs = [r for r in recs if r["_score"] >= threshold]
    recs.sort(key=lambda r: (str(r["Chr"]), r["Start"]))
    lines = [format_record(r, r.get("_score") if scores is not None else None) for r in recs]
    return header(sample_name) + "".join(line + "\n" for line in lines)
