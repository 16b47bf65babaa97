"""Learned candidate filter: data, labels and evaluation.

Candidates are the alleles the device pipeline scores (rv_score_candidates:
every position where a non-reference allele was seen at least twice keeps
all its alleles); each gets the 40 device-computed features.  A candidate is
a true variant when its key names a planted variant of that sample at that
position (the key grammar of the CIGAR walk: an SNV is its base, an MNV
"A&CG", an insertion "+SEQ" at the base before it, a deletion "-N" at its
first deleted base; indel keys may sit up to 20 bp to the 3' side after
left-alignment in repeats).  The hard filter is simple mode's own decision
(the allele is emitted as a record).  The learned filter is compared with it
at equal recall: the score threshold is the one that keeps as many true
candidates as the hard filter keeps.
"""
from __future__ import annotations

import numpy as np

from . import api, synth


def truth_keys(variants) -> tuple[set, dict]:
    """Exact (1-based position, key) pairs, plus indel keys for the 3'-shift
    tolerance."""
    exact, indel = set(), {}
    for v in variants:
        if v.vaf <= 0:
            continue
        if v.kind == "snv":
            exact.add((v.pos + 1, v.alt))
        elif v.kind == "mnv":
            exact.add((v.pos + 1, v.alt[0] + "&" + v.alt[1:]))
        elif v.kind == "ins":
            k = "+" + v.alt
            exact.add((v.pos, k))
            indel.setdefault(k, []).append(v.pos)
        elif v.kind == "del":
            k = "-%d" % len(v.ref)
            exact.add((v.pos + 1, k))
            indel.setdefault(k, []).append(v.pos + 1)
    return exact, indel


def label(table, variants) -> np.ndarray:
    exact, indel = truth_keys(variants)
    y = np.zeros(len(table), np.float32)
    for i, (_, pos, key, _) in enumerate(table):
        if (pos, key) in exact:
            y[i] = 1
        elif key in indel and any(0 <= pos - p <= 20 for p in indel[key]):
            y[i] = 1
    return y


def sample_candidates(ctx: api.Context, g, rs, regions, min_count: int = 2):
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    ctx.submit(api.Batch.from_readset(rs), regions)
    ctx.pileup()
    ctx.realign()
    ctx.score_candidates(min_count)
    return ctx.candidates()


def deep_panel(seed: int, n_regions: int = 8, region_len: int = 5000, depth: float = 1500.0):
    """Deep targeted panel (the deep somatic shape, scaled to what the
    synthetic generator makes in seconds): `n_regions` adjacent regions of
    `region_len` bp at `depth`x, germline SNV/indels, low-VAF somatic
    SNV/MNV/indels (VAF log-uniform 0.005..0.1, so that a few reads carry
    them) and C>A artifacts at 1e-4 per read base with quality ~Phred 20."""
    rng = np.random.default_rng(seed)
    margin = 1000
    length = n_regions * region_len + 2 * margin
    g = synth.make_genome(length, rng)
    germ = synth.plant_variants(g, rng, 1e-3, 1e-4, lambda r: 0.5 if r.random() < 0.7 else 1.0)
    som = synth.plant_variants(g, rng, 2e-3, 3e-4, lambda r: float(np.exp(r.uniform(np.log(0.005), np.log(0.1)))),
                               mnv_frac=0.2, avoid=germ)
    regions = [(margin + 1 + i * region_len, margin + (i + 1) * region_len) for i in range(n_regions)]
    rs = synth.simulate(g, germ + som, depth, rng, artifact_rate=1e-4, artifact_q=20, tail_margin=300)
    return g, germ + som, rs, regions


def dataset(seeds, min_count: int = 2, **kw):
    """Features, labels and hard-filter flags over the deep-panel samples."""
    X, Y, Hd = [], [], []
    ctx = api.Context(api.default_params(local_realign=0))
    for s in seeds:
        g, truth, rs, regions = deep_panel(s, **kw)
        f, table = sample_candidates(ctx, g, rs, regions, min_count)
        X.append(f)
        Y.append(label(table, truth))
        Hd.append(np.array([t[3] for t in table], np.float32))
    ctx.close()
    return np.concatenate(X), np.concatenate(Y), np.concatenate(Hd)


def compare(scores: np.ndarray, y: np.ndarray, hard: np.ndarray) -> dict:
    """Precision, recall and F1 of the hard filter and of the learned filter
    thresholded at the hard filter's recall; also the learned filter's
    highest recall at the hard filter's precision and its best F1."""
    pos = y > 0.5
    tp_h = float(np.sum(pos & (hard > 0.5)))
    n_h = float(np.sum(hard > 0.5))
    rec_h = tp_h / max(1.0, float(pos.sum()))
    prec_h = tp_h / max(1.0, n_h)
    f1_h = 2 * prec_h * rec_h / max(1e-12, prec_h + rec_h)
    # threshold keeping the same number of true candidates
    k = int(tp_h)
    order = np.sort(scores[pos])[::-1]
    thr = order[k - 1] if k > 0 else np.inf
    sel = scores >= thr
    tp_l = float(np.sum(pos & sel))
    prec_l = tp_l / max(1.0, float(sel.sum()))
    rec_l = tp_l / max(1.0, float(pos.sum()))
    f1_l = 2 * prec_l * rec_l / max(1e-12, prec_l + rec_l)
    # the learned filter's whole precision/recall curve: the highest recall
    # it reaches at the hard filter's precision (or better), and its best F1
    order_all = np.argsort(-scores, kind="stable")
    tp_c = np.cumsum(pos[order_all])
    n_c = np.arange(1, len(order_all) + 1)
    prec_c = tp_c / n_c
    rec_c = tp_c / max(1.0, float(pos.sum()))
    f1_c = 2 * prec_c * rec_c / np.maximum(1e-12, prec_c + rec_c)
    # only cut points between distinct scores are thresholds
    cut = np.ones(len(order_all), bool)
    if len(order_all) > 1:
        s_sorted = scores[order_all]
        cut[:-1] = s_sorted[:-1] != s_sorted[1:]
    ok = cut & (prec_c >= prec_h - 1e-12)
    if ok.any():
        j = int(np.flatnonzero(ok)[np.argmax(rec_c[ok])])
        eq_prec = {"precision": float(prec_c[j]), "recall": float(rec_c[j]), "f1": float(f1_c[j]),
                   "called": int(n_c[j]), "threshold": float(scores[order_all][j])}
    else:
        eq_prec = {"precision": 0.0, "recall": 0.0, "f1": 0.0, "called": 0, "threshold": float("inf")}
    jb = int(np.argmax(np.where(cut, f1_c, -1.0))) if len(order_all) else 0
    best = {"precision": float(prec_c[jb]), "recall": float(rec_c[jb]), "f1": float(f1_c[jb]),
            "called": int(n_c[jb]), "threshold": float(scores[order_all][jb])} if len(order_all) else {}
    return {"candidates": int(len(y)), "true": int(pos.sum()),
            "hard": {"precision": prec_h, "recall": rec_h, "f1": f1_h, "called": int(n_h)},
            "learned": {"precision": prec_l, "recall": rec_l, "f1": f1_l, "called": int(sel.sum()),
                        "threshold": float(thr)},
            "learned_at_hard_precision": eq_prec,
            "learned_best_f1": best}


def shape_samples(seed: int, deep_regions: int = 12, amp_regions: int = 150, pair_len: int = 300_000):
    """One seed's samples at the shapes of the three calling workloads: a
    slice of the deep somatic panel (tumor 5000x, low-VAF somatic variants,
    C>A artifacts at Q20), a slice of the amplicon panel (log-normal depth,
    PCR duplicates) and the tumor of a 200x/100x somatic pair (strand-biased
    artifacts, which are not truth).  Yields (genome, truth, reads, regions)."""
    g, (germ, som), t, _, regions = synth.deep_somatic_panel(seed=seed, n_regions=max(deep_regions, 1),
                                                            tumor_depth=5000.0, normal_depth=1.0,
                                                            only=list(range(deep_regions)))
    yield g, germ + som, synth.unpacked(t), regions
    ga, va, ra, rega = synth.amplicon_panel_native(seed=seed + 7, n_regions=amp_regions,
                                                    genome_len=amp_regions * 5000)
    yield ga, va, synth.unpacked(ra), rega
    gp, (germp, somp, _art), tp, _np = synth.somatic_pair(seed=seed + 13, length=pair_len)
    tiles = [(1 + 10_000 * i, 10_000 * (i + 1)) for i in range(pair_len // 10_000)]
    yield gp, germp + somp, tp, tiles


def dataset_shapes(seeds, min_count: int = 2, **kw):
    """Features, labels and hard-filter flags of every candidate of the
    shape samples of `seeds` (see shape_samples); also the per-seed slices
    (start, end) of the arrays."""
    X, Y, Hd, bounds = [], [], [], []
    ctx = api.Context(api.default_params(local_realign=0))
    n = 0
    for s in seeds:
        n0 = n
        for g, truth, rs, regions in shape_samples(s, **kw):
            f, table = sample_candidates(ctx, g, rs, regions, min_count)
            X.append(f)
            Y.append(label(table, truth))
            Hd.append(np.array([t[3] for t in table], np.float32))
            n += len(table)
        bounds.append((n0, n))
    ctx.close()
    return np.concatenate(X), np.concatenate(Y), np.concatenate(Hd), bounds
