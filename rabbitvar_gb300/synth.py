"""Seeded synthetic genomes and read sets with planted variants.

The reference's own accuracy data (SEQC-II HCC1395 BAMs) is not available, so
every workload here is generated from a seed: a random contig (uniform ACGT
at a chosen GC fraction with homopolymer runs), planted SNVs / MNVs / indels
with per-variant allele fractions, and 2x150 bp read pairs with Phred
qualities, sequencing errors, N bases, soft clips, MAPQ and NM tags.

A read set is held as a structure of arrays (`ReadSet`) in exactly the layout
the GPU library consumes (BAM-native 4-bit bases, Phred quals, BAM CIGAR
words).  `write_bam` serialises the same reads to a BGZF-compressed,
coordinate-sorted BAM plus FASTA/.fai so the reference binary can read them.
"""
from __future__ import annotations

import dataclasses
import struct
import zlib

import numpy as np

NT16 = "=ACMGRSVTWYHKDBN"
# 2-bit genome alphabet A,C,G,T -> BAM 4-bit codes 1,2,4,8; N -> 15
CODE_OF = np.array([1, 2, 4, 8], dtype=np.uint8)
CODE_N = 15
ASCII_OF_CODE = np.frombuffer(NT16.encode(), dtype=np.uint8)
OP_M, OP_I, OP_D, OP_S = 0, 1, 2, 4


@dataclasses.dataclass
class Variant:
    pos: int          # 0-based reference position of the first changed base
    kind: str         # "snv", "mnv", "ins", "del"
    ref: str
    alt: str
    vaf: float
    strand_bias: float = 0.0   # fraction of carrying reads forced onto one strand (artifacts)
    strand: int = 0            # strand the artifact prefers (0 fwd, 1 rev)
    vq: int | None = None      # base quality forced on the changed bases of carrying reads (SNV/MNV)


@dataclasses.dataclass
class ReadSet:
    """Reads of one contig, coordinate-sorted, in the GPU batch layout.

    pos:   int32  0-based leftmost aligned position (BAM POS)
    flag:  uint16 SAM flag
    mapq:  uint8
    mpos:  int32  0-based mate position
    isize: int32
    nm:    int32  NM tag value
    n_cigar, cig_off: uint16 / uint32 -> cigar (uint32 BAM words)
    l_qseq, base_off: int32 / uint64 -> seq4 (one 4-bit code per base, unpacked)
                       and qual (uint8 Phred); base_off is a multiple of 32
    """
    contig: str
    contig_len: int
    pos: np.ndarray
    flag: np.ndarray
    mapq: np.ndarray
    mpos: np.ndarray
    isize: np.ndarray
    nm: np.ndarray
    n_cigar: np.ndarray
    cig_off: np.ndarray
    cigar: np.ndarray
    l_qseq: np.ndarray
    base_off: np.ndarray
    seq4: np.ndarray | None
    qual: np.ndarray
    name_id: np.ndarray
    packed: np.ndarray | None = None   # BAM-packed bases (native generator; seq4 is then None)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def packed_seq(self) -> np.ndarray:
        """BAM-packed 4-bit sequence (two bases per byte, high nibble first),
        indexed by base_off // 2 for every read."""
        if self.packed is not None:
            return self.packed
        s = self.seq4
        if s.shape[0] % 2:
            s = np.concatenate([s, np.zeros(1, np.uint8)])
        return ((s[0::2] << 4) | s[1::2]).astype(np.uint8)


def subset(rs: ReadSet, keep: np.ndarray) -> ReadSet:
    """The reads of `rs` where `keep` is true, in the same order and layout."""
    return take(rs, np.nonzero(keep)[0])


def unpacked(rs: ReadSet) -> ReadSet:
    """The same reads with one 4-bit code per byte (seq4), as the numpy
    generator holds them (a read set of the native generator has only the
    packed bases)."""
    if rs.seq4 is not None:
        return rs
    seq4 = np.empty(rs.packed.shape[0] * 2, dtype=np.uint8)
    seq4[0::2] = rs.packed >> 4
    seq4[1::2] = rs.packed & 15
    return dataclasses.replace(rs, seq4=seq4, packed=None)


def read_range(rs: ReadSet, a: int, b: int) -> ReadSet:
    """Reads [a, b) of `rs` (a contiguous, coordinate-sorted slice) with
    unpacked bases."""
    stride = int(rs.base_off[1] - rs.base_off[0]) if rs.n > 1 else 160
    c0 = int(rs.cig_off[a]) if a < rs.n else int(rs.cigar.shape[0])
    c1 = int(rs.cig_off[b]) if b < rs.n else int(rs.cigar.shape[0])
    b0, b1 = a * stride, b * stride
    if rs.packed is not None:
        pk = rs.packed[b0 // 2:b1 // 2]
        seq4 = np.empty(pk.shape[0] * 2, dtype=np.uint8)
        seq4[0::2] = pk >> 4
        seq4[1::2] = pk & 15
    else:
        seq4 = rs.seq4[b0:b1].copy()
    return ReadSet(contig=rs.contig, contig_len=rs.contig_len, pos=rs.pos[a:b].copy(), flag=rs.flag[a:b].copy(),
                   mapq=rs.mapq[a:b].copy(), mpos=rs.mpos[a:b].copy(), isize=rs.isize[a:b].copy(),
                   nm=rs.nm[a:b].copy(), n_cigar=rs.n_cigar[a:b].copy(),
                   cig_off=(rs.cig_off[a:b] - np.uint32(c0)).astype(np.uint32), cigar=rs.cigar[c0:c1].copy(),
                   l_qseq=rs.l_qseq[a:b].copy(), base_off=(rs.base_off[a:b] - np.uint64(b0)).astype(np.uint64),
                   seq4=seq4, qual=rs.qual[b0:b1].copy(), name_id=rs.name_id[a:b].copy())


def take(rs: ReadSet, idx: np.ndarray) -> ReadSet:
    """The reads rs[idx] (indices may repeat: exact duplicate records), in
    the order of `idx`, in the same layout."""
    idx = np.asarray(idx, dtype=np.int64)
    n = idx.shape[0]
    n_cigar = rs.n_cigar[idx]
    cig_off = np.zeros(n, dtype=np.uint32)
    if n:
        cig_off[1:] = np.cumsum(n_cigar[:-1].astype(np.uint32))
    cigar = np.concatenate([rs.cigar[int(rs.cig_off[i]):int(rs.cig_off[i]) + int(rs.n_cigar[i])] for i in idx]
                           ) if n else np.zeros(0, np.uint32)
    stride = int(rs.base_off[1] - rs.base_off[0]) if rs.n > 1 else 160
    base_off = np.arange(n, dtype=np.uint64) * stride
    seq4 = np.zeros(n * stride, dtype=np.uint8)
    qv = np.zeros(n * stride, dtype=np.uint8)
    for j, i in enumerate(idx.tolist()):
        a = int(rs.base_off[i])
        seq4[j * stride:(j + 1) * stride] = rs.seq4[a:a + stride]
        qv[j * stride:(j + 1) * stride] = rs.qual[a:a + stride]
    return ReadSet(contig=rs.contig, contig_len=rs.contig_len, pos=rs.pos[idx], flag=rs.flag[idx],
                   mapq=rs.mapq[idx], mpos=rs.mpos[idx], isize=rs.isize[idx], nm=rs.nm[idx],
                   n_cigar=n_cigar, cig_off=cig_off, cigar=cigar.astype(np.uint32), l_qseq=rs.l_qseq[idx],
                   base_off=base_off, seq4=seq4, qual=qv, name_id=rs.name_id[idx])


def make_genome(length: int, rng: np.random.Generator, gc: float = 0.41,
                homopolymer_rate: float = 0.01) -> np.ndarray:
    """Uniform random contig (0..3 = A,C,G,T) with GC fraction `gc`; a
    fraction `homopolymer_rate` of positions start a 5-20 bp homopolymer."""
    p_at = (1.0 - gc) / 2
    p_gc = gc / 2
    g = rng.choice(4, size=length, p=[p_at, p_gc, p_gc, p_at]).astype(np.uint8)
    starts = np.nonzero(rng.random(length) < homopolymer_rate)[0]
    lens = rng.integers(5, 21, size=starts.shape[0])
    for s, ln in zip(starts.tolist(), lens.tolist()):
        g[s:s + ln] = g[s]
    return g


def genome_str(g: np.ndarray) -> str:
    return np.frombuffer(b"ACGT", dtype=np.uint8)[g].tobytes().decode()


def _rand_other(base: int, rng) -> int:
    return int((base + rng.integers(1, 4)) % 4)


def plant_variants(g: np.ndarray, rng: np.random.Generator, snv_rate: float,
                   indel_rate: float, vaf_fn, mnv_frac: float = 0.0,
                   max_indel: int = 10, margin: int = 200,
                   spacing: int = 15, avoid=None) -> list[Variant]:
    """Plant SNVs (and MNVs, a fraction `mnv_frac` of SNV sites) and 1..max_indel
    bp insertions/deletions at the given per-bp rates, at least `spacing` bp
    apart.  `vaf_fn(rng)` draws the allele fraction of each variant."""
    L = g.shape[0]
    out: list[Variant] = []
    taken = np.zeros(L, dtype=bool)
    if avoid is not None:
        for v in avoid:
            taken[max(0, v.pos - spacing):v.pos + spacing + 12] = True
    n_snv = rng.binomial(L - 2 * margin, snv_rate)
    n_ind = rng.binomial(L - 2 * margin, indel_rate)
    cand = rng.integers(margin, L - margin, size=n_snv + n_ind)
    for i, p in enumerate(cand.tolist()):
        lo, hi = max(0, p - spacing), min(L, p + spacing + 12)
        if taken[lo:hi].any():
            continue
        taken[lo:hi] = True
        vaf = float(vaf_fn(rng))
        if i < n_snv:
            if rng.random() < mnv_frac:
                k = int(rng.integers(2, 4))
                ref = "".join("ACGT"[x] for x in g[p:p + k].tolist())
                alt = "".join("ACGT"[_rand_other(int(x), rng)] for x in g[p:p + k].tolist())
                out.append(Variant(p, "mnv", ref, alt, vaf))
            else:
                out.append(Variant(p, "snv", "ACGT"[g[p]], "ACGT"[_rand_other(int(g[p]), rng)], vaf))
        else:
            k = int(rng.integers(1, max_indel + 1))
            if rng.random() < 0.5:
                ins = "".join("ACGT"[x] for x in rng.integers(0, 4, size=k).tolist())
                out.append(Variant(p, "ins", "", ins, vaf))
            else:
                ref = "".join("ACGT"[x] for x in g[p:p + k].tolist())
                out.append(Variant(p, "del", ref, "", vaf))
    out.sort(key=lambda v: v.pos)
    return out


def _qualities(n_reads: int, L: int, rng) -> np.ndarray:
    """Phred mixture centred at 37 (range 2..41): most bases near 37 with a
    mild decline along the read, a minority drawn from a low-quality tail."""
    base = rng.normal(37.0, 2.0, size=(n_reads, L))
    decline = np.linspace(0.0, 3.0, L)[None, :]
    q = base - decline
    low = rng.random((n_reads, L)) < 0.08
    q = np.where(low, rng.uniform(2, 30, size=(n_reads, L)), q)
    return np.clip(np.rint(q), 2, 41).astype(np.uint8)


def simulate(genome: np.ndarray, variants: list[Variant], depth: float,
             rng: np.random.Generator, contig: str = "ctg", read_len: int = 150,
             insert_mean: float = 350.0, insert_sd: float = 50.0,
             softclip_frac: float = 0.02, mapq0_frac: float = 0.05,
             n_rate: float = 2e-4, span: tuple[int, int] | None = None,
             name_base: int = 0, artifact_rate: float = 0.0,
             artifact_q: int | None = None, tail_margin: int = 0) -> ReadSet:
    """Simulate coordinate-sorted 2x`read_len` pairs at `depth`x over
    `span` (default: the whole contig).  Each read independently carries
    each overlapping variant with probability vaf (strand-biased variants put
    a `strand_bias` fraction of carriers on their preferred strand)."""
    G = genome.shape[0]
    L = read_len
    lo, hi = span if span is not None else (0, G)
    n_frag = int(round(depth * (hi - lo) / (2 * L)))
    ins = np.clip(np.rint(rng.normal(insert_mean, insert_sd, n_frag)), L + 20, 3 * L).astype(np.int64)
    fstart = rng.integers(max(0, lo - L // 2), np.maximum(max(0, lo - L // 2) + 1, hi - ins + L // 2))
    fstart = np.clip(fstart, 0, G - tail_margin - ins)
    r1_fwd = rng.random(n_frag) < 0.5
    # read A = leftmost (forward strand), read B = rightmost (reverse strand)
    startA = fstart
    startB = fstart + ins - L
    n = 2 * n_frag
    start = np.concatenate([startA, startB])
    rev = np.concatenate([np.zeros(n_frag, bool), np.ones(n_frag, bool)])
    frag = np.concatenate([np.arange(n_frag), np.arange(n_frag)])
    is_r1 = np.concatenate([r1_fwd, ~r1_fwd])
    mate_start = np.concatenate([startB, startA])
    isize = np.concatenate([ins, -ins])

    seq = genome[start[:, None] + np.arange(L)[None, :]].copy()  # 0..3
    qual = _qualities(n, L, rng)
    # quality profile runs in sequencing direction: reverse it for reverse reads
    qual[rev] = qual[rev][:, ::-1]

    order_by_start = np.argsort(start, kind="stable")
    s_sorted = start[order_by_start]

    # per-read list of (variant index) for indels that the read carries
    carried_indels: dict[int, list[int]] = {}
    for vi, v in enumerate(variants):
        vlen = max(len(v.ref), 1)
        a = np.searchsorted(s_sorted, v.pos - L + 1, side="left")
        b = np.searchsorted(s_sorted, v.pos + vlen, side="left")
        idx = order_by_start[a:b]
        if idx.size == 0:
            continue
        p_carry = np.full(idx.size, v.vaf)
        if v.strand_bias > 0:
            on = rev[idx] == bool(v.strand)
            # a fraction strand_bias of carriers sit on the preferred strand
            w_on = v.strand_bias / max(on.mean(), 1e-9)
            w_off = (1 - v.strand_bias) / max(1 - on.mean(), 1e-9)
            p_carry = np.clip(v.vaf * np.where(on, w_on, w_off), 0, 1)
        carry = idx[rng.random(idx.size) < p_carry]
        if v.kind in ("snv", "mnv"):
            for k, ch in enumerate(v.alt):
                col = v.pos + k - start[carry]
                ok = (col >= 0) & (col < L)
                seq[carry[ok], col[ok]] = "ACGT".index(ch)
                if v.vq is not None:
                    qual[carry[ok], col[ok]] = v.vq
        else:
            # indel carriers need at least 3 aligned bases on each side
            off = v.pos - start[carry]
            ok = (off >= 3) & (off + len(v.ref) <= L - 3) & (start[carry] + L + len(v.ref) + 4 < G)
            for r in carry[ok].tolist():
                carried_indels.setdefault(r, []).append(vi)

    # sequencing errors: substitution with probability 10^(-q/10)
    err = rng.random((n, L)) < np.power(10.0, -qual.astype(np.float64) / 10.0)
    if artifact_rate > 0:
        # oxidation-like C>A artifacts on C bases, at a skewed low quality
        art = (seq == 1) & (rng.random((n, L)) < artifact_rate)
        seq = np.where(art, 0, seq)
        if artifact_q is not None:
            qual = np.where(art, np.uint8(artifact_q), qual)
    seq = np.where(err, (seq + rng.integers(1, 4, size=(n, L))) % 4, seq).astype(np.uint8)
    codes = CODE_OF[seq]
    nmask = rng.random((n, L)) < n_rate
    codes[nmask] = CODE_N
    qual[nmask] = 2

    mapq = np.where(rng.random(n) < mapq0_frac, 0, 60).astype(np.uint8)
    pos = start.astype(np.int64).copy()
    cig_list: list[list[int] | None] = [None] * n
    ref_codes = CODE_OF[genome]

    # indel-carrying reads: rebuild sequence and CIGAR from the haplotype
    for r, vis in carried_indels.items():
        s0 = int(start[r])
        bases: list[int] = []
        ops: list[list[int]] = []

        def push(op, ln):
            if ln <= 0:
                return
            if ops and ops[-1][0] == op:
                ops[-1][1] += ln
            else:
                ops.append([op, ln])
        p = s0
        vq = [variants[i] for i in sorted(vis, key=lambda i: variants[i].pos)]
        j = 0
        while len(bases) < L:
            if j < len(vq) and p == vq[j].pos:
                v = vq[j]
                j += 1
                if v.kind == "ins":
                    k = min(len(v.alt), L - len(bases))
                    bases.extend("ACGT".index(c) for c in v.alt[:k])
                    push(OP_I, k)
                    continue
                else:
                    push(OP_D, len(v.ref))
                    p += len(v.ref)
                    continue
            bases.append(int(genome[p]))
            push(OP_M, 1)
            p += 1
        # keep the simulated error/N pattern on the matched bases
        b = np.array(bases[:L], dtype=np.uint8)
        c = CODE_OF[b]
        keep_err = err[r] | nmask[r]
        c = np.where(nmask[r], CODE_N, np.where(err[r], CODE_OF[(b + 1) % 4], c))
        codes[r] = c
        if ops[-1][0] != OP_M:   # never end on an indel
            ops[-1][0] = OP_S if ops[-1][0] == OP_I else ops[-1][0]
        cig_list[r] = [(ln << 4) | op for op, ln in ops]
        del keep_err

    # soft clips on a fraction of the plain reads
    clip = (rng.random(n) < softclip_frac)
    clip_len = rng.integers(5, 31, size=n)
    clip_5p = rng.random(n) < 0.5
    junk = rng.random(n) < 0.5
    for r in np.nonzero(clip)[0].tolist():
        if cig_list[r] is not None:
            continue
        k = int(clip_len[r])
        if junk[r]:
            rnd = CODE_OF[rng.integers(0, 4, size=k)]
            if clip_5p[r]:
                codes[r, :k] = rnd
            else:
                codes[r, L - k:] = rnd
        if clip_5p[r]:
            cig_list[r] = [(k << 4) | OP_S, ((L - k) << 4) | OP_M]
            pos[r] += k
        else:
            cig_list[r] = [((L - k) << 4) | OP_M, (k << 4) | OP_S]

    # NM: mismatches (N included) over aligned bases plus inserted/deleted bases
    ref_win = ref_codes[np.clip(start[:, None] + np.arange(L)[None, :], 0, G - 1)]
    nm = (codes != ref_win).sum(axis=1).astype(np.int32)
    for r in [i for i in range(n) if cig_list[i] is not None]:
        cg = cig_list[r]
        q = 0
        rp = int(pos[r])
        m = 0
        for w in cg:
            op, ln = w & 15, w >> 4
            if op == OP_M:
                m += int((codes[r, q:q + ln] != ref_codes[rp:rp + ln]).sum())
                q += ln
                rp += ln
            elif op == OP_I:
                m += ln
                q += ln
            elif op == OP_D:
                m += ln
                rp += ln
            elif op == OP_S:
                q += ln
        nm[r] = m

    # mate fields follow the (possibly clipped) alignment starts
    mate_of = np.concatenate([np.arange(n_frag, n), np.arange(0, n_frag)])
    mpos = pos[mate_of]
    flag = (0x1 | 0x2 | np.where(rev, 0x10, 0) | np.where(rev[mate_of], 0x20, 0)
            | np.where(is_r1, 0x40, 0x80)).astype(np.uint16)

    order = np.lexsort((frag, pos))
    return _pack(contig, G, order, pos, flag, mapq, mpos, isize, nm, cig_list, codes, qual,
                 frag + name_base, L)


def _pack(contig, G, order, pos, flag, mapq, mpos, isize, nm, cig_list, codes, qual, names, L):
    n = order.shape[0]
    n_cigar = np.ones(n, dtype=np.uint16)
    cig_words = []
    default = np.uint32((L << 4) | OP_M)
    for i, r in enumerate(order.tolist()):
        cg = cig_list[r]
        if cg is None:
            cig_words.append([int(default)])
        else:
            n_cigar[i] = len(cg)
            cig_words.append(cg)
    cig_off = np.zeros(n, dtype=np.uint32)
    cig_off[1:] = np.cumsum(n_cigar[:-1].astype(np.uint32))
    cigar = np.fromiter((w for cg in cig_words for w in cg), dtype=np.uint32)
    stride = (L + 31) // 32 * 32
    base_off = (np.arange(n, dtype=np.uint64) * stride)
    seq4 = np.zeros(n * stride, dtype=np.uint8)
    qv = np.zeros(n * stride, dtype=np.uint8)
    seq4.reshape(n, stride)[:, :L] = codes[order]
    qv.reshape(n, stride)[:, :L] = qual[order]
    return ReadSet(contig=contig, contig_len=int(G), pos=pos[order].astype(np.int32),
                   flag=flag[order], mapq=mapq[order], mpos=mpos[order].astype(np.int32),
                   isize=isize[order].astype(np.int32), nm=nm[order],
                   n_cigar=n_cigar, cig_off=cig_off, cigar=cigar,
                   l_qseq=np.full(n, L, dtype=np.int32), base_off=base_off,
                   seq4=seq4, qual=qv, name_id=names[order].astype(np.int64))


_OPS = {"M": 0, "I": 1, "D": 2, "N": 3, "S": 4, "H": 5}
_BASE = {"A": 0, "C": 1, "G": 2, "T": 3}


def explicit_reads(contig: str, genome: np.ndarray, reads: list[dict]) -> ReadSet:
    """A read set written out read by read, for cases that pin one code path.

    Each read is a dict: `pos` (0-based leftmost reference base the CIGAR
    starts at) and `segs`, a list of CIGAR segments:
      ("M", n) or ("M", n, {offset: "ACGTN"})  aligned bases, substitutions at
                                              offsets within the segment
      ("I", "ACG")                            inserted bases
      ("D", n) / ("N", n)                     reference skipped
      ("S", "ACG")                            clipped bases as given
      ("S", n)                                clipped bases copied from the
                                              reference beside the clip
      ("H", n)                                hard clip (no bases)
    and optionally `qual` (an int for every base, or a list), `qual_at`
    ({read offset: Phred}), `rev` (reverse strand), `flag`, `mapq`, `mpos`
    and `nm` (default: substitutions + inserted + deleted bases).  Reads are
    sorted by position (stable), as a coordinate-sorted BAM holds them.
    """
    G = int(genome.shape[0])
    recs = []
    for i, r in enumerate(reads):
        pos = int(r["pos"])
        rp = pos
        codes, cig = [], []
        nm = 0
        segs = r["segs"]
        for j, sg in enumerate(segs):
            op = sg[0]
            if op == "M":
                n = int(sg[1])
                subs = sg[2] if len(sg) > 2 else {}
                for k in range(n):
                    if k in subs:
                        b = subs[k]
                        c = CODE_N if b == "N" else int(CODE_OF[_BASE[b]])
                        if b == "N" or _BASE[b] != int(genome[rp + k]):
                            nm += 1
                    else:
                        c = int(CODE_OF[int(genome[rp + k])])
                    codes.append(c)
                rp += n
            elif op == "I":
                codes += [int(CODE_OF[_BASE[b]]) for b in sg[1]]
                nm += len(sg[1])
                n = len(sg[1])
            elif op in ("D", "N"):
                n = int(sg[1])
                rp += n
                if op == "D":
                    nm += n
            elif op == "S":
                if isinstance(sg[1], str):
                    codes += [CODE_N if b == "N" else int(CODE_OF[_BASE[b]]) for b in sg[1]]
                    n = len(sg[1])
                else:
                    n = int(sg[1])
                    at = pos - n if j == 0 or all(x[0] == "H" for x in segs[:j]) else rp
                    codes += [int(CODE_OF[int(genome[at + k])]) for k in range(n)]
            elif op == "H":
                n = int(sg[1])
            else:
                raise ValueError(op)
            cig.append((n << 4) | _OPS[op])
        L = len(codes)
        q = r.get("qual", 37)
        qual = list(q) if not isinstance(q, int) else [q] * L
        for k, v in r.get("qual_at", {}).items():
            qual[k] = v
        assert len(qual) == L and rp <= G
        flag = r.get("flag", 0x1 | 0x2 | (0x10 if r.get("rev") else 0x20) | 0x40)
        recs.append((pos, i, flag, r.get("mapq", 60), r.get("mpos", pos + 200), r.get("nm", nm), cig, codes, qual))
    recs.sort(key=lambda t: (t[0], t[1]))
    n = len(recs)
    stride = max([32] + [(len(t[7]) + 31) // 32 * 32 for t in recs])
    seq4 = np.zeros(n * stride, np.uint8)
    qv = np.zeros(n * stride, np.uint8)
    for k, t in enumerate(recs):
        seq4[k * stride:k * stride + len(t[7])] = t[7]
        qv[k * stride:k * stride + len(t[8])] = t[8]
    n_cigar = np.array([len(t[6]) for t in recs], np.uint16)
    cig_off = np.zeros(n, np.uint32)
    if n:
        cig_off[1:] = np.cumsum(n_cigar[:-1].astype(np.uint32))
    pos = np.array([t[0] for t in recs], np.int32)
    mpos = np.array([t[4] for t in recs], np.int32)
    return ReadSet(contig=contig, contig_len=G, pos=pos, flag=np.array([t[2] for t in recs], np.uint16),
                   mapq=np.array([t[3] for t in recs], np.uint8), mpos=mpos, isize=(mpos - pos + 150).astype(np.int32),
                   nm=np.array([t[5] for t in recs], np.int32), n_cigar=n_cigar, cig_off=cig_off,
                   cigar=np.array([w for t in recs for w in t[6]], np.uint32),
                   l_qseq=np.array([len(t[7]) for t in recs], np.int32),
                   base_off=np.arange(n, dtype=np.uint64) * stride, seq4=seq4, qual=qv,
                   name_id=np.array([t[1] for t in recs], np.int64))


# --------------------------------------------------------------------------
# writers (BGZF/BAM per SAM spec 4.1-4.2, FASTA + .fai, BED)
# --------------------------------------------------------------------------
_BGZF_EOF = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")


def _bgzf_block(data: bytes, level: int) -> bytes:
    co = zlib.compressobj(level, zlib.DEFLATED, -15)
    cdata = co.compress(data) + co.flush()
    bsize = len(cdata) + 25
    hdr = struct.pack("<BBBBIBBHBBHH", 31, 139, 8, 4, 0, 0, 255, 6, 66, 67, 2, bsize)
    return hdr + cdata + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data))


def write_bgzf(path: str, payload: bytes, level: int = 1) -> None:
    with open(path, "wb") as f:
        step = 0xFF00
        for i in range(0, len(payload), step):
            f.write(_bgzf_block(payload[i:i + step], level))
        f.write(_BGZF_EOF)


def _reg2bin(beg: int, end: int) -> int:
    """UCSC binning scheme (SAM spec 5.3)."""
    end -= 1
    if beg >> 14 == end >> 14:
        return ((1 << 15) - 1) // 7 + (beg >> 14)
    if beg >> 17 == end >> 17:
        return ((1 << 12) - 1) // 7 + (beg >> 17)
    if beg >> 20 == end >> 20:
        return ((1 << 9) - 1) // 7 + (beg >> 20)
    if beg >> 23 == end >> 23:
        return ((1 << 6) - 1) // 7 + (beg >> 23)
    if beg >> 26 == end >> 26:
        return ((1 << 3) - 1) // 7 + (beg >> 26)
    return 0


def _segments(dst_start: np.ndarray, src_start: np.ndarray, length: np.ndarray):
    """Flat (destination, source) byte indices of variable-length segments."""
    length = length.astype(np.int64)
    tot = int(length.sum())
    within = np.arange(tot, dtype=np.int64) - np.repeat(np.cumsum(length) - length, length)
    return np.repeat(dst_start.astype(np.int64), length) + within, np.repeat(src_start.astype(np.int64), length) + within


def bam_bytes(rs: ReadSet, sample: str = "S") -> bytes:
    """Uncompressed BAM stream of a read set (records built with numpy)."""
    text = f"@HD\tVN:1.6\tSO:coordinate\n@SQ\tSN:{rs.contig}\tLN:{rs.contig_len}\n@RG\tID:{sample}\tSM:{sample}\n".encode()
    head = b"".join([b"BAM\x01", struct.pack("<I", len(text)), text, struct.pack("<I", 1),
                     struct.pack("<I", len(rs.contig) + 1), rs.contig.encode() + b"\x00",
                     struct.pack("<I", rs.contig_len)])
    n = rs.n
    if n == 0:
        return head
    names = np.frombuffer(b"".join(b"r%d\x00" % int(x) for x in rs.name_id), np.uint8)
    l_name = np.char.str_len(np.char.mod("r%d", rs.name_id.astype(np.int64))).astype(np.int64) + 1
    nc = rs.n_cigar.astype(np.int64)
    L = rs.l_qseq.astype(np.int64)
    bo = rs.base_off.astype(np.int64)
    co = rs.cig_off.astype(np.int64)
    # reference span for the bin
    words = rs.cigar.astype(np.int64)
    consumes = np.isin(words & 15, (0, 2, 3, 7, 8))
    span_w = np.where(consumes, words >> 4, 0)
    csum = np.concatenate([[0], np.cumsum(span_w)])
    ref_len = csum[co + nc] - csum[co]
    p = rs.pos.astype(np.int64)
    end = p + np.maximum(ref_len, 1) - 1
    bins = np.zeros(n, np.int64)
    done = np.zeros(n, bool)
    for shift, off in ((14, ((1 << 15) - 1) // 7), (17, ((1 << 12) - 1) // 7), (20, ((1 << 9) - 1) // 7),
                       (23, ((1 << 6) - 1) // 7), (26, ((1 << 3) - 1) // 7)):
        hit = ~done & ((p >> shift) == (end >> shift))
        bins[hit] = off + (p[hit] >> shift)
        done |= hit
    rec_len = 32 + l_name + 4 * nc + (L + 1) // 2 + L + 7
    start = np.concatenate([[0], np.cumsum(rec_len + 4)[:-1]])
    buf = np.zeros(int((rec_len + 4).sum()), np.uint8)
    fixed = np.zeros(n, dtype=np.dtype([("bs", "<u4"), ("tid", "<i4"), ("pos", "<i4"), ("lrn", "u1"), ("mapq", "u1"),
                                        ("bin", "<u2"), ("nc", "<u2"), ("flag", "<u2"), ("lq", "<i4"),
                                        ("ntid", "<i4"), ("npos", "<i4"), ("tlen", "<i4")]))
    fixed["bs"] = rec_len
    fixed["pos"] = p
    fixed["lrn"] = l_name
    fixed["mapq"] = rs.mapq
    fixed["bin"] = bins
    fixed["nc"] = nc
    fixed["flag"] = rs.flag
    fixed["lq"] = L
    fixed["npos"] = rs.mpos
    fixed["tlen"] = rs.isize
    fb = fixed.view(np.uint8).reshape(n, 36)
    buf[(start[:, None] + np.arange(36)[None, :]).ravel()] = fb.ravel()
    at = start + 36
    d, sidx = _segments(at, np.concatenate([[0], np.cumsum(l_name)[:-1]]), l_name)
    buf[d] = names[sidx]
    at = at + l_name
    cb = rs.cigar.astype("<u4").view(np.uint8)
    d, sidx = _segments(at, 4 * co, 4 * nc)
    buf[d] = cb[sidx]
    at = at + 4 * nc
    packed = rs.packed_seq()
    d, sidx = _segments(at, bo // 2, (L + 1) // 2)
    buf[d] = packed[sidx]
    at = at + (L + 1) // 2
    d, sidx = _segments(at, bo, L)
    buf[d] = rs.qual[sidx]
    at = at + L
    aux = np.zeros(n, dtype=np.dtype([("t", "S3"), ("v", "<i4")]))
    aux["t"] = b"NMi"
    aux["v"] = rs.nm
    buf[(at[:, None] + np.arange(7)[None, :]).ravel()] = aux.view(np.uint8).reshape(n, 7).ravel()
    return head + buf.tobytes()


def write_bam(path: str, rs: ReadSet, sample: str = "S") -> None:
    write_bgzf(path, bam_bytes(rs, sample))
    # the shim builds its own in-memory index; an empty .bai marks the file as indexed
    open(path + ".bai", "wb").close()


def write_fasta(path: str, name: str, genome: np.ndarray, width: int = 60) -> None:
    s = genome_str(genome)
    with open(path, "w") as f:
        hdr = f">{name}\n"
        f.write(hdr)
        for i in range(0, len(s), width):
            f.write(s[i:i + width] + "\n")
    with open(path + ".fai", "w") as f:
        f.write(f"{name}\t{len(s)}\t{len(hdr)}\t{width}\t{width + 1}\n")


def write_bed(path: str, contig: str, regions: list[tuple[int, int]], name: str = "g") -> None:
    """4-column BED (0-based start, end), the layout RabbitVar treats as
    zero-based (src/RegionBuilder.cpp buildRegions)."""
    with open(path, "w") as f:
        for s, e in regions:
            f.write(f"{contig}\t{s}\t{e}\t{name}\n")


# --------------------------------------------------------------------------
# workload presets (shapes of the reference's benchmark configurations)
# --------------------------------------------------------------------------
def germline_small(seed: int = 0x5EED0000, length: int = 100_000, depth: float = 30.0):
    """100 kb contig, 30x 2x150 pairs, SNVs 1e-3/bp (VAF 0.5|1.0), indels
    1-10 bp at 1e-4/bp: the single-sample germline shape."""
    rng = np.random.default_rng(seed)
    g = make_genome(length, rng)
    vs = plant_variants(g, rng, 1e-3, 1e-4, lambda r: 0.5 if r.random() < 0.7 else 1.0)
    rs = simulate(g, vs, depth, rng)
    return g, vs, rs


def somatic_pair(seed: int = 0x5EED0001, length: int = 1_000_000, tumor_depth: float = 200.0,
                 normal_depth: float = 100.0):
    """Tumor/normal pair: germline SNVs 1e-3/bp in both, somatic SNV/MNV
    2e-5/bp with VAF ~U(0.01, 0.5) in the tumor, strand-biased artifacts
    5e-6/bp with a 95% single-strand fraction."""
    rng = np.random.default_rng(seed)
    g = make_genome(length, rng)
    germ = plant_variants(g, rng, 1e-3, 1e-4, lambda r: 0.5 if r.random() < 0.7 else 1.0)
    som = plant_variants(g, rng, 2e-5, 0.0, lambda r: r.uniform(0.01, 0.5), mnv_frac=0.3, avoid=germ)
    art = plant_variants(g, rng, 5e-6, 0.0, lambda r: r.uniform(0.05, 0.2), avoid=germ + som)
    for v in art:
        v.strand_bias = 0.95
        v.strand = int(rng.integers(0, 2))
    tumor = simulate(g, germ + som + art, tumor_depth, rng, name_base=0)
    normal = simulate(g, germ, normal_depth, rng, name_base=10_000_000)
    return g, (germ, som, art), tumor, normal


def somatic_mix(seed: int = 0x5EED0051, length: int = 30_000, tumor_depth: float = 80.0,
                normal_depth: float = 40.0, gap: tuple[int, int] | None = (12_000, 12_400),
                tail_margin: int = 0):
    """Small tumor/normal pair that reaches every somatic label: shared
    germline variants, tumor-only somatic SNV/MNV/indels, heterozygous normal
    variants lost (VAF 0.02) or made homozygous (VAF 1.0) in the tumor,
    strand-biased artifacts in both samples, shared SNVs with low-quality
    normal reads, and a window `gap` (0-based,
    half-open) where the normal has no reads."""
    rng = np.random.default_rng(seed)
    g = make_genome(length, rng)
    germ = plant_variants(g, rng, 2e-3, 4e-4, lambda r: 0.5 if r.random() < 0.7 else 1.0)
    som = plant_variants(g, rng, 1e-3, 3e-4, lambda r: r.uniform(0.01, 0.5), mnv_frac=0.3, avoid=germ)
    loh = plant_variants(g, rng, 1e-3, 2e-4, lambda r: 0.5, mnv_frac=0.2, avoid=germ + som)
    art = plant_variants(g, rng, 6e-4, 0.0, lambda r: r.uniform(0.05, 0.3), avoid=germ + som + loh)
    for v in art:
        v.strand_bias = 0.95
        v.strand = int(rng.integers(0, 2))
    # shared SNVs whose normal reads carry low base quality (called in the
    # tumor, present but failing the quality filter in the normal)
    lowq = plant_variants(g, rng, 4e-4, 0.0, lambda r: 0.35, avoid=germ + som + loh + art)
    lowq_n = [dataclasses.replace(v, vaf=0.3, vq=12) for v in lowq]
    loh_t = [dataclasses.replace(v, vaf=0.02 if i % 2 == 0 else 1.0) for i, v in enumerate(loh)]
    art_t, art_n = art[0::2], art[1::2]
    tumor = simulate(g, germ + som + loh_t + art_t + lowq, tumor_depth, rng, name_base=0, softclip_frac=0.04,
                     tail_margin=tail_margin)
    normal = simulate(g, germ + loh + art_n + lowq_n, normal_depth, rng, name_base=10_000_000,
                      softclip_frac=0.04, tail_margin=tail_margin)
    if gap is not None:
        end = normal.pos + 150
        normal = subset(normal, (end <= gap[0]) | (normal.pos >= gap[1]))
    return g, (germ, som, loh, art, lowq), tumor, normal


def amplicon_panel(seed: int = 0x5EED0002, n_regions: int = 10_000, genome_len: int = 50_000_000,
                   median_depth: float = 500.0, read_len: int = 150, dup_frac: float = 0.005,
                   max_depth: float = 5000.0, min_depth: float = 50.0):
    """Batched amplicon panel: `n_regions` regions with lengths ~U(100, 2000)
    spread over a `genome_len` contig, per-region depth log-normal (median
    `median_depth`, sigma ln(10)/3, clipped to [min_depth, max_depth]).
    Each region is tiled by amplicons of 250..350 bp; read 1 starts at the
    amplicon start (forward strand), read 2 ends at the amplicon end
    (reverse strand), so the two reads of a pair overlap.  A fraction
    `dup_frac` of pairs is duplicated as exact copies (PCR duplicates, no
    duplicate flag).  Germline SNVs at 1e-3/bp with VAF 0.5 or 1.0;
    substitution errors from the quality model.  Returns (genome, variants,
    reads, regions)."""
    rng = np.random.default_rng(seed)
    L = read_len
    g = make_genome(genome_len, rng)
    lens = rng.integers(100, 2001, size=n_regions)
    slot = genome_len // n_regions
    starts = np.array([i * slot + int(rng.integers(600, max(601, slot - int(lens[i]) - 600)))
                       for i in range(n_regions)])
    regions = [(int(s) + 1, int(s + ln)) for s, ln in zip(starts.tolist(), lens.tolist())]
    depth = np.clip(np.exp(np.log(median_depth) + rng.normal(0, np.log(10) / 3, n_regions)), min_depth, max_depth)
    snv_pos = []
    for a, b in regions:
        k = rng.binomial(b - a + 1, 1e-3)
        snv_pos += sorted(rng.integers(a - 1, b, size=k).tolist())
    variants = [Variant(pos=int(p), kind="snv", ref="ACGT"[int(g[p])], alt="ACGT"[_rand_other(int(g[p]), rng)],
                        vaf=0.5 if rng.random() < 0.7 else 1.0) for p in sorted(set(snv_pos))]
    var_at = {v.pos: v for v in variants}
    # amplicons: (start, end) 0-based half-open, covering each region
    a_lo, a_hi, a_n = [], [], []
    for (a, b), d in zip(regions, depth.tolist()):
        p = a - 1 - 100
        while p < b:
            ln = int(rng.integers(250, 351))
            n_pairs = max(1, int(round(d * ln / (2 * L))))
            a_lo.append(p)
            a_hi.append(p + ln)
            a_n.append(n_pairs)
            p += ln - 60
    a_lo, a_hi, a_n = np.array(a_lo), np.array(a_hi), np.array(a_n)
    frag_lo = np.repeat(a_lo, a_n)
    frag_hi = np.repeat(a_hi, a_n)
    dups = rng.random(frag_lo.shape[0]) < dup_frac
    frag_lo = np.concatenate([frag_lo, frag_lo[dups]])
    frag_hi = np.concatenate([frag_hi, frag_hi[dups]])
    nf = frag_lo.shape[0]
    start = np.concatenate([frag_lo, frag_hi - L])
    rev = np.concatenate([np.zeros(nf, bool), np.ones(nf, bool)])
    mate = np.concatenate([frag_hi - L, frag_lo])
    isize = np.concatenate([frag_hi - frag_lo, frag_lo - frag_hi])
    is_r1 = np.concatenate([np.ones(nf, bool), np.zeros(nf, bool)])
    frag = np.concatenate([np.arange(nf), np.arange(nf)])
    n = 2 * nf
    seq = g[start[:, None] + np.arange(L)[None, :]]
    # germline SNVs: one haplotype draw per fragment (both reads of a pair agree)
    for p, v in var_at.items():
        hit = np.nonzero((start <= p) & (start + L > p))[0]
        if hit.size == 0:
            continue
        carry_f = rng.random(nf) < v.vaf
        c = hit[carry_f[frag[hit]]]
        seq[c, p - start[c]] = "ACGT".index(v.alt)
    # exact duplicates keep their original's bases and qualities
    qual = _qualities(n, L, rng)
    qual[rev] = qual[rev][:, ::-1]
    err = rng.random((n, L)) < np.power(10.0, -qual.astype(np.float64) / 10.0)
    seq = np.where(err, (seq + rng.integers(1, 4, size=(n, L))) % 4, seq).astype(np.uint8)
    n_orig = nf - int(dups.sum())
    src = np.nonzero(dups)[0]
    for half in (0, nf):
        seq[half + n_orig:half + nf] = seq[half + src]
        qual[half + n_orig:half + nf] = qual[half + src]
    codes = CODE_OF[seq]
    mapq = np.full(n, 60, dtype=np.uint8)
    flag = (1 | 2 | np.where(rev, 16, 32) | np.where(is_r1, 64, 128)).astype(np.uint16)
    ref_win = CODE_OF[g[start[:, None] + np.arange(L)[None, :]]]
    nm = (codes != ref_win).sum(axis=1).astype(np.int32)
    order = np.lexsort((frag, start))
    return g, variants, _pack("ctg", genome_len, order, start, flag, mapq, mate, isize, nm, [None] * n, codes, qual,
                              frag, L), regions


def dense_multi(seed: int = 0x5EED00D0, length: int = 60_000, depth: float = 60.0):
    """A small contig with dense SNV/MNV/indel planting, more soft clips and
    reads kept away from the contig end, for exercising every pileup path."""
    rng = np.random.default_rng(seed)
    g = make_genome(length, rng, homopolymer_rate=0.02)
    vs = plant_variants(g, rng, 4e-3, 1e-3, lambda r: r.choice([0.2, 0.5, 1.0]), mnv_frac=0.2, spacing=12)
    rs = simulate(g, vs, depth, rng, softclip_frac=0.06, n_rate=1e-3, tail_margin=300)
    return g, vs, rs


# --------------------------------------------------------------------------
# native generator (rv_synth.cpp -> librvsynth.so) for the large workloads
# --------------------------------------------------------------------------
_KIND_CODE = {"snv": 0, "mnv": 1, "ins": 2, "del": 3}
_native = None


def _native_lib():
    global _native
    if _native is None:
        import ctypes as C
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "librvsynth.so")
        if not os.path.exists(path):
            from . import build
            build.build()
        L = C.CDLL(path)
        L.rvs_region_reads.restype = C.c_int64
        L.rvs_region_reads.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.rvs_simulate_region.restype = C.c_int64
        L.rvs_simulate_region.argtypes = ([C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int64] +
                                          [C.c_void_p] * 11)
        L.rvs_max_ops.restype = C.c_int
        _native = L
    return _native


_VAR_DT = np.dtype([("pos", np.int64), ("kind", np.int32), ("ref_len", np.int32), ("alt_off", np.int32),
                    ("alt_len", np.int32), ("vaf", np.float64), ("strand_bias", np.float64), ("strand", np.int32),
                    ("vq", np.int32)], align=True)
_PAR_DT = np.dtype([("seed", np.uint64), ("read_len", np.int32), ("amplicon", np.int32), ("depth", np.float64),
                    ("lo", np.int64), ("hi", np.int64), ("insert_mean", np.float64), ("insert_sd", np.float64),
                    ("softclip_frac", np.float64), ("mapq0_frac", np.float64), ("n_rate", np.float64),
                    ("artifact_rate", np.float64), ("artifact_q", np.int32), ("tail_margin", np.int32),
                    ("name_base", np.int64), ("dup_frac", np.float64)], align=True)


def _variant_table(variants: list[Variant]):
    tab = np.zeros(len(variants), dtype=_VAR_DT)
    alt = bytearray()
    for i, v in enumerate(variants):
        tab[i]["pos"] = v.pos
        tab[i]["kind"] = _KIND_CODE[v.kind]
        tab[i]["ref_len"] = len(v.ref) if v.kind == "del" else max(len(v.alt), 1)
        tab[i]["alt_off"] = len(alt)
        tab[i]["alt_len"] = len(v.alt)
        tab[i]["vaf"] = v.vaf
        tab[i]["strand_bias"] = v.strand_bias
        tab[i]["strand"] = v.strand
        tab[i]["vq"] = v.vq or 0
        alt += bytes("ACGT".index(c) for c in v.alt)
    return tab, np.frombuffer(bytes(alt) or b"\0", dtype=np.uint8)


def simulate_regions(genome: np.ndarray, variants: list[Variant], spans: list[tuple[int, int]], depth, seed: int,
                     contig: str = "ctg", read_len: int = 150, softclip_frac: float = 0.02,
                     mapq0_frac: float = 0.05, n_rate: float = 2e-4, artifact_rate: float = 0.0,
                     artifact_q: int = 0, name_base: int = 0, amplicons=None, dup_frac: float = 0.0,
                     threads: int | None = None, span_ids: list[int] | None = None) -> ReadSet:
    """Reads over disjoint, ascending `spans` (0-based, half-open) from the
    native generator, one seeded stream per span (`depth` a number or one
    per span): 2x`read_len` pairs with fragments over each span (or, with
    `amplicons` = per span a list of (lo, hi, pairs), the given amplicons),
    the same error / quality / clip / MAPQ model as `simulate`.  Spans must
    be far enough apart that their reads do not interleave (the result is
    the concatenation of the per-span sorted reads).  `span_ids` picks the
    spans to generate (each span's stream is seeded by its index, so a span
    gives the same reads alone as in the whole set).  Returns a ReadSet with
    packed bases (seq4 None)."""
    import concurrent.futures as cf
    import ctypes as C
    import os
    L = _native_lib()
    G = genome.shape[0]
    g = np.ascontiguousarray(genome, dtype=np.uint8)
    vt, alt = _variant_table(sorted(variants, key=lambda v: v.pos))
    vpos = vt["pos"]
    depths = [float(depth)] * len(spans) if np.isscalar(depth) else [float(d) for d in depth]
    ids = list(range(len(spans))) if span_ids is None else list(span_ids)
    pars, counts, amp = [], [], []
    for i in ids:
        lo, hi = spans[i]
        p = np.zeros(1, dtype=_PAR_DT)
        p["seed"] = np.uint64((seed * 0x9E3779B97F4A7C15 + i * 0xD1B54A32D192ED03) % (1 << 64))
        p["read_len"] = read_len
        p["depth"] = depths[i]
        p["lo"], p["hi"] = lo, hi
        p["insert_mean"], p["insert_sd"] = 350.0, 50.0
        p["softclip_frac"], p["mapq0_frac"], p["n_rate"] = softclip_frac, mapq0_frac, n_rate
        p["artifact_rate"], p["artifact_q"] = artifact_rate, artifact_q
        p["name_base"] = name_base + i * 100_000_000
        p["dup_frac"] = dup_frac
        a_lo = a_hi = a_n = None
        if amplicons is not None and i < len(amplicons):
            p["amplicon"] = 1
            arr = np.array(amplicons[i], dtype=np.int64).reshape(-1, 3)
            a_lo, a_hi, a_n = (np.ascontiguousarray(arr[:, 0]), np.ascontiguousarray(arr[:, 1]),
                               np.ascontiguousarray(arr[:, 2].astype(np.int32)))
        amp.append((a_lo, a_hi, a_n))
        pars.append(p)
        counts.append(int(L.rvs_region_reads(p.ctypes.data, a_n.ctypes.data if a_n is not None else None,
                                             len(a_n) if a_n is not None else 0)))
    n = sum(counts)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    stride = (read_len + 31) // 32 * 32
    pos = np.empty(n, np.int32)
    mpos = np.empty(n, np.int32)
    isize = np.empty(n, np.int32)
    nm = np.empty(n, np.int32)
    flag = np.empty(n, np.uint16)
    mapq = np.empty(n, np.uint8)
    ncig = np.empty(n, np.uint16)
    name = np.empty(n, np.int64)
    packed = np.empty(n * stride // 2, np.uint8)
    qual = np.empty(n * stride, np.uint8)
    max_ops = int(L.rvs_max_ops())
    cigars = [None] * len(ids)

    def one(i):
        lo, hi = spans[ids[i]]
        a = int(np.searchsorted(vpos, lo - 400))
        b = int(np.searchsorted(vpos, hi + 400))
        sub = np.ascontiguousarray(vt[a:b])
        k0, k1 = int(off[i]), int(off[i + 1])
        cg = np.empty(max(1, (k1 - k0) * max_ops), np.uint32)
        a_lo, a_hi, a_n = amp[i]
        ptr = lambda x: x.ctypes.data if x is not None else None  # noqa: E731
        nw = L.rvs_simulate_region(
            g.ctypes.data, G, sub.ctypes.data, len(sub), alt.ctypes.data, pars[i].ctypes.data, ptr(a_lo), ptr(a_hi),
            ptr(a_n), len(a_n) if a_n is not None else 0, k1 - k0,
            pos[k0:].ctypes.data, mpos[k0:].ctypes.data, isize[k0:].ctypes.data, nm[k0:].ctypes.data,
            flag[k0:].ctypes.data, mapq[k0:].ctypes.data, ncig[k0:].ctypes.data, name[k0:].ctypes.data,
            packed[k0 * stride // 2:].ctypes.data, qual[k0 * stride:].ctypes.data, cg.ctypes.data)
        if nw < 0:
            raise RuntimeError(f"native generator failed on span {i}")
        cigars[i] = cg[:nw].copy()

    with cf.ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        list(ex.map(one, range(len(ids))))
    cigar = np.concatenate(cigars) if cigars else np.zeros(0, np.uint32)
    cig_off = np.zeros(n, dtype=np.uint32)
    if n:
        cig_off[1:] = np.cumsum(ncig[:-1].astype(np.uint64)).astype(np.uint32)
    del C
    return ReadSet(contig=contig, contig_len=int(G), pos=pos, flag=flag, mapq=mapq, mpos=mpos, isize=isize, nm=nm,
                   n_cigar=ncig, cig_off=cig_off, cigar=cigar, l_qseq=np.full(n, read_len, dtype=np.int32),
                   base_off=np.arange(n, dtype=np.uint64) * np.uint64(stride), seq4=None, qual=qual, name_id=name,
                   packed=packed)


def deep_somatic_panel(seed: int = 0x5EED0003, n_regions: int = 400, region_len: int = 5000, gap: int = 1000,
                       tumor_depth: float = 5000.0, normal_depth: float = 1000.0, threads: int | None = None,
                       only: list[int] | None = None):
    """Deep targeted somatic panel: `n_regions` regions of `region_len` bp
    (2 Mb for 400 x 5 kb) on one contig, `gap` bp apart; tumor 5000x and
    normal 1000x 2x150 pairs (native generator).  Germline SNVs 1e-3/bp
    (VAF 0.5 or 1.0) and indels 1e-4/bp in both samples; low-VAF somatic SNVs
    (1e-4/bp, 10 % MNVs) and indels (2e-5/bp) with VAF ~log-uniform(0.001,
    0.05) in the tumor; oxidation-like C>A artifacts at 1e-4 per C base with
    quality 20 in both samples.  Returns (genome, (germline, somatic),
    tumor, normal, regions) with regions 1-based inclusive.  With `only` (a
    list of region indexes) only those regions' reads are generated; each
    region's reads are the same as in the whole panel (one seeded stream per
    region)."""
    rng = np.random.default_rng(seed)
    glen = n_regions * (region_len + gap) + gap
    g = make_genome(glen, rng)
    regions = [(gap + i * (region_len + gap) + 1, gap + i * (region_len + gap) + region_len)
               for i in range(n_regions)]
    germ = plant_variants(g, rng, 1e-3, 1e-4, lambda r: 0.5 if r.random() < 0.7 else 1.0)
    lo_v, hi_v = np.log(0.001), np.log(0.05)
    som = plant_variants(g, rng, 1e-4, 2e-5, lambda r: float(np.exp(r.uniform(lo_v, hi_v))), mnv_frac=0.1,
                         avoid=germ)
    spans = [(a - 1, b) for a, b in regions]
    idx = list(range(n_regions)) if only is None else sorted(only)
    tumor = simulate_regions(g, germ + som, spans, tumor_depth, seed=seed * 2 + 1, artifact_rate=1e-4,
                             artifact_q=20, threads=threads, span_ids=idx)
    normal = simulate_regions(g, germ, spans, normal_depth, seed=seed * 2 + 2, artifact_rate=1e-4, artifact_q=20,
                              name_base=1 << 40, threads=threads, span_ids=idx)
    return g, (germ, som), tumor, normal, regions


def amplicon_panel_native(seed: int = 0x5EED0002, n_regions: int = 10_000, genome_len: int = 50_000_000,
                          median_depth: float = 500.0, read_len: int = 150, dup_frac: float = 0.005,
                          max_depth: float = 5000.0, min_depth: float = 50.0, threads: int | None = None,
                          only: list[int] | None = None):
    """The batched amplicon panel (the shape of `amplicon_panel`) from the
    native generator, for its full size (10,000 regions, ~47 M reads):
    regions of U(100, 2000) bp, one per genome_len / n_regions slot; per-region
    depth log-normal (median `median_depth`, sigma ln(10)/3, clipped to
    [min_depth, max_depth]); each region tiled by amplicons of 250..350 bp
    with read 1 at the amplicon start (forward) and read 2 ending at its end
    (reverse); a fraction `dup_frac` of pairs duplicated as exact copies;
    germline SNVs at 1e-3/bp with VAF 0.5 or 1.0, carried per read.  Returns
    (genome, variants, reads, regions of the reads); `only` picks regions
    (each region's reads are the same as in the whole panel)."""
    rng = np.random.default_rng(seed)
    L = read_len
    g = make_genome(genome_len, rng)
    lens = rng.integers(100, 2001, size=n_regions)
    slot = genome_len // n_regions
    starts = np.array([i * slot + int(rng.integers(600, max(601, slot - int(lens[i]) - 600)))
                       for i in range(n_regions)])
    regions = [(int(s) + 1, int(s + ln)) for s, ln in zip(starts.tolist(), lens.tolist())]
    depth = np.clip(np.exp(np.log(median_depth) + rng.normal(0, np.log(10) / 3, n_regions)), min_depth, max_depth)
    variants = []
    for a, b in regions:
        k = rng.binomial(b - a + 1, 1e-3)
        for p in sorted(set(rng.integers(a - 1, b, size=k).tolist())):
            variants.append(Variant(pos=int(p), kind="snv", ref="ACGT"[int(g[p])],
                                    alt="ACGT"[_rand_other(int(g[p]), rng)],
                                    vaf=0.5 if rng.random() < 0.7 else 1.0))
    amplicons, spans = [], []
    for (a, b), d in zip(regions, depth.tolist()):
        p = a - 1 - 100
        amps = []
        while p < b:
            ln = int(rng.integers(250, 351))
            amps.append((p, p + ln, max(1, int(round(d * ln / (2 * L))))))
            p += ln - 60
        amplicons.append(amps)
        spans.append((a - 1 - 100, p + 350))
    idx = list(range(n_regions)) if only is None else sorted(only)
    rs = simulate_regions(g, variants, spans, 0.0, seed=seed * 2 + 3, read_len=L, softclip_frac=0.0,
                          mapq0_frac=0.0, n_rate=0.0, amplicons=amplicons, dup_frac=dup_frac, threads=threads,
                          span_ids=idx)
    return g, variants, rs, [regions[i] for i in idx]
