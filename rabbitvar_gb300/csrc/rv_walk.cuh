// Device CIGAR walker: the per-read state machine of CigarParser::parseCigar
// (src/parseCigar.cpp:497-974) and its helpers, parameterised by a Sink that
// decides where observations go (shared-memory tile histogram, direct global
// cells for the in-order exact walker, or a probe that only watches for one
// key).  One thread walks one read.
#pragma once
#include "rv_internal.h"
#include "rv_cigar.cuh"
#include "rv_hash.cuh"

namespace rv {

__device__ __forceinline__ int cig_op(uint32_t c) { return (int)(c & 15u); }
__device__ __forceinline__ int cig_len(uint32_t c) { return (int)(c >> 4); }

__device__ __constant__ char kNt16Dev[17] = "=ACMGRSVTWYHKDBN";

// 'A','C','G','T' -> 0..3, anything else -> -1
__device__ __forceinline__ int base_index(char c) {
    switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1;
    }
}

struct KeyBuf {
    char b[kMaxKey];
    int n;
    bool overflow;
    __device__ void clear() { n = 0; overflow = false; }
    __device__ void push(char c) {
        if (n < kMaxKey) b[n++] = c; else overflow = true;
    }
    __device__ void push_int(int v) {
        char t[12];
        int k = 0;
        if (v < 0) { push('-'); v = -v; }
        do { t[k++] = (char)('0' + v % 10); v /= 10; } while (v);
        while (k) push(t[--k]);
    }
};

// View of one read of the batch.
struct ReadView {
    const uint8_t *seq;   // packed 4-bit
    const uint8_t *qual;
    const uint32_t *cig;
    int lseq, n_cigar;
    __device__ char base(int i) const {
        uint8_t b = __ldg(seq + (i >> 1));
        return kNt16Dev[(i & 1) ? (b & 15) : (b >> 4)];
    }
    // quality byte i; index -1 is the byte before the quals in a BAM record
    // (the last packed-sequence byte), indexes past the end read as 0
    __device__ int q(int i) const {
        if (i < 0) return __ldg(seq + ((lseq + 1) >> 1) - 1);
        if (i >= lseq) return 0;
        return __ldg(qual + i);
    }
    // CIGAR word k; words past the last op are the bytes that follow the
    // CIGAR in a BAM record (packed bases, then quals)
    __device__ uint32_t word(int k) const {
        if (k < n_cigar) return __ldg(cig + k);
        int off = 4 * (k - n_cigar);
        uint32_t v = 0;
        int nseqb = (lseq + 1) >> 1;
        for (int j = 3; j >= 0; j--) {
            int o = off + j;
            uint32_t byte = o < nseqb ? __ldg(seq + o) : (o - nseqb < lseq ? __ldg(qual + (o - nseqb)) : 0u);
            v = (v << 8) | byte;
        }
        return v;
    }
};

__device__ __forceinline__ uint32_t pick_word(const uint4 &v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// BAM 4-bit code -> 0..3 for A/C/G/T, -1 otherwise
__device__ __forceinline__ int code_base(int code) {
    // the one-bit codes 1, 2, 4, 8 are A, C, G, T
    return __popc((unsigned)code) == 1 ? __ffs(code) - 1 : -1;
}

// Sinks without an inline fast path for single-base observations.
// Reference base code for the per-base loop: 0-3 for A/C/G/T (base_index),
// 5 for 'N', 4 for anything else.
__device__ __forceinline__ int ref_code_of(char c) {
    const int b = base_index(c);
    return b >= 0 ? b : (c == 'N' ? 5 : 4);
}

struct NoFast {
    __device__ __forceinline__ char ref(const char *refp, int p) const { return __ldg(refp + p - 1); }
    __device__ __forceinline__ int ref_code(const char *refp, int p) const { return ref_code_of(__ldg(refp + p - 1)); }
    __device__ __forceinline__ bool emit(int, int, int, int, int, int, int) const { return false; }
};

// Observation destined for an allele key.
struct Obs {
    int dir;
    int tp;          // read position contribution (meanPosition)
    double q;        // base quality contribution (meanQuality)
    int mapq;
    int nm;
    bool std_rel;    // participates in pstd/qstd
    bool creates;    // counts toward positionTo*Count / mnp
};

template <class Sink>
struct Walker {
    const DevParams &P;
    Sink &S;
    const Region &R;
    const char *ref;
    int ref_len;
    ReadView rv;
    int64_t read_idx;
    // CigarParser state
    int start, offset, cel, rpis, rpes, n_cigar;
    // cleanupCigar (src/parseCigar.cpp:1858-1892) turns the insertions before
    // the first and after the last M/=/X op into soft clips; applied on read
    int lead_end, trail_start;
    // M-loop iteration state shared with the out-of-line slow iteration
    int m_i, m_ci, m_nmoff, m_moffset, m_cop;
    bool m_dir;
    int m_mapq, m_nom, m_rlen, m_tlen;
    KeyBuf key;
    // -k 1: the rewritten CIGAR (written over the record's first words), and
    // the record's own word count
    uint32_t mod_w[kCigTok];
    int mod_n;

    __device__ Walker(const DevParams &p, Sink &s, const Region &r, const char *rf, int rl)
        : P(p), S(s), R(r), ref(rf), ref_len(rl) {}

    // record memory word k: the rewritten words first, then the record's own
    // words and the bytes after them
    __device__ uint32_t mem(int k) const {
        if (k < mod_n) return mod_w[k];
        return k < rv.n_cigar ? __ldg(rv.cig + k) : rv.word(k);
    }
    __device__ uint32_t W(int k) const {
        if (k >= n_cigar) return mem(k);
        uint32_t w = mem(k);
        if ((w & 15u) == 1u && (k < lead_end || k > trail_start)) w = (w & ~15u) | 4u;
        return w;
    }
    // reference, bases and qualities as CigarEdit reads them
    struct EditAcc {
        const Walker *w;
        __device__ bool has(int p) const { return w->has(p); }
        __device__ char at(int p) const { return w->at(p); }
        __device__ char base(int i) const { return i >= 0 && i < w->rv.lseq ? w->rv.base(i) : (char)0; }
        __device__ int q(int i) const { return w->rv.q(i); }
        __device__ int lseq() const { return w->rv.lseq; }
    };
    // CigarModifier (src/parseCigar.cpp:547-571) of a read whose CIGAR is
    // one M op of length L >= 8 (most reads): no indel rule applies, so the
    // rewrite is the two end scans, captureMisSoftly3Mismatches (:531-566)
    // and then combineBeginDigM (:412-439), with the same reference lookups as
    // rewrite_cigar and no token lists; at most 3 bases become a soft clip at
    // either end.
    __device__ __forceinline__ void rewrite_single_m(int L, int &position) {
        int mch = L, tail = 0, head = 0;
        {
            // back_scan(L, position + L, L)
            const int refoff = position + L;
            int rn = 0, rrn = 0, rmch = 0;
            while (rrn < mch && rn < mch) {
                const int p = refoff - rrn - 1;
                if (!has(p)) break;
                if (at(p) != rv.base(L - rrn - 1)) { rn = rrn + 1; rmch = 0; }
                else rmch++;
                rrn++;
                if (rmch >= 3) break;
            }
            if (rn > 0 && rn <= 3) { mch -= rn; tail = rn; }
        }
        {
            int rn = 0, rrn = 0, rmch = 0;
            while (rrn < mch && rn < mch) {
                const int p = position + rrn;
                if (!has(p)) break;
                if (at(p) != rv.base(rrn)) { rn = rrn + 1; rmch = 0; }
                else rmch++;
                rrn++;
                if (rmch >= 3) break;
            }
            if (rn > 0 && rn <= 3) { mch -= rn; head = rn; position += rn; }
        }
        if (!head && !tail) return;
        int k = 0;
        if (head) mod_w[k++] = ((uint32_t)head << 4) | 4u;
        mod_w[k++] = (uint32_t)mch << 4;
        if (tail) mod_w[k++] = ((uint32_t)tail << 4) | 4u;
        mod_n = k;
        n_cigar = k;
    }
    // CigarModifier (src/parseCigar.cpp:547-571); false when the read is not supported
    __device__ __noinline__ bool rewrite_cigar(int idl, int &position) {
        const int n0 = rv.n_cigar;
        if (n0 > kCigTok || cig_op(__ldg(rv.cig)) == 2) return false;  // the leading-D pointer shift (:249)
        EditAcc acc{this};
        CigarEdit<EditAcc> ce{acc, CigTok(), position};
        CigTok orig;
        orig.n = 0;
        orig.bad = false;
        int nm = n0;
        if (__ldg(rv.cig + n0 - 1) == 2u) nm--;  // whole-word compare (:251)
        ce.t.n = 0;
        ce.t.bad = false;
        for (int k = 0; k < n0; k++) {
            const uint32_t w = __ldg(rv.cig + k);
            orig.len[k] = cig_len(w);
            orig.op[k] = op_char(w);
            if (orig.op[k] == '?') return false;
        }
        orig.n = n0;
        for (int k = 0; k < nm; k++) {
            uint32_t w = __ldg(rv.cig + k);
            if (k == 0 && cig_op(w) == 1) w = (w & ~15u) | 2u;  // a leading I becomes D (:253-255)
            if (k == nm - 1 && w == 1u) w = 2u;                 // whole-word compare (:256-258)
            ce.t.len[k] = cig_len(w);
            ce.t.op[k] = op_char(w);
        }
        ce.t.n = nm;
        ce.run(idl);
        if (ce.t.bad) return false;
        if (ce.t.eq(orig)) return true;
        for (int k = 0; k < ce.t.n; k++) mod_w[k] = ((uint32_t)ce.t.len[k] << 4) | op_code(ce.t.op[k]);
        mod_n = ce.t.n;
        n_cigar = ce.t.n;
        position = ce.position;
        return true;
    }
    __device__ int cop(int k) const { return cig_op(W(k)); }
    __device__ int clen(int k) const { return cig_len(W(k)); }

    // reference lookups with the window semantics of the reference's map
    __device__ bool has(int p) const { return (p >= R.ws && p <= R.we) || S.phantom(p); }
    __device__ char at(int p) const { return (p >= R.ws && p <= R.we) ? ref[p - 1] : (char)0; }
    __device__ char idx(int p) {  // operator[]: inserts a 0 entry when missing
        if (p >= R.ws && p <= R.we) return ref[p - 1];
        S.touch_phantom(p);
        return 0;
    }
    __device__ bool has_eq(char c, int p) const { return has(p) && at(p) == c; }
    __device__ bool has_ne(char c, int p) const { return has(p) && at(p) != c; }

    __device__ int tp_of(int rlen) const { return rpes < rlen - rpes ? rpes + 1 : rlen - rpes; }

    __device__ bool trim(bool dir, int tlen) const {
        if (P.trim_bases_after != 0) {
            if (!dir) return rpis > P.trim_bases_after;
            return tlen - rpis > P.trim_bases_after;
        }
        return false;
    }

    // A single-base key: A/C/G/T go to the per-position cells, whose
    // creation count is also the position's coverage increment; any other
    // letter (IUPAC codes) is a string key plus an explicit coverage bump.
    __device__ void single(int p, char ch, const Obs &o) {
        int b = base_index(ch);
        if (b >= 0) {
            S.single(p, b, o, read_idx);
        } else {
            char kb[1] = {ch};
            S.event(KIND_NONINS, p, kb, 1, o, read_idx);
            S.cov(p, 1);
        }
    }

    // findOffset: src/parseCigar.cpp:208-256
    __device__ int find_offset(int refp, int readp, int cl, int &tnm, int &qsum) {
        int off = 0, vsn = 0;
        tnm = 0;
        for (int vi = 0; vsn <= P.vext && vi < cl; vi++) {
            if (rv.base(readp + vi) == 'N') break;
            if (rv.q(readp + vi) < P.goodq) break;
            if (has(refp + vi)) {
                if (rv.base(readp + vi) != at(refp + vi)) { off = vi + 1; tnm++; vsn = 0; }
                else vsn++;
            }
        }
        qsum = 0;
        if (off > 0) {
            for (int i = readp; i < readp + off; i++) qsum += rv.q(i);
            for (int i = 0; i < off; i++) S.cov(refp + i, 1);
        }
        return off;
    }

    __device__ bool indel_next_matched(int ci) const {  // src/parseCigar.cpp:1817-1826
        return P.local_realign && n_cigar > ci + 2 && clen(ci + 1) <= P.vext && cop(ci + 1) == 0 &&
               (cop(ci + 2) == 1 || cop(ci + 2) == 2) && cop(ci + 3) != 1 && cop(ci + 3) != 2;
    }
    __device__ bool next_matched(int ci) const { return P.local_realign && n_cigar > ci + 1 && cop(ci + 1) == 0; }
    __device__ bool next_after_num_matched(int ci, int number) const { return n_cigar > ci + number && cop(ci + 1) == 0; }

    __device__ void append_read(int from, int len) {
        for (int i = 0; i < len; i++) key.push(rv.base(from + i));
    }

    // appendSegments: src/parseCigar.cpp:1756-1815
    __device__ void append_segments(int ci, long long &qsum, int &qcnt, int mlen, int indel_len, int begin, bool is_ins) {
        key.push('#');
        append_read(begin, mlen);
        for (int i = begin; i < begin + mlen; i++) qsum += rv.q(i);
        key.push('^');
        if (cop(ci + 2) == 1) append_read(begin + mlen, indel_len);
        else key.push_int(indel_len);
        if (cop(ci + 2) == 1) {
            for (int i = begin + mlen; i < begin + mlen + indel_len; i++) qsum += rv.q(i);
            qcnt += indel_len;
        } else if (is_ins) {
            qsum += rv.q(begin + mlen);
            qcnt += 1;
        }
    }

    // addCnt-style single observation for soft-clip re-alignment
    __device__ Obs plain_obs(bool dir, int rp, int bq, int mapq, int nom) const {
        Obs o;
        o.dir = dir; o.tp = rp; o.q = bq; o.mapq = mapq; o.nm = nom; o.std_rel = false; o.creates = false;
        return o;
    }

    // process_softclip: src/parseCigar.cpp:1112-1301
    __device__ __noinline__ void softclip(int ci, bool dir, int mapq, int nom, int position, int tlen) {
        if (ci == 0) {
            while (cel - 1 >= 0 && start - 1 > 0 && start - 1 <= ref_len && has_eq(rv.base(cel - 1), start - 1) &&
                   rv.q(cel - 1) > 10) {
                single(start - 1, idx(start - 1), plain_obs(dir, cel, rv.q(cel - 1), mapq, nom));
                start--;
                cel--;
            }
            if (cel > 0) {
                int sumq = 0, nhq = 0, nlq = 0;
                for (int si = cel - 1; si >= 0; si--) {
                    if (rv.base(si) == 'N') break;
                    int bq = rv.q(si);
                    if (bq <= 12) nlq++;
                    if (nlq > 1) break;
                    sumq += bq;
                    nhq++;
                }
                if (nhq >= 1 && nhq > nlq && start >= R.start && start <= R.end) {
                    for (int si = cel - 1; cel - si <= nhq; si--) {
                        char kb[3];
                        int idx_ = cel - 1 - si;
                        kb[0] = (char)(idx_ & 0xff); kb[1] = (char)(idx_ >> 8); kb[2] = rv.base(si);
                        Obs so = plain_obs(dir, si - (cel - nhq), rv.q(si), mapq, nom);
                        so.creates = true;  // Sclip.nt[idx][ch] counts every observation
                        S.event(KIND_SC5_SEQ, start, kb, 3, so, read_idx);
                    }
                    Obs a = plain_obs(dir, cel, 0, mapq, nom);
                    a.q = sumq / (double)nhq;
                    S.event(KIND_SC5, start, nullptr, 0, a, read_idx);
                }
            }
            cel = clen(ci);
        } else if (ci == n_cigar - 1) {
            while (rpis < rv.lseq && has_eq(rv.base(rpis), start) && rv.q(rpis) > 10) {
                single(start, at(start), plain_obs(dir, tlen - rpes, rv.q(rpis), mapq, nom));
                rpis++;
                start++;
                cel--;
                rpes++;
            }
            if (rpis < rv.lseq) {
                int sumq = 0, nhq = 0, nlq = 0;
                for (int si = 0; si < cel; si++) {
                    if (rv.base(rpis + si) == 'N') break;
                    int bq = rv.q(rpis + si);
                    if (bq <= 12) nlq++;
                    if (nlq > 1) break;
                    sumq += bq;
                    nhq++;
                }
                if (nhq >= 1 && nhq > nlq && start >= R.start && start <= R.end) {
                    for (int si = 0; si < nhq; si++) {
                        char kb[3];
                        kb[0] = (char)(si & 0xff); kb[1] = (char)(si >> 8); kb[2] = rv.base(rpis + si);
                        Obs so = plain_obs(dir, nhq - si, rv.q(rpis + si), mapq, nom);
                        so.creates = true;
                        S.event(KIND_SC3_SEQ, start, kb, 3, so, read_idx);
                    }
                    Obs a = plain_obs(dir, cel, 0, mapq, nom);
                    a.q = sumq / (double)nhq;
                    S.event(KIND_SC3, start, nullptr, 0, a, read_idx);
                }
            }
        }
        rpis += cel;
        offset = 0;
        start = position;
    }

    // adjInsPos: include/VariationUtils.h:99-113, on key.b[1..n) (after '+')
    __device__ int adj_ins_pos(int bi, char *ins, int len, char *rot) {
        int n = 1;
        while (idx(bi) == ins[len - n]) {
            n++;
            if (n > len) n = 1;
            bi--;
        }
        int k = 0;
        if (n > 1) {
            for (int i = len - (n - 1); i < len; i++) rot[k++] = ins[i];
            for (int i = 0; i < len - (n - 1); i++) rot[k++] = ins[i];
        } else {
            for (int i = 0; i < len; i++) rot[k++] = ins[i];
        }
        return bi;
    }

    // process_insertion: src/parseCigar.cpp:1303-1523
    __device__ __noinline__ int insertion(int ci, bool dir, int mapq, int nom, int position, int rlen) {
        if ((n_cigar > ci + 1 && cop(ci + 1) == 3) || (ci > 0 && cop(ci - 1) == 3)) {
            rpis += cel;
            return ci;
        }
        key.clear();
        key.push('+');
        append_read(rpis, cel);
        long long qsum = 0;
        int qcnt = 0;
        for (int i = rpis; i < rpis + cel; i++) qsum += rv.q(i);
        qcnt += cel;
        int ss_from = -1, ss_len = 0;  // the matched tail appended after '&'
        int multoffs = 0, multoffp = 0, nmoff = 0;
        if (indel_next_matched(ci)) {
            int mlen = clen(ci + 1), il = clen(ci + 2);
            int begin = rpis + cel;
            append_segments(ci, qsum, qcnt, mlen, il, begin, true);
            multoffs += mlen + (cop(ci + 2) == 2 ? il : 0);
            multoffp += mlen + (cop(ci + 2) == 1 ? il : 0);
            int ci6 = n_cigar > ci + 3 ? clen(ci + 3) : 0;
            if (ci6 != 0 && cop(ci + 3) == 0) {
                int tnm, qs;
                offset = find_offset(start + multoffs, rpis + cel + multoffp, ci6, tnm, qs);
                ss_from = rpis + cel + multoffp;
                ss_len = offset;
                qsum += qs;
                qcnt += offset;
            }
            ci += 2;
        } else if (next_matched(ci)) {
            int vsn = 0;
            for (int vi = 0; vsn <= P.vext && vi < clen(ci + 1); vi++) {
                if (rv.base(rpis + cel + vi) == 'N') break;
                if (rv.q(rpis + cel + vi) < P.goodq) break;
                if (has(start + vi)) {
                    if (rv.base(rpis + cel + vi) != at(start + vi)) { offset = vi + 1; nmoff++; vsn = 0; }
                    else vsn++;
                }
            }
            if (offset != 0) {
                ss_from = rpis + cel;
                ss_len = offset;
                for (int i = rpis + cel; i < rpis + cel + offset; i++) qsum += rv.q(i);
                qcnt += offset;
                for (int osi = 0; osi < offset; osi++) S.cov(start + osi, 1);
            }
        }
        if (offset > 0) {
            key.push('&');
            append_read(ss_from, ss_len);
        }
        bool has_n = false;
        for (int i = 1; i < key.n; i++) if (key.b[i] == 'N') has_n = true;
        if (start - 1 >= R.start && start - 1 <= R.end && !has_n) {
            if (key.overflow) { S.error(ERR_KEY_TOO_LONG); }
            int inspos = start - 1;
            bool acgt = key.n > 1;
            for (int i = 1; i < key.n; i++) if (base_index(key.b[i]) < 0) acgt = false;
            if (acgt) {
                char rot[kMaxKey];
                int bi = adj_ins_pos(start - 1, key.b + 1, key.n - 1, rot);
                if (rpis - 1 - (start - 1 - bi) > 0) {
                    inspos = bi;
                    for (int i = 1; i < key.n; i++) key.b[i] = rot[i - 1];
                }
            }
            int tp = tp_of(rlen);
            double tmpq = (double)qsum / qcnt;
            Obs o;
            o.dir = dir; o.tp = tp; o.q = tmpq; o.mapq = mapq; o.nm = nom - nmoff; o.std_rel = true; o.creates = true;
            S.event(KIND_INS, inspos, key.b, key.n, o, read_idx);
            int index = rpis - 1 - (start - 1 - inspos);
            char rb = index >= 0 ? rv.base(index) : (char)0;
            if (inspos > position && index >= 0 && has_eq(rb, inspos)) {
                int b = base_index(rb);
                if (b >= 0) S.subtract(inspos, b, dir, tp, rv.q(index), mapq, nom - nmoff, read_idx, ci);
                else S.error(ERR_UNSUPPORTED);
            }
            if (ci == 1 && (cop(0) == 4 || cop(0) == 5)) {
                // ttref (src/parseCigar.cpp:1497-1515) copies the insertion's pstd/qstd
                // flags; cleanupCigar turns an insertion after a leading clip into a
                // clip, so this branch is not reached for well-formed records.
                S.error(ERR_UNSUPPORTED);
            }
        }
        rpis += cel + offset + multoffp;
        rpes += cel + offset + multoffp;
        start += offset + multoffs;
        return ci;
    }

    // process_deletion + addVariationForDeletion: src/parseCigar.cpp:1525-1727, 1036-1082
    __device__ __noinline__ int deletion(int ci, bool dir, int mapq, int nom, int rlen) {
        if ((n_cigar > ci && cop(ci + 1) == 3) || (ci > 1 && cop(ci - 1) == 3)) {
            rpis += cel;
            return ci;
        }
        key.clear();
        key.push('-');
        key.push_int(cel);
        int app_from = -1;
        int qlast = rv.q(rpis - 1);
        long long qsum = 0;
        int qcnt = 0;
        int multoffs = 0, multoffp = 0, nmoff = 0;
        if (indel_next_matched(ci)) {
            int mlen = clen(ci + 1), il = clen(ci + 2);
            append_segments(ci, qsum, qcnt, mlen, il, rpis, false);
            multoffs += mlen + (cop(ci + 2) == 2 ? il : 0);
            multoffp += mlen + (cop(ci + 2) == 1 ? il : 0);
            if (next_after_num_matched(ci, 3)) {
                int vsn = 0, tn = rpis + multoffp, ts = start + multoffs + cel;
                for (int vi = 0; vsn <= P.vext && vi < clen(ci + 3); vi++) {
                    if (rv.base(tn + vi) == 'N') break;
                    if (rv.q(tn + vi) < P.goodq) break;
                    if (has_eq('N', ts + vi)) break;
                    if (has(ts + vi)) {
                        if (rv.base(tn + vi) != at(ts + vi)) { offset = vi + 1; nmoff++; vsn = 0; }
                        else vsn++;
                    }
                }
                if (offset != 0) {
                    app_from = tn;
                    for (int i = tn; i < tn + offset; i++) qsum += rv.q(i);
                    qcnt += offset;
                }
            }
            ci += 2;
        } else if (P.local_realign && n_cigar > ci + 1 && cop(ci + 1) == 1) {
            int il = clen(ci + 1);
            key.push('^');
            append_read(rpis, il);
            for (int i = rpis; i < rpis + il; i++) qsum += rv.q(i);
            qcnt += il;
            multoffp += il;
            ci += 1;
        } else if (next_matched(ci)) {
            int mlen = clen(ci + 1), vsn = 0;
            for (int vi = 0; vsn <= P.vext && vi < mlen; vi++) {
                char sc = rv.base(rpis + vi);
                if (sc == 'N') break;
                if (rv.q(rpis + vi) < P.goodq) break;
                if (has(start + cel + vi)) {
                    char rc = at(start + cel + vi);
                    if (rc == 'N') break;
                    if (sc != rc) { offset = vi + 1; nmoff++; vsn = 0; }
                    else vsn++;
                }
            }
            if (offset != 0) {
                app_from = rpis;
                for (int i = rpis; i < rpis + offset; i++) qsum += rv.q(i);
                qcnt += offset;
            }
        }
        if (offset > 0) {
            key.push('&');
            append_read(app_from, offset);
        }
        if (rpis + offset >= rv.lseq) {
            qsum += qlast;
            qcnt += 1;
        } else {
            int qo = rv.q(rpis + offset);
            qsum += qlast > qo ? qlast : qo;
            qcnt += 1;
        }
        if (start >= R.start && start <= R.end) {
            if (key.overflow) S.error(ERR_KEY_TOO_LONG);
            Obs o;
            o.dir = dir; o.tp = tp_of(rlen); o.q = (double)qsum / qcnt; o.mapq = mapq; o.nm = nom - nmoff;
            o.std_rel = true; o.creates = true;
            S.event(KIND_NONINS, start, key.b, key.n, o, read_idx);
            for (int i = 0; i < cel; i++) S.cov(start + i, 1);
        }
        start += cel + offset + multoffs;
        rpis += offset + multoffp;
        rpes += offset + multoffp;
        return ci;
    }

    // One iteration of the M-op base loop for a base that may start an MNV
    // or a complex indel tail (src/parseCigar.cpp:678-959); the common
    // single-base case is handled inline by walk().
    __device__ __noinline__ void m_iteration() {
            const bool dir = m_dir;
            const int mapq = m_mapq, nom = m_nom, rlen = m_rlen, tlen = m_tlen, c_op = m_cop;
            int &i = m_i, &ci = m_ci, &nmoff = m_nmoff, &moffset = m_moffset;
            bool tr = trim(dir, tlen);
            char ch1 = rv.base(rpis);
            if (ch1 == 'N') {
                start++;
                rpis++;
                rpes++;
                return;
            }
            int q0 = rv.q(rpis);
            long long qv = q0;
            int qbases = 1, qibases = 0;
            bool swd = false;
            int ddlen = 0;
            bool simple = true;   // key is the single base ch1
            // MNV growth: src/parseCigar.cpp:711-767
            if ((start + 1) >= R.start && (start + 1) <= R.end && (i + 1) < cel && qv >= P.goodq &&
                has_ne(ch1, start) && idx(start) != 'N') {
                key.clear();
                key.push(ch1);
                int sslen = 0;
                while ((start + 1) >= R.start && (start + 1) <= R.end && (i + 1) < cel && qv >= P.goodq &&
                       has_ne(rv.base(rpis), start) && idx(start) != 'N') {
                    if (rv.q(rpis + 1) < P.goodq + 5) break;
                    char nuc = rv.base(rpis + 1);
                    if (nuc == 'N') break;
                    if (has_eq('N', start + 1)) break;
                    if (idx(start + 1) != nuc) {
                        if (sslen == 0) key.push('&');
                        key.push(nuc);
                        sslen++;
                        qv += rv.q(rpis + 1);
                        qbases++;
                        rpis++; rpes++; i++; start++; nmoff++;
                    } else {
                        int ssn = 0;
                        for (int ssi = 1; ssi <= P.vext; ssi++) {
                            if (i + 1 + ssi >= cel) break;
                            if (rpis + 1 + ssi < rv.lseq && has_ne(rv.base(rpis + 1 + ssi), start + 1 + ssi)) {
                                ssn = ssi + 1;
                                break;
                            }
                        }
                        if (ssn == 0) break;
                        if (rv.q(rpis + ssn) < P.goodq + 5) break;
                        for (int ssi = 1; ssi <= ssn; ssi++) {
                            if (sslen == 0) key.push('&');
                            key.push(rv.base(rpis + ssi));
                            sslen++;
                            qv += rv.q(rpis + ssi);
                            qbases++;
                        }
                        rpis += ssn; rpes += ssn; i += ssn; start += ssn;
                    }
                }
                simple = sslen == 0;
            }
            // complex tails next to a deletion / insertion: src/parseCigar.cpp:779-882
            bool ss_nonempty = !simple;
            if (P.local_realign && cel - i <= P.vext && ci + 1 < n_cigar &&
                (cop(ci + 1) == 2 || cop(ci + 1) == 1) && has(start) &&
                (ss_nonempty || rv.base(rpis) != at(start)) && rv.q(rpis) >= P.goodq) {
                if (simple) { key.clear(); key.push(ch1); }
                simple = false;
                if (cop(ci + 1) == 2) {
                    while (i + 1 < cel) {
                        key.push(rv.base(rpis + 1));
                        qv += rv.q(rpis + 1);
                        qbases++; i++; rpis++; rpes++; start++;
                    }
                    // "-" dellen "&" + key without its first '&'
                    char tmp[kMaxKey];
                    int tn = 0;
                    bool dropped = false;
                    for (int k = 0; k < key.n; k++) {
                        if (!dropped && key.b[k] == '&') { dropped = true; continue; }
                        tmp[tn++] = key.b[k];
                    }
                    ddlen = clen(ci + 1);
                    key.clear();
                    key.push('-');
                    key.push_int(ddlen);
                    key.push('&');
                    for (int k = 0; k < tn; k++) key.push(tmp[k]);
                    swd = true;
                    ci += 1;
                    if (n_cigar > ci + 1 && cop(ci + 1) == 1) {
                        int nl = clen(ci + 1);
                        key.push('^');
                        append_read(rpis + 1, nl);
                        for (int qi = 1; qi <= nl; qi++) { qv += rv.q(rpis + 1 + qi); qibases++; }
                        rpis += nl; rpes += nl; ci += 1;
                    }
                    if (next_after_num_matched(ci, 1)) {
                        int tnm, qs;
                        int to = find_offset(start + ddlen + 1, rpis + 1, clen(ci + 1), tnm, qs);
                        if (to != 0) {
                            moffset = to;
                            nmoff += tnm;
                            key.push('&');
                            append_read(rpis + 1, to);
                        }
                    }
                } else {
                    while (i + 1 < cel) {
                        key.push(rv.base(rpis + 1));
                        qv += rv.q(rpis + 1);
                        qbases++; i++; rpis++; rpes++; start++;
                    }
                    char tmp[kMaxKey];
                    int tn = 0;
                    bool dropped = false;
                    for (int k = 0; k < key.n; k++) {
                        if (!dropped && key.b[k] == '&') { dropped = true; continue; }
                        tmp[tn++] = key.b[k];
                    }
                    int nl = clen(ci + 1);
                    for (int k = 0; k < nl; k++) tmp[tn++] = rv.base(rpis + 1 + k);
                    // s.insert(nl, "&") then "+" prefix
                    key.clear();
                    key.push('+');
                    for (int k = 0; k < tn; k++) {
                        if (k == nl) key.push('&');
                        key.push(tmp[k]);
                    }
                    if (nl == tn) key.push('&');
                    for (int qi = 1; qi <= nl; qi++) { qv += rv.q(rpis + 1 + qi); qibases++; }
                    rpis += nl; rpes += nl; ci += 1;
                    qibases--;
                    qbases++;
                }
            }
            if (!tr) {
                int p = start - qbases + 1;
                if (p >= R.start && p <= R.end) {
                    int tp = tp_of(rlen);
                    Obs o;
                    o.dir = dir; o.tp = tp; o.mapq = mapq; o.nm = nom - nmoff; o.std_rel = true; o.creates = true;
                    if (simple) {
                        o.q = (double)q0;
                        single(p, ch1, o);
                    } else {
                        o.q = (double)qv / (qbases + qibases);
                        if (key.overflow) S.error(ERR_KEY_TOO_LONG);
                        S.event(KIND_NONINS, p, key.b, key.n, o, read_idx);
                        for (int qi = 1; qi <= qbases; qi++) S.cov(start - qi + 1, 1);
                        if (swd)
                            for (int qi = 1; qi < ddlen; qi++) S.cov(start + qi, 1);
                    }
                }
            }
            if (swd) start += ddlen;
            if (c_op != 1) start++;
            if (c_op != 2) { rpis++; rpes++; }
            }

    // The MNV growth loop of src/parseCigar.cpp:711-767, entered at a
    // high-quality mismatch (read base rp against reference position st,
    // base i of an M op of cel bases, no indel within vext after it): true
    // when the loop ends in its first iteration without growing the key, so
    // the allele is the single read base (the general path would emit it
    // exactly as a match is emitted).  False when the key grows, and when
    // the answer needs a reference lookup outside the window (the general
    // path then decides, with the map's insert-on-lookup semantics).
    __device__ __forceinline__ bool snv_stays_single(const typename Sink::Fast &fe, int rp, int st, int i, int cel,
                                                     int goodq) const {
        if (rv.q(rp + 1) < goodq + 5) return true;  // integer q: q < goodq + 5 exactly when q < goodq_i + 5
        const char nuc = rv.base(rp + 1);
        if (nuc == 'N') return true;
        const int p1 = st + 1;
        if (p1 < R.ws || p1 > R.we) return false;
        const char r1 = fe.ref(ref, p1);
        if (r1 == 'N') return true;
        if (r1 != nuc) return false;  // the next base mismatches too: an MNV
        int ssn = 0;
        for (int ssi = 1; ssi <= P.vext; ssi++) {
            if (i + 1 + ssi >= cel) break;
            if (rp + 1 + ssi < rv.lseq) {
                const int p = p1 + ssi;
                if (p < R.ws || p > R.we) return false;
                if (fe.ref(ref, p) != rv.base(rp + 1 + ssi)) {
                    ssn = ssi + 1;
                    break;
                }
            }
        }
        if (ssn == 0) return true;
        return rv.q(rp + ssn) < goodq + 5;
    }

    // parseCigar: src/parseCigar.cpp:497-974
    __device__ void walk(const Batch &B, int64_t r) {
        read_idx = r;
        rv.seq = B.seq + (B.base_off[r] >> 1);
        rv.qual = B.qual + B.base_off[r];
        rv.cig = B.cigar + B.cig_off[r];
        rv.lseq = B.l_qseq[r];
        rv.n_cigar = B.n_cigar[r];
        n_cigar = rv.n_cigar;
        mod_n = 0;
        if (n_cigar <= 0) return;
        int flag = B.flag[r];
        int idl = 0;
        for (int i = 0; i < n_cigar; i++) {
            const uint32_t w = __ldg(rv.cig + i);  // original ops (before cleanup)
            if (cig_op(w) == 1 || cig_op(w) == 2) idl += cig_len(w);
        }
        int nmtag = B.nm[r];
        int nom = 0;
        if (nmtag != INT32_MIN) {
            nom = nmtag - idl;
            if (nom > P.mismatch) return;
        } else if (flag & 4) {
            return;
        }
        bool dir = (flag & 16) != 0;
        int mapq = B.mapq[r];
        int position = B.pos[r] + 1;
        rpis = rpes = 0;
        if (P.local_realign) {
            const uint32_t w0 = __ldg(rv.cig);
            if (n_cigar == 1 && cig_op(w0) == 0 && cig_len(w0) >= 8 && cig_len(w0) == rv.lseq) {
                rewrite_single_m(cig_len(w0), position);
            } else if (!rewrite_cigar(idl, position)) {
                S.error(ERR_UNSUPPORTED);
                return;
            }
        }
        // cleanupCigar (src/parseCigar.cpp:1858-1892), applied on read by W()
        lead_end = n_cigar;
        trail_start = -1;
        for (int k = 0; k < n_cigar; k++) {
            int o = cig_op(mem(k));
            if (o == 0 || o == 7 || o == 8) {
                if (lead_end == n_cigar) lead_end = k;
                trail_start = k;
            }
        }
        start = position;
        offset = 0;
        if (cop(0) == 4 && clen(0) >= 10 && cop(n_cigar - 1) == 4 && clen(n_cigar - 1) >= 10) return;
        int rlen = 0, tlen = 0, orig_ref_len = 0;
        for (int i = 0; i < n_cigar; i++) {
            int o = cop(i);
            if (o == 0 || o == 1) rlen += clen(i);
            if (o == 0 || o == 1 || o == 4) tlen += clen(i);
        }
        // the record's end (bam_endpos): its own word count over the words now in memory
        for (int i = 0; i < rv.n_cigar; i++) {
            int o = cig_op(mem(i));
            if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) orig_ref_len += cig_len(mem(i));
        }
        if (P.minmatch != 0 && rlen < P.minmatch) return;
        S.max_len(tlen);
        if (flag & 2048) return;
        int mate_start = B.mpos[r] + 1;
        int endpos = orig_ref_len ? B.pos[r] + orig_ref_len : B.pos[r] + 1;
        // skipOverlappingReads, evaluated once at ci == 0 (src/parseCigar.cpp:180-206, 629-634)
        if (P.unique_fwd && (flag & 1) && !dir && start >= mate_start) return;
        if (P.unique_first && (flag & 1)) {
            bool ov;
            if (position >= mate_start) ov = start >= mate_start && start <= mate_start + orig_ref_len - 1;
            else ov = start >= mate_start && mate_start <= endpos;
            if (ov) return;
        }
        m_dir = dir;
        m_mapq = mapq;
        m_nom = nom;
        m_rlen = rlen;
        m_tlen = tlen;
        typename Sink::Fast fe = S.fast();
        const int rs = R.start, re = R.end, ws = R.ws, we = R.we;
        const int goodq = P.goodq_i;  // integer qualities: q >= goodq_i exactly when q >= goodq
        const int ttr = P.trim_bases_after;
        for (int ci = 0; ci < n_cigar; ++ci) {
            if (S.done()) return;
            int c_op = cop(ci);
            cel = clen(ci);
            if ((ci == 0 || ci == n_cigar - 1) && c_op == 1) c_op = 4;
            if (c_op == 3) {  // processNotMatched: src/parseCigar.cpp:1733-1753
                char kb[24];
                int k = 0, a = start - 1, b2 = start + cel - 1;
                KeyBuf &t = key;
                t.clear(); t.push_int(a); t.push('-'); t.push_int(b2);
                for (int i = 0; i < t.n && k < 24; i++) kb[k++] = t.b[i];
                Obs o = plain_obs(dir, 0, 0, 0, 0);
                o.creates = true;
                S.event(KIND_SPLICE, 0, kb, k, o, read_idx);
                start += cel;
                offset = 0;
                continue;
            }
            if (c_op == 4) { softclip(ci, dir, mapq, nom, position, tlen); continue; }
            if (c_op == 5) { offset = 0; continue; }
            if (c_op == 1) { offset = 0; ci = insertion(ci, dir, mapq, nom, position, rlen); continue; }
            if (c_op == 2) { offset = 0; ci = deletion(ci, dir, mapq, nom, rlen); continue; }
            int nmoff = 0, moffset = 0;
            // with local realignment, bases within vext of a following indel
            // may build complex keys: take the out-of-line iteration for them
            const int tail_from = (P.local_realign && ci + 1 < n_cigar && (cop(ci + 1) == 1 || cop(ci + 1) == 2))
                                      ? cel - P.vext : INT32_MAX;
            // hot loop: every value it touches lives in registers (the walker
            // object itself is in local memory for the out-of-line paths)
            int st = start, rp = rpis, rq = rpes;
            int celr = cel;
            const uint4 *seq16 = reinterpret_cast<const uint4 *>(rv.seq);
            const uint4 *qual16 = reinterpret_cast<const uint4 *>(rv.qual);
            const char *refp = ref;
            uint4 qw = make_uint4(0, 0, 0, 0), sw = make_uint4(0, 0, 0, 0);
            int qblk = -1, sblk = -1;
            for (int i = offset; i < celr; i++) {
                if ((rp >> 5) != sblk) { sblk = rp >> 5; sw = __ldg(seq16 + sblk); }
                const uint32_t swd_ = pick_word(sw, (rp & 31) >> 3);
                const int code = (int)((swd_ >> (((rp & 7) ^ 1) * 4)) & 15u);
                if (code == 15) {  // 'N': skipped (src/parseCigar.cpp:686-692)
                    st++; rp++; rq++;
                    continue;
                }
                if ((rp >> 4) != qblk) { qblk = rp >> 4; qw = __ldg(qual16 + qblk); }
                const int q0 = (int)((pick_word(qw, (rp & 15) >> 2) >> ((rp & 3) * 8)) & 255u);
                const int b = code_base(code);
                const bool hs = st >= ws && st <= we;
                // the reference base's code (ref_code_of): a mismatch is any
                // code but the read base's, 'N' is code 5
                const int rcode = hs ? fe.ref_code(refp, st) : 4;
                const bool mm = hs && rcode != b;
                bool slow = b < 0 || i >= tail_from;
                // a high-quality mismatch enters the MNV growth; most end
                // there as the single base and are emitted like a match
                if (!slow && mm && q0 >= goodq && st + 1 >= rs && st + 1 <= re && i + 1 < celr && rcode != 5)
                    slow = !snv_stays_single(fe, rp, st, i, celr, goodq);
                if (!slow) {
                    const bool tr = ttr != 0 && (dir ? tlen - rp > ttr : rp > ttr);
                    if (!tr && st >= rs && st <= re) {
                        const int tp = rq < rlen - rq ? rq + 1 : rlen - rq;
                        if (!fe.emit(st, b, dir, tp, q0, mapq, nom - nmoff)) {
                            Obs o;
                            o.dir = dir; o.tp = tp; o.q = (double)q0; o.mapq = mapq; o.nm = nom - nmoff;
                            o.std_rel = true; o.creates = true;
                            S.single(st, b, o, read_idx);
                            if (S.done()) return;
                        }
                    }
                    st++; rp++; rq++;
                    continue;
                }
                start = st; rpis = rp; rpes = rq;
                m_i = i; m_ci = ci; m_nmoff = nmoff; m_moffset = moffset; m_cop = c_op;
                m_iteration();
                st = start; rp = rpis; rq = rpes;
                i = m_i; ci = m_ci; nmoff = m_nmoff; moffset = m_moffset;
                celr = cel;
            }
            start = st; rpis = rp; rpes = rq;
            if (moffset != 0) {
                offset = moffset;
                rpis += moffset;
                start += moffset;
                rpes += moffset;
            }
            if (start > R.end) break;
        }
    }
};

}  // namespace rv
