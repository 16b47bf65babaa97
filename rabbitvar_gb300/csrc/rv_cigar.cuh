// Device CIGAR rewrite of local realignment (-k 1): CigarModifier::modifyCigar
// (src/cigarModifier.cpp:219-390) and its helpers (:395-1000), on the CIGAR as
// a short token list instead of its text.  The reference matches regular
// expressions (include/patterns.h:52-153) against the CIGAR text; every
// pattern it uses is a fixed sequence of (number, operator) tokens, anchored
// at the start, at the end, or searched from the left, and a leftmost match
// always starts at a token boundary, so each rule below is the same test on
// tokens.  Two places where the text semantics matter are kept: rule
// NOTDIG_DIG_I_... looks for its I-M-(D|I) group after some operator letter
// but the replacement rewrites the first such group of the CIGAR, which can
// be an earlier one; and a rewrite never leaves a negative length behind
// (the reference writes the original CIGAR back then), here such reads are
// reported as unsupported because later rules would parse the text of a
// negative number differently.
#pragma once
#include "rv_internal.h"

namespace rv {

constexpr int kCigTok = 16;   // tokens a rewritten CIGAR may have

struct CigTok {
    int len[kCigTok];
    char op[kCigTok];
    int n;
    bool bad;   // overflow or a negative length: the read is not supported

    __device__ void erase_range(int a, int cnt) {
        for (int k = a; k + cnt < n; k++) { len[k] = len[k + cnt]; op[k] = op[k + cnt]; }
        n -= cnt;
    }
    // replace tokens [a, a + cnt) by the list (l[i], o[i]) of m tokens
    __device__ void replace(int a, int cnt, const int *l, const char *o, int m) {
        if (n - cnt + m > kCigTok) { bad = true; return; }
        if (m < cnt) erase_range(a + m, cnt - m);
        else if (m > cnt) {
            for (int k = n - 1; k >= a + cnt; k--) { len[k + m - cnt] = len[k]; op[k + m - cnt] = op[k]; }
            n += m - cnt;
        }
        for (int i = 0; i < m; i++) {
            len[a + i] = l[i];
            op[a + i] = o[i];
            if (l[i] < 0) bad = true;
        }
    }
    __device__ void rep1(int a, int cnt, int l0, char o0) { replace(a, cnt, &l0, &o0, 1); }
    __device__ void rep2(int a, int cnt, int l0, char o0, int l1, char o1) {
        int l[2] = {l0, l1};
        char o[2] = {o0, o1};
        replace(a, cnt, l, o, 2);
    }
    __device__ bool is(int k, char o) const { return k >= 0 && k < n && op[k] == o; }
    __device__ bool id(int k) const { return k >= 0 && k < n && (op[k] == 'I' || op[k] == 'D'); }
    __device__ bool eq(const CigTok &o) const {
        if (n != o.n) return false;
        for (int k = 0; k < n; k++)
            if (len[k] != o.len[k] || op[k] != o.op[k]) return false;
        return true;
    }
    // first k >= from with tokens k.. matching the operator string (I|D written as '*')
    __device__ int find(const char *pat, int from = 0) const {
        int m = 0;
        while (pat[m]) m++;
        for (int k = from; k + m <= n; k++) {
            bool ok = true;
            for (int j = 0; j < m && ok; j++) ok = pat[j] == '*' ? (op[k + j] == 'I' || op[k + j] == 'D') : op[k + j] == pat[j];
            if (ok) return k;
        }
        return -1;
    }
    // globalFindAndSum over the prefix tokens [0, k): lengths of the listed operators
    __device__ int sum(int k, const char *ops) const {
        int s = 0;
        for (int i = 0; i < k; i++)
            for (const char *p = ops; *p; p++)
                if (op[i] == *p) s += len[i];
        return s;
    }
};

__device__ __forceinline__ char op_char(uint32_t w) {
    const int o = (int)(w & 15u);
    return o <= 9 ? "MIDNSHP=XB"[o] : '?';
}
__device__ __forceinline__ uint32_t op_code(char c) {
    switch (c) {
    case 'M': return 0;
    case 'I': return 1;
    case 'D': return 2;
    case 'N': return 3;
    case 'S': return 4;
    case 'H': return 5;
    case 'P': return 6;
    case '=': return 7;
    case 'X': return 8;
    default: return 9;
    }
}

// The rewrite for one read.  Acc gives has(p) / at(p) of the region's
// reference map (insert-on-lookup entries included), base(i) (decoded read
// base) and q(i) (base quality).
template <class Acc>
struct CigarEdit {
    const Acc &A;
    CigTok t;
    int position;

    __device__ bool eqb(int p, int i) const { return A.has(p) && A.at(p) == A.base(i); }
    __device__ bool neb(int p, int i) const { return A.has(p) && A.at(p) != A.base(i); }

    // combineBeginDigM (:412-439)
    __device__ void begin_dig_m() {
        int mch = t.len[0], rn = 0, rrn = 0, rmch = 0;
        while (rrn < mch && rn < mch) {
            if (!A.has(position + rrn)) break;
            if (neb(position + rrn, rrn)) { rn = rrn + 1; rmch = 0; }
            else if (eqb(position + rrn, rrn)) rmch++;
            rrn++;
            if (rmch >= 3) break;
        }
        if (rn > 0 && rn <= 3) {
            mch -= rn;
            if (t.is(0, 'M')) t.rep2(0, 1, rn, 'S', mch, 'M');
            position += rn;
        }
    }
    __device__ void rep_sm(int soft, int mch) {  // DIG_S_DIG_M replaceFirst
        if (!(t.is(0, 'S') && t.is(1, 'M'))) return;
        if (soft > 0) t.rep2(0, 2, soft, 'S', mch, 'M');
        else t.rep1(0, 2, mch, 'M');
    }
    // combineDigSDigM (:445-525)
    __device__ void dig_s_dig_m() {
        int mch = t.len[1], soft = t.len[0], rn = 0;
        unsigned rnset = 0;
        while (rn < soft && eqb(position - rn - 1, soft - rn - 1) && A.q(soft - rn - 1) > 10) rn++;
        if (rn > 0) {
            mch += rn;
            soft -= rn;
            rep_sm(soft, mch);
            position -= rn;
            rn = 0;
        }
        if (soft > 0) {
            while (rn + 1 < soft && eqb(position - rn - 2, soft - rn - 2) && A.q(soft - rn - 2) > 10) {
                rn++;
                if (A.has(position - rn - 2)) rnset |= 1u << ((unsigned char)A.at(position - rn - 2) & 31);
            }
            const int rn_nt = __popc(rnset);
            if ((rn > 4 && rn_nt > 1) || eqb(position - 1, soft - 1)) {
                mch += rn + 1;
                soft -= rn + 1;
                rep_sm(soft, mch);
                position -= rn + 1;
            }
            if (rn == 0) {
                int rrn = 0, rmch = 0;
                while (rrn < mch && rn < mch) {
                    if (!A.has(position + rrn)) break;
                    if (neb(position + rrn, soft + rrn)) { rn = rrn + 1; rmch = 0; }
                    else if (eqb(position + rrn, soft + rrn)) rmch++;
                    rrn++;
                    if (rmch >= 3) break;
                }
                if (rn > 0 && rn < mch) {
                    soft += rn;
                    mch -= rn;
                    rep_sm(soft, mch);
                    position += rn;
                }
            }
        }
    }
    // the backward mismatch scan of captureMisSoftly*
    __device__ int back_scan(int mch, int refoff, int rdoff) const {
        int rn = 0, rrn = 0, rmch = 0;
        while (rrn < mch && rn < mch) {
            if (!A.has(refoff - rrn - 1)) break;
            if (rrn < rdoff && A.at(refoff - rrn - 1) != A.base(rdoff - rrn - 1)) { rn = rrn + 1; rmch = 0; }
            else if (rrn < rdoff && A.at(refoff - rrn - 1) == A.base(rdoff - rrn - 1)) rmch++;
            rrn++;
            if (rmch >= 3) break;
        }
        return rn;
    }
    // captureMisSoftly3Mismatches (:531-566); the CIGAR ends with M
    __device__ void mis3() {
        const int k = t.n - 1;
        int mch = t.len[k];
        const int refoff = position + mch + t.sum(k, "MND"), rdoff = mch + t.sum(k, "MIS");
        const int rn = back_scan(mch, refoff, rdoff);
        mch -= rn;
        if (rn > 0 && rn <= 3 && t.is(t.n - 1, 'M')) t.rep2(t.n - 1, 1, mch, 'M', rn, 'S');
    }
    __device__ void rep_ms(int mch, int soft) {  // DIG_M_DIG_S_END replaceFirst
        if (!(t.n >= 2 && t.is(t.n - 2, 'M') && t.is(t.n - 1, 'S'))) return;
        if (soft > 0) t.rep2(t.n - 2, 2, mch, 'M', soft, 'S');
        else t.rep1(t.n - 2, 2, mch, 'M');
    }
    // captureMisSoftlyMS (:572-653); the CIGAR ends with M S
    __device__ void mis_ms() {
        const int k = t.n - 2;
        int mch = t.len[k], soft = t.len[k + 1];
        const int refoff = position + mch + t.sum(k, "MND"), rdoff = mch + t.sum(k, "MIS");
        int rn = 0;
        unsigned rnset = 0;
        while (rn < soft && eqb(refoff + rn, rdoff + rn) && A.q(rdoff + rn) > 10) rn++;
        if (rn > 0) {
            mch += rn;
            soft -= rn;
            rep_ms(mch, soft);
            rn = 0;
        }
        if (soft > 0) {
            while (rn + 1 < soft && eqb(refoff + rn + 1, rdoff + rn + 1) && A.q(rdoff + rn + 1) > 10) {
                rn++;
                if (A.has(refoff + rn + 1)) rnset |= 1u << ((unsigned char)A.at(refoff + rn + 1) & 31);
            }
            if (rn > 4 && __popc(rnset) > 1) {
                mch += rn + 1;
                soft -= rn + 1;
                rep_ms(mch, soft);
            }
            if (rn == 0) {
                rn = back_scan(mch, refoff, rdoff);
                if (rn > 0 && rn < mch) {
                    soft += rn;
                    mch -= rn;
                    rep_ms(mch, soft);
                }
            }
        }
    }
    // matched bases from (rdoff, refoff) onwards, for the three-event rules
    __device__ int run_match(int rdoff, int refoff) const {
        int rn = 0;
        while (rdoff + rn < A.lseq() && A.has(refoff + rn) && A.at(refoff + rn) == A.base(rdoff + rn)) rn++;
        return rn;
    }
    // twoDeletionsInsertionToComplex (:920-972): tokens k..k+6 = M D M I M D M
    __device__ bool two_del_ins(int k, bool flag) {
        int tslen = t.len[k + 2] + t.len[k + 3] + t.len[k + 4];
        int dlen = t.len[k + 1] + t.len[k + 2] + t.len[k + 4] + t.len[k + 5];
        const int mid = t.len[k + 2] + t.len[k + 4];
        const int mch = t.len[k];
        const int refoff = position + mch + t.sum(k, "MND"), rdoff = mch + t.sum(k, "MIS");
        int RDOFF = mch, rm = t.len[k + 6];
        const int rn = run_match(rdoff, refoff);
        RDOFF += rn;
        dlen -= rn;
        tslen -= rn;
        if (mid <= 15) {
            if (tslen <= 0) {
                dlen -= tslen;
                rm += tslen;
                int l[3] = {RDOFF, dlen, rm};
                char o[3] = {'M', 'D', 'M'};
                t.replace(k, 7, l, o, 3);
            } else {
                int l[4] = {RDOFF, dlen, tslen, rm};
                char o[4] = {'M', 'D', 'I', 'M'};
                t.replace(k, 7, l, o, 4);
            }
            flag = true;
        }
        return flag;
    }
    // threeDeletions (:856-910): tokens k..k+6 = M D M D M D M
    __device__ bool three_deletions(int k, bool flag) {
        int tslen = t.len[k + 2] + t.len[k + 4];
        int dlen = t.len[k + 1] + t.len[k + 2] + t.len[k + 3] + t.len[k + 4] + t.len[k + 5];
        const int mid = t.len[k + 2] + t.len[k + 4];
        const int refoff = position + t.len[k] + t.sum(k, "MND"), rdoff = t.len[k] + t.sum(k, "MIS");
        int RDOFF = t.len[k], rm = t.len[k + 6];
        const int rn = run_match(rdoff, refoff);
        RDOFF += rn;
        dlen -= rn;
        tslen -= rn;
        if (mid <= 15) {
            if (tslen <= 0) {
                dlen -= tslen;
                rm += tslen;
                int l[3] = {RDOFF, dlen, rm};
                char o[3] = {'M', 'D', 'M'};
                t.replace(k, 7, l, o, 3);
            } else {
                int l[4] = {RDOFF, dlen, tslen, rm};
                char o[4] = {'M', 'D', 'I', 'M'};
                t.replace(k, 7, l, o, 4);
            }
            flag = true;
        }
        return flag;
    }
    // threeIndels (:755-846): tokens k..k+6 = M (I|D) M (I|D) M (I|D) M
    __device__ bool three_indels(int k, bool flag) {
        const int mid = t.len[k + 2] + t.len[k + 4];
        int tslen = mid, dlen = mid;
        for (int j = 1; j <= 5; j += 2) {
            if (t.op[k + j] == 'I') tslen += t.len[k + j];
            if (t.op[k + j] == 'D') dlen += t.len[k + j];
        }
        const int refoff = position + t.len[k] + t.sum(k, "MND"), rdoff = t.len[k] + t.sum(k, "MIS");
        int RDOFF = t.len[k], rm = t.len[k + 6];
        const int rn = run_match(rdoff, refoff);
        RDOFF += rn;
        dlen -= rn;
        tslen -= rn;
        int l[4];
        char o[4];
        int m = 0;
        auto put = [&](int a, char b) { l[m] = a; o[m] = b; m++; };
        if (tslen <= 0) {
            dlen -= tslen;
            rm += tslen;
            if (dlen == 0) {
                RDOFF += rm;
                put(RDOFF, 'M');
            } else if (dlen < 0) {
                tslen = -dlen;
                rm += dlen;
                if (rm < 0) {
                    RDOFF += rm;
                    put(RDOFF, 'M');
                    put(tslen, 'I');
                } else {
                    put(RDOFF, 'M');
                    put(tslen, 'I');
                    put(rm, 'M');
                }
            } else {
                put(RDOFF, 'M');
                put(dlen, 'D');
                put(rm, 'M');
            }
        } else {
            put(RDOFF, 'M');
            if (dlen == 0) {
                put(tslen, 'I');
                put(rm, 'M');
            } else if (dlen < 0) {
                rm += dlen;
                put(tslen, 'I');
                put(rm, 'M');
            } else {
                put(dlen, 'D');
                put(tslen, 'I');
                put(rm, 'M');
            }
        }
        if (mid <= 15) {
            t.replace(k, 7, l, o, m);
            flag = true;
        }
        return flag;
    }
    // beginDigitMNumberIorDNumberM (:982-1000): tokens 0..2 = M(1 digit) (I|D) M
    __device__ bool begin_digit_m() {
        const int tmid = t.len[0];
        int mlen = t.len[2], tn = 0;
        int tslen = tmid + (t.op[1] == 'I' ? t.len[1] : 0);
        position += tmid + (t.op[1] == 'D' ? t.len[1] : 0);
        while (tn < mlen && A.has(position + tn) && A.at(position + tn) != A.base(tslen + tn)) tn++;
        tslen += tn;
        mlen -= tn;
        position += tn;
        t.rep2(0, 3, tslen, 'S', mlen, 'M');
        return true;
    }

    // the optional trailing insertion of DIG_?_DIG_M_DIG_DI_DIGI at tokens k..
    __device__ int span_with_i(int k) const { return t.is(k + 3, 'I') ? 4 : 3; }

    __device__ void run(int indel) {
        bool flag = true;
        int guard = 0;
        while (flag && indel > 0 && !t.bad) {
            if (++guard > 64) { t.bad = true; break; }
            flag = false;
            // BEGIN_NUMBER_S_NUMBER_IorD
            if (t.is(0, 'S') && t.id(1)) {
                const int ts = t.len[0] + (t.op[1] == 'I' ? t.len[1] : 0);
                position += t.op[1] == 'D' ? t.len[1] : 0;
                t.rep1(0, 2, ts, 'S');
                flag = true;
            }
            // NUMBER_IorD_NUMBER_S_END
            if (t.n >= 2 && t.id(t.n - 2) && t.is(t.n - 1, 'S')) {
                const int ts = t.len[t.n - 1] + (t.op[t.n - 2] == 'I' ? t.len[t.n - 2] : 0);
                t.rep1(t.n - 2, 2, ts, 'S');
                flag = true;
            }
            // BEGIN_NUMBER_S_NUMBER_M_NUMBER_IorD
            if (t.is(0, 'S') && t.is(1, 'M') && t.id(2)) {
                const int tmid = t.len[1];
                if (tmid <= 10) {
                    const int ts = t.len[0] + tmid + (t.op[2] == 'I' ? t.len[2] : 0);
                    position += tmid + (t.op[2] == 'D' ? t.len[2] : 0);
                    t.rep1(0, 3, ts, 'S');
                    flag = true;
                }
            }
            // NUMBER_IorD_NUMBER_M_NUMBER_S_END
            if (t.n >= 3 && t.id(t.n - 3) && t.is(t.n - 2, 'M') && t.is(t.n - 1, 'S')) {
                const int tmid = t.len[t.n - 2];
                if (tmid <= 10) {
                    const int ts = t.len[t.n - 1] + tmid + (t.op[t.n - 3] == 'I' ? t.len[t.n - 3] : 0);
                    t.rep1(t.n - 3, 3, ts, 'S');
                    flag = true;
                }
            }
            // BEGIN_DIGIT_M_NUMBER_IorD_NUMBER_M
            if (t.is(0, 'M') && t.len[0] <= 9 && t.id(1) && t.is(2, 'M')) flag = begin_digit_m();
            // NUMBER_IorD_DIGIT_M_END
            if (t.n >= 2 && t.id(t.n - 2) && t.is(t.n - 1, 'M') && t.len[t.n - 1] <= 9) {
                const int ts = t.len[t.n - 1] + (t.op[t.n - 2] == 'I' ? t.len[t.n - 2] : 0);
                t.rep1(t.n - 2, 2, ts, 'S');
                flag = true;
            }
            // the three complex rules, all searched before any of them rewrites
            const int k7 = t.find("MDMIMDM"), k9 = t.find("MDMDMDM"), k10 = t.find("M*M*M*M");
            if (k7 >= 0) flag = two_del_ins(k7, flag);
            else if (k9 >= 0) flag = three_deletions(k9, flag);
            else if (k10 >= 0) flag = three_indels(k10, flag);
            // DIG_D_DIG_M_DIG_DI_DIGI
            int k = t.find("DM*");
            if (k >= 0 && t.len[k + 1] <= 15) {
                int dlen = t.len[k] + t.len[k + 1], ilen = t.len[k + 1];
                const int sp = span_with_i(k);
                if (t.op[k + 2] == 'I') ilen += t.len[k + 2];
                else {
                    dlen += t.len[k + 2];
                    if (sp == 4) ilen += t.len[k + 3];
                }
                t.rep2(k, sp, dlen, 'D', ilen, 'I');
                flag = true;
            }
            // NOTDIG_DIG_I_DIG_M_DIG_DI_DIGI: the group after some operator letter;
            // the rewrite goes to the first I-M-(D|I) group of the CIGAR
            k = t.find("IM*", 1);
            if (k >= 1 && t.op[k - 1] != 'D' && t.op[k - 1] != 'H' && t.len[k + 1] <= 15) {
                int dlen = t.len[k + 1], ilen = t.len[k] + t.len[k + 1];
                if (t.op[k + 2] == 'I') ilen += t.len[k + 2];
                else {
                    dlen += t.len[k + 2];
                    if (span_with_i(k) == 4) ilen += t.len[k + 3];
                }
                const int k0 = t.find("IM*");
                t.rep2(k0, span_with_i(k0), dlen, 'D', ilen, 'I');
                flag = true;
            }
            // DIG_D_DIG_D, DIG_I_DIG_I
            k = t.find("DD");
            if (k >= 0) { t.rep1(k, 2, t.len[k] + t.len[k + 1], 'D'); flag = true; }
            k = t.find("II");
            if (k >= 0) { t.rep1(k, 2, t.len[k] + t.len[k + 1], 'I'); flag = true; }
        }
        if (t.bad) return;
        if (t.n >= 2 && t.is(t.n - 2, 'M') && t.is(t.n - 1, 'S')) mis_ms();
        else if (t.n >= 1 && t.is(t.n - 1, 'M')) mis3();
        if (t.is(0, 'S') && t.is(1, 'M')) dig_s_dig_m();
        else if (t.is(0, 'M')) begin_dig_m();
    }
};

}  // namespace rv
