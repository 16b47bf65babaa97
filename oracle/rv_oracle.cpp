// Oracle test infrastructure -- not part of the product (see rv_oracle.h).
//
// A sequential CPU restatement of RabbitVar's per-region path, written to be
// read beside the reference: every function names the reference lines it
// restates.  Containers are ordered std::maps (the reference uses robin_hood
// hash maps); where the reference's behaviour depends on its hash map's
// iteration order this restatement uses an order measured from the
// reference's map (noted at the use), or ascending position order.
#include "rv_oracle.h"
#include "fisher_oracle.h"

#include <omp.h>
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <regex>
#include <set>
#include <string>
#include <vector>

namespace {

using std::map;
using std::string;
using std::vector;

const char kNt16[] = "=ACMGRSVTWYHKDBN";

enum { OP_M = 0, OP_I = 1, OP_D = 2, OP_N = 3, OP_S = 4, OP_H = 5 };

// Statistics of one allele key: include/Variation.h:12-82.
struct Stat {
    int cnt = 0, fwd = 0, rev = 0;
    double pmean = 0, qmean = 0, mq = 0, nm = 0;
    int lo = 0, hi = 0;
    bool pstd = false, qstd = false;
    int pp = 0;
    double pq = 0;
    int extracnt = 0;
    void inc_dir(bool d) { d ? ++rev : ++fwd; }
};

// Soft-clip aggregate: include/Sclip.h:10-39.
struct Clip : Stat {
    map<int, map<char, int>> nt;
    map<int, map<char, Stat>> seq;
    string cons;  // cached consensus ("" = not computed yet)
    bool used = false;
};

using KeyMap = map<string, Stat>;

struct Maps {
    map<int, KeyMap> nonins, ins;
    map<int, int> cov;
    map<int, Clip> sc5, sc3;
    map<int, map<string, int>> inscnt, delcnt, mnp;
    int max_read_len = 0;
};

// Reference window: RecordPreprocessor::makeReference
// (src/recordPreprocessor.cpp:41-78) loads [lo, hi] where
// hi = min(len, end + x + ext) - CONF_SEED_1 (17).  Lookups through the hash
// map's operator[] insert a 0 for a missing position (robin_hood semantics);
// those "phantom" entries then count as present with base 0.
struct Ref {
    const char *contig = nullptr;
    int clen = 0, lo = 1, hi = 0;
    std::set<int> phantom;
    static char up(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }
    bool has(int p) const { return (p >= lo && p <= hi) || phantom.count(p); }
    char at(int p) const { return (p >= lo && p <= hi) ? up(contig[p - 1]) : 0; }
    char idx(int p) {  // operator[]
        if (p >= lo && p <= hi) return up(contig[p - 1]);
        phantom.insert(p);
        return 0;
    }
    bool has_eq(char c, int p) const { return has(p) && at(p) == c; }
    bool has_ne(char c, int p) const { return has(p) && at(p) != c; }
};

struct UnsupportedRead {};

struct ReadView {
    int32_t pos, mpos, nm;
    uint16_t flag;
    uint8_t mapq;
    int lseq;
    vector<uint32_t> cig;      // CIGAR words followed by the bytes that follow them in a BAM record
    int n_cigar;
    vector<char> seq;          // decoded bases
    vector<uint8_t> qual_buf;  // [byte preceding quals] + quals
    const uint8_t *qual() const { return qual_buf.data() + 1; }
};

// ---------------------------------------------------------------------------
// -k 1 CIGAR rewrite: CigarModifier (src/cigarModifier.cpp), on the CIGAR
// string with the reference's own pattern grammar (include/patterns.h:52-153)
// ---------------------------------------------------------------------------
struct CigarMod {
    Ref &R;
    const vector<char> &seq;
    const uint8_t *qual;
    int lseq;
    int position;
    string cs;

    static const std::regex &re(int i) {
        static const std::regex tab[] = {
            std::regex("^(\\d+)S(\\d+)([ID])"),                                           // 0
            std::regex("(\\d+)([ID])(\\d+)S$"),                                           // 1
            std::regex("^(\\d+)S(\\d+)M(\\d+)([ID])"),                                    // 2
            std::regex("(\\d+)([ID])(\\d+)M(\\d+)S$"),                                    // 3
            std::regex("^(\\d)M(\\d+)([ID])(\\d+)M"),                                     // 4
            std::regex("^\\dM\\d+[ID]\\d+M"),                                             // 5
            std::regex("(\\d+)([ID])(\\d)M$"),                                            // 6
            std::regex("^(.*?)(\\d+)M(\\d+)D(\\d+)M(\\d+)I(\\d+)M(\\d+)D(\\d+)M"),        // 7
            std::regex("(\\d+)M(\\d+)D(\\d+)M(\\d+)I(\\d+)M(\\d+)D(\\d+)M"),              // 8
            std::regex("^(.*?)(\\d+)M(\\d+)D(\\d+)M(\\d+)D(\\d+)M(\\d+)D(\\d+)M"),        // 9
            std::regex("^(.*?)(\\d+)M(\\d+)([DI])(\\d+)M(\\d+)([DI])(\\d+)M(\\d+)([DI])(\\d+)M"),  // 10
            std::regex("\\d+M\\d+[DI]\\d+M\\d+[DI]\\d+M\\d+[DI]\\d+M"),                   // 11
            std::regex("\\d+M\\d+D\\d+M\\d+D\\d+M\\d+D\\d+M"),                            // 12
            std::regex("(\\d+)D(\\d+)M(\\d+)([DI])(\\d+I)?"),                             // 13
            std::regex("(\\d+)I(\\d+)M(\\d+)([DI])(\\d+I)?"),                             // 14
            std::regex("(\\D)(\\d+)I(\\d+)M(\\d+)([DI])(\\d+I)?"),                        // 15
            std::regex("(\\d+)D(\\d+)D"),                                                 // 16
            std::regex("(\\d+)I(\\d+)I"),                                                 // 17
            std::regex("^(.*?)(\\d+)M$"),                                                 // 18
            std::regex("\\d+M$"),                                                         // 19
            std::regex("^(\\d+)M"),                                                       // 20
            std::regex("^(\\d+)S(\\d+)M"),                                                // 21
            std::regex("\\d+M\\d+S$"),                                                    // 22
            std::regex("^(.*?)(\\d+)M(\\d+)S$"),                                          // 23
            std::regex("(\\d+)[MND]"),                                                    // 24
            std::regex("(\\d+)[MIS]"),                                                    // 25
        };
        return tab[i];
    }
    static int I(const std::smatch &m, int k) { return std::stoi(m.str(k)); }
    static int sum_of(int rx, const string &s) {  // globalFindAndSum (include/util.h:186-199)
        int r = 0;
        for (std::sregex_iterator it(s.begin(), s.end(), re(rx)), e; it != e; ++it) r += std::stoi((*it)[1].str());
        return r;
    }
    void rep_first(int rx, const string &to) {
        cs = std::regex_replace(cs, re(rx), to, std::regex_constants::format_first_only);
    }
    void rep_all(int rx, const string &to) { cs = std::regex_replace(cs, re(rx), to); }
    bool eq(int p, int i) const { return R.has(p) && R.at(p) == seq[i]; }    // isHasAndEquals(ref, p, seq, i)
    bool ne(int p, int i) const { return R.has(p) && R.at(p) != seq[i]; }    // isHasAndNotEquals(ref, p, seq, i)

    // combineBeginDigM (:412-439)
    void begin_dig_m(const std::smatch &m) {
        int mch = I(m, 1), rn = 0, rrn = 0, rmch = 0;
        while (rrn < mch && rn < mch) {
            if (!R.has(position + rrn)) break;
            if (ne(position + rrn, rrn)) { rn = rrn + 1; rmch = 0; }
            else if (eq(position + rrn, rrn)) rmch++;
            rrn++;
            if (rmch >= 3) break;
        }
        if (rn > 0 && rn <= 3) {
            mch -= rn;
            rep_first(20, std::to_string(rn) + "S" + std::to_string(mch) + "M");
            position += rn;
        }
    }
    // combineDigSDigM (:445-525)
    void dig_s_dig_m(const std::smatch &m) {
        int mch = I(m, 2), soft = I(m, 1), rn = 0;
        std::set<char> RN;
        while (rn < soft && eq(position - rn - 1, soft - rn - 1) && qual[soft - rn - 1] > 10) rn++;
        if (rn > 0) {
            mch += rn;
            soft -= rn;
            rep_first(21, soft > 0 ? std::to_string(soft) + "S" + std::to_string(mch) + "M" : std::to_string(mch) + "M");
            position -= rn;
            rn = 0;
        }
        if (soft > 0) {
            while (rn + 1 < soft && eq(position - rn - 2, soft - rn - 2) && qual[soft - rn - 2] > 10) {
                rn++;
                if (R.has(position - rn - 2)) RN.insert(R.at(position - rn - 2));
            }
            int rn_nt = (int)RN.size();
            if ((rn > 4 && rn_nt > 1) || eq(position - 1, soft - 1)) {
                mch += rn + 1;
                soft -= rn + 1;
                rep_first(21, soft > 0 ? std::to_string(soft) + "S" + std::to_string(mch) + "M"
                                       : std::to_string(mch) + "M");
                position -= rn + 1;
            }
            if (rn == 0) {
                int rrn = 0, rmch = 0;
                while (rrn < mch && rn < mch) {
                    if (!R.has(position + rrn)) break;
                    if (ne(position + rrn, soft + rrn)) { rn = rrn + 1; rmch = 0; }
                    else if (eq(position + rrn, soft + rrn)) rmch++;
                    rrn++;
                    if (rmch >= 3) break;
                }
                if (rn > 0 && rn < mch) {
                    soft += rn;
                    mch -= rn;
                    rep_first(21, std::to_string(soft) + "S" + std::to_string(mch) + "M");
                    position += rn;
                }
            }
        }
    }
    // captureMisSoftly3Mismatches (:531-566)
    void mis3(const std::smatch &m) {
        string ov5 = m.str(1);
        int mch = I(m, 2), refoff = position + mch, rdoff = mch;
        if (!ov5.empty()) { refoff += sum_of(24, ov5); rdoff += sum_of(25, ov5); }
        int rn = 0, rrn = 0, rmch = 0;
        while (rrn < mch && rn < mch) {
            if (!R.has(refoff - rrn - 1)) break;
            if (rrn < rdoff && R.at(refoff - rrn - 1) != seq[rdoff - rrn - 1]) { rn = rrn + 1; rmch = 0; }
            else if (rrn < rdoff && R.at(refoff - rrn - 1) == seq[rdoff - rrn - 1]) rmch++;
            rrn++;
            if (rmch >= 3) break;
        }
        mch -= rn;
        if (rn > 0 && rn <= 3) rep_first(19, std::to_string(mch) + "M" + std::to_string(rn) + "S");
    }
    // captureMisSoftlyMS (:572-653)
    void mis_ms(const std::smatch &m) {
        string ov5 = m.str(1);
        int mch = I(m, 2), soft = I(m, 3), refoff = position + mch, rdoff = mch;
        if (!ov5.empty()) { refoff += sum_of(24, ov5); rdoff += sum_of(25, ov5); }
        int rn = 0;
        std::set<char> RN;
        while (rn < soft && eq(refoff + rn, rdoff + rn) && qual[rdoff + rn] > 10) rn++;
        if (rn > 0) {
            mch += rn;
            soft -= rn;
            rep_first(22, soft > 0 ? std::to_string(mch) + "M" + std::to_string(soft) + "S" : std::to_string(mch) + "M");
            rn = 0;
        }
        if (soft > 0) {
            while (rn + 1 < soft && eq(refoff + rn + 1, rdoff + rn + 1) && qual[rdoff + rn + 1] > 10) {
                rn++;
                if (R.has(refoff + rn + 1)) RN.insert(R.at(refoff + rn + 1));
            }
            int rn_nt = (int)RN.size();
            if (rn > 4 && rn_nt > 1) {
                mch += rn + 1;
                soft -= rn + 1;
                rep_first(22, soft > 0 ? std::to_string(mch) + "M" + std::to_string(soft) + "S"
                                       : std::to_string(mch) + "M");
            }
            if (rn == 0) {
                int rrn = 0, rmch = 0;
                while (rrn < mch && rn < mch) {
                    if (!R.has(refoff - rrn - 1)) break;
                    if (rrn < rdoff && R.at(refoff - rrn - 1) != seq[rdoff - rrn - 1]) { rn = rrn + 1; rmch = 0; }
                    else if (rrn < rdoff && R.at(refoff - rrn - 1) == seq[rdoff - rrn - 1]) rmch++;
                    rrn++;
                    if (rmch >= 3) break;
                }
                if (rn > 0 && rn < mch) {
                    soft += rn;
                    mch -= rn;
                    rep_first(22, std::to_string(mch) + "M" + std::to_string(soft) + "S");
                }
            }
        }
    }
    // combineToCloseToOne (:662-707)
    bool close_to_one(const std::smatch &m, bool flag) {
        string op = m.str(5);
        int g2 = I(m, 2), g3 = I(m, 3), g4 = I(m, 4);
        if (g3 <= 15) {
            int dlen = g3, ilen = g2 + g3;
            if (op == "I") ilen += g4;
            else if (op == "D") {
                dlen += g4;
                string istr = m.str(6);
                if (!istr.empty()) ilen += std::stoi(istr.substr(0, istr.size() - 1));
            }
            rep_first(14, std::to_string(dlen) + "D" + std::to_string(ilen) + "I");
            flag = true;
        }
        return flag;
    }
    // combineToCloseToCorrect (:717-745)
    bool close_to_correct(const std::smatch &m, bool flag) {
        int g1 = I(m, 1), g2 = I(m, 2), g3 = I(m, 3);
        if (g2 <= 15) {
            string op = m.str(4);
            int dlen = g1 + g2, ilen = g2;
            if (op == "I") ilen += g3;
            else if (op == "D") {
                dlen += g3;
                string istr = m.str(5);
                if (!istr.empty()) ilen += std::stoi(istr.substr(0, istr.size() - 1));
            }
            rep_first(13, std::to_string(dlen) + "D" + std::to_string(ilen) + "I");
            flag = true;
        }
        return flag;
    }
    // the matched-bases scan shared by the three-event rules
    int run_match(int rdoff, int refoff) const {
        int rn = 0;
        while (rdoff + rn < lseq && R.has(refoff + rn) && R.at(refoff + rn) == seq[rdoff + rn]) rn++;
        return rn;
    }
    // threeIndels (:755-846)
    bool three_indels(const std::smatch &m, bool flag) {
        int mid = I(m, 5) + I(m, 8), tslen = mid, dlen = mid;
        for (int k : {4, 7, 10}) {
            if (m.str(k) == "I") tslen += I(m, k - 1);
            if (m.str(k) == "D") dlen += I(m, k - 1);
        }
        string ov5 = m.str(1);
        int refoff = position + I(m, 2), rdoff = I(m, 2), RDOFF = I(m, 2), rm = I(m, 11);
        if (!ov5.empty()) { refoff += sum_of(24, ov5); rdoff += sum_of(25, ov5); }
        int rn = run_match(rdoff, refoff);
        RDOFF += rn;
        dlen -= rn;
        tslen -= rn;
        string nc = std::to_string(RDOFF) + "M";
        if (tslen <= 0) {
            dlen -= tslen;
            rm += tslen;
            if (dlen == 0) {
                RDOFF += rm;
                nc = std::to_string(RDOFF) + "M";
            } else if (dlen < 0) {
                tslen = -dlen;
                rm += dlen;
                if (rm < 0) {
                    RDOFF += rm;
                    nc = std::to_string(RDOFF) + "M" + std::to_string(tslen) + "I";
                } else {
                    nc += std::to_string(tslen) + "I" + std::to_string(rm) + "M";
                }
            } else {
                nc += std::to_string(dlen) + "D" + std::to_string(rm) + "M";
            }
        } else {
            if (dlen == 0) nc += std::to_string(tslen) + "I" + std::to_string(rm) + "M";
            else if (dlen < 0) { rm += dlen; nc += std::to_string(tslen) + "I" + std::to_string(rm) + "M"; }
            else nc += std::to_string(dlen) + "D" + std::to_string(tslen) + "I" + std::to_string(rm) + "M";
        }
        if (mid <= 15) { rep_first(11, nc); flag = true; }
        return flag;
    }
    // threeDeletions (:856-910)
    bool three_deletions(const std::smatch &m, bool flag) {
        int tslen = I(m, 4) + I(m, 6), dlen = I(m, 3) + I(m, 4) + I(m, 5) + I(m, 6) + I(m, 7);
        int mid = I(m, 4) + I(m, 6);
        string ov5 = m.str(1);
        int refoff = position + I(m, 2), rdoff = I(m, 2), RDOFF = I(m, 2), rm = I(m, 8);
        if (!ov5.empty()) { refoff += sum_of(24, ov5); rdoff += sum_of(25, ov5); }
        int rn = run_match(rdoff, refoff);
        RDOFF += rn;
        dlen -= rn;
        tslen -= rn;
        string nc = std::to_string(RDOFF) + "M";
        if (tslen <= 0) { dlen -= tslen; rm += tslen; nc += std::to_string(dlen) + "D" + std::to_string(rm) + "M"; }
        else nc += std::to_string(dlen) + "D" + std::to_string(tslen) + "I" + std::to_string(rm) + "M";
        if (mid <= 15) { rep_first(12, nc); flag = true; }
        return flag;
    }
    // twoDeletionsInsertionToComplex (:920-972)
    bool two_del_ins(const std::smatch &m, bool flag) {
        int tslen = I(m, 4) + I(m, 5) + I(m, 6), dlen = I(m, 3) + I(m, 4) + I(m, 6) + I(m, 7);
        int mid = I(m, 4) + I(m, 6);
        string ov5 = m.str(1);
        int mch = I(m, 2), refoff = position + mch, rdoff = mch, RDOFF = mch, rm = I(m, 8);
        if (!ov5.empty()) { refoff += sum_of(24, ov5); rdoff += sum_of(25, ov5); }
        int rn = run_match(rdoff, refoff);
        RDOFF += rn;
        dlen -= rn;
        tslen -= rn;
        string nc = std::to_string(RDOFF) + "M";
        if (tslen <= 0) { dlen -= tslen; rm += tslen; nc += std::to_string(dlen) + "D" + std::to_string(rm) + "M"; }
        else nc += std::to_string(dlen) + "D" + std::to_string(tslen) + "I" + std::to_string(rm) + "M";
        if (mid <= 15) { rep_first(8, nc); flag = true; }
        return flag;
    }
    // beginDigitMNumberIorDNumberM (:982-1000)
    bool begin_digit_m(const std::smatch &m) {
        int tmid = I(m, 1), mlen = I(m, 4), tn = 0;
        int tslen = tmid + (m.str(3) == "I" ? I(m, 2) : 0);
        position += tmid + (m.str(3) == "D" ? I(m, 2) : 0);
        while (tn < mlen && R.has(position + tn) && R.at(position + tn) != seq[tslen + tn]) tn++;
        tslen += tn;
        mlen -= tn;
        position += tn;
        rep_first(5, std::to_string(tslen) + "S" + std::to_string(mlen) + "M");
        return true;
    }

    // modifyCigar (:219-390) after the leading/trailing D and I handling,
    // which returns before reaching here for the CIGARs this restatement takes
    void rules(int indel) {
        std::smatch m;
        bool flag = true;
        while (flag && indel > 0) {
            flag = false;
            if (std::regex_search(cs, m, re(0))) {
                string t = std::to_string(I(m, 1) + (m.str(3) == "I" ? I(m, 2) : 0)) + "S";
                position += m.str(3) == "D" ? I(m, 2) : 0;
                rep_all(0, t);
                flag = true;
            }
            if (std::regex_search(cs, m, re(1))) {
                string t = std::to_string(I(m, 3) + (m.str(2) == "I" ? I(m, 1) : 0)) + "S";
                rep_all(1, t);
                flag = true;
            }
            if (std::regex_search(cs, m, re(2))) {
                int tmid = I(m, 2);
                if (tmid <= 10) {
                    string t = std::to_string(I(m, 1) + tmid + (m.str(4) == "I" ? I(m, 3) : 0)) + "S";
                    position += tmid + (m.str(4) == "D" ? I(m, 3) : 0);
                    rep_all(2, t);
                    flag = true;
                }
            }
            if (std::regex_search(cs, m, re(3))) {
                int tmid = I(m, 3);
                if (tmid <= 10) {
                    string t = std::to_string(I(m, 4) + tmid + (m.str(2) == "I" ? I(m, 1) : 0)) + "S";
                    rep_all(3, t);
                    flag = true;
                }
            }
            if (std::regex_search(cs, m, re(4))) flag = begin_digit_m(m);
            if (std::regex_search(cs, m, re(6))) {
                string t = std::to_string(I(m, 3) + (m.str(2) == "I" ? I(m, 1) : 0)) + "S";
                rep_all(6, t);
                flag = true;
            }
            std::smatch mt, md;
            bool m7 = std::regex_search(cs, m, re(7));
            bool m10 = std::regex_search(cs, mt, re(10));
            bool m9 = std::regex_search(cs, md, re(9));
            if (m7) flag = two_del_ins(m, flag);
            else if (m9) flag = three_deletions(md, flag);
            else if (m10) flag = three_indels(mt, flag);
            if (std::regex_search(cs, m, re(13))) flag = close_to_correct(m, flag);
            if (std::regex_search(cs, m, re(15)) && m.str(1) != "D" && m.str(1) != "H") flag = close_to_one(m, flag);
            if (std::regex_search(cs, m, re(16))) {
                rep_first(16, std::to_string(I(m, 1) + I(m, 2)) + "D");
                flag = true;
            }
            if (std::regex_search(cs, m, re(17))) {
                rep_first(17, std::to_string(I(m, 1) + I(m, 2)) + "I");
                flag = true;
            }
        }
        if (std::regex_search(cs, m, re(23))) mis_ms(m);
        else if (std::regex_search(cs, m, re(18))) mis3(m);
        if (std::regex_search(cs, m, re(21))) dig_s_dig_m(m);
        else if (std::regex_search(cs, m, re(20))) begin_dig_m(m);
    }
};

string cigar_string(const vector<uint32_t> &c, int n) {  // get_cigar_string (include/VariationUtils.h:563-570)
    string s;
    for (int i = 0; i < n; i++) s += std::to_string(c[i] >> 4) + "MIDNSHP=XB??????"[c[i] & 15];
    return s;
}

// cigarstr_2cigar (include/VariationUtils.h:608-629); false on a negative length
bool parse_cigar_string(string s, vector<uint32_t> &out) {
    out.clear();
    while (!s.empty()) {
        size_t po = 0;
        int num = std::stoi(s, &po);
        if (num < 0) return false;
        const char *ops = "MIDNSHP=XB";
        const char *q = strchr(ops, s[po]);
        int op = (q && s[po]) ? (int)(q - ops) : 0;
        out.push_back(((uint32_t)num << 4) | (uint32_t)op);
        s = s.substr(po + 1);
    }
    return true;
}

// ---------------------------------------------------------------------------
// per-read walk: CigarParser (src/parseCigar.cpp)
// ---------------------------------------------------------------------------
struct Walker {
    const rvo_params &P;
    Maps &M;
    Ref &R;
    int rs, re;  // region start/end
    int chr_len;
    // CigarParser members
    int start = 0, offset = 0, cel = 0, rpis = 0, rpes = 0, n_cigar = 0;
    vector<uint32_t> *cigar = nullptr;
    const ReadView *rv = nullptr;

    Walker(const rvo_params &p, Maps &m, Ref &r, int s, int e, int cl) : P(p), M(m), R(r), rs(s), re(e), chr_len(cl) {}

    static int op(uint32_t c) { return (int)(c & 15); }
    static int oplen(uint32_t c) { return (int)(c >> 4); }
    int cop(int i) const { return op((*cigar)[i]); }
    int clen_(int i) const { return oplen((*cigar)[i]); }

    Stat &getvar(map<int, KeyMap> &h, int p, const string &k) { return h[p][k]; }

    // addCnt: src/parseCigar.cpp:318-343
    void add_cnt(Stat &v, bool dir, int rp, double bq, int mq, int nm) {
        v.cnt++;
        dir ? v.rev++ : v.fwd++;
        v.pmean += rp;
        v.qmean += bq;
        v.mq += mq;
        v.nm += nm;
        if (bq >= P.goodq) v.hi++; else v.lo++;
    }

    int tp_of(int rlen) const {  // src/parseCigar.cpp:896-898
        return rpes < rlen - rpes ? rpes + 1 : rlen - rpes;
    }

    void pq_update(Stat &v, int tp, double q) {  // pstd/qstd rule, src/parseCigar.cpp:902-914
        if (!v.pstd && v.pp != 0 && tp != v.pp) v.pstd = true;
        if (!v.qstd && v.pq != 0 && q != v.pq) v.qstd = true;
    }

    // isTrimAtOptTBases: src/parseCigar.cpp:158-167
    bool trim(bool dir, int tlen) const {
        if (P.trim_bases_after != 0) {
            if (!dir) return rpis > P.trim_bases_after;
            return tlen - rpis > P.trim_bases_after;
        }
        return false;
    }

    // findOffset: src/parseCigar.cpp:208-256
    int find_offset(int refp, int readp, int clen, string &sq, long &qsum, int &tnm) {
        const vector<char> &s = rv->seq;
        const uint8_t *q = rv->qual();
        int off = 0, vsn = 0;
        tnm = 0;
        for (int vi = 0; vsn <= P.vext && vi < clen; vi++) {
            if (s[readp + vi] == 'N') break;
            if (q[readp + vi] < P.goodq) break;
            if (R.has(refp + vi)) {
                if (s[readp + vi] != R.at(refp + vi)) { off = vi + 1; tnm++; vsn = 0; }
                else vsn++;
            }
        }
        qsum = 0;
        sq.clear();
        if (off > 0) {
            sq.assign(&s[readp], off);
            for (int i = readp; i < readp + off; i++) qsum += q[i];
            for (int i = 0; i < off; i++) M.cov[refp + i]++;
        }
        return off;
    }

    // isInsertionOrDeletionWithNextMatched: src/parseCigar.cpp:1817-1826
    // (reads the CIGAR word at ci+3 even when it lies past the last op)
    bool indel_next_matched(int ci) const {
        return P.local_realign && n_cigar > ci + 2 && clen_(ci + 1) <= P.vext && cop(ci + 1) == OP_M &&
               (cop(ci + 2) == OP_I || cop(ci + 2) == OP_D) && cop(ci + 3) != OP_I && cop(ci + 3) != OP_D;
    }
    bool next_matched(int ci) const { return P.local_realign && n_cigar > ci + 1 && cop(ci + 1) == OP_M; }
    bool next_after_num_matched(int ci, int number) const {  // src/parseCigar.cpp:1084-1087
        return n_cigar > ci + number && cop(ci + 1) == OP_M;
    }

    // appendSegments: src/parseCigar.cpp:1756-1815
    void append_segments(int ci, string &desc, long &qsum, int &qcnt, int mlen, int indel_len, int begin, bool is_ins) {
        const vector<char> &s = rv->seq;
        const uint8_t *q = rv->qual();
        desc += "#";
        desc.append(&s[begin], mlen);
        for (int i = begin; i < begin + mlen; i++) qsum += q[i];
        desc += "^";
        if (cop(ci + 2) == OP_I) desc.append(&s[begin + mlen], indel_len);
        else desc += std::to_string(indel_len);
        if (cop(ci + 2) == OP_I) {
            for (int i = begin + mlen; i < begin + mlen + indel_len; i++) qsum += q[i];
            qcnt += indel_len;
        } else if (is_ins) {
            qsum += q[begin + mlen];
            qcnt += 1;
        }
    }

    // process_softclip: src/parseCigar.cpp:1112-1301
    void softclip(int ci, bool dir, int mapq, int nom, int position, int tlen) {
        const vector<char> &s = rv->seq;
        const uint8_t *q = rv->qual();
        if (ci == 0) {
            while (cel - 1 >= 0 && start - 1 > 0 && start - 1 <= chr_len && R.has_eq(s[cel - 1], start - 1) &&
                   q[cel - 1] > 10) {
                Stat &v = getvar(M.nonins, start - 1, string(1, R.idx(start - 1)));
                add_cnt(v, dir, cel, q[cel - 1], mapq, nom);
                M.cov[start - 1]++;
                start--;
                cel--;
            }
            if (cel > 0) {
                int sumq = 0, nhq = 0, nlq = 0;
                for (int si = cel - 1; si >= 0; si--) {
                    if (s[si] == 'N') break;
                    int bq = q[si];
                    if (bq <= 12) nlq++;
                    if (nlq > 1) break;
                    sumq += bq;
                    nhq++;
                }
                if (nhq >= 1 && nhq > nlq && start >= rs && start <= re) {
                    Clip &sc = M.sc5[start];
                    for (int si = cel - 1; cel - si <= nhq; si--) {
                        char ch = s[si];
                        int idx = cel - 1 - si;
                        sc.nt[idx][ch]++;
                        add_cnt(sc.seq[idx][ch], dir, si - (cel - nhq), q[si], mapq, nom);
                    }
                    add_cnt(sc, dir, cel, sumq / (double)nhq, mapq, nom);
                }
            }
            cel = clen_(ci);
        } else if (ci == n_cigar - 1) {
            while (rpis < rv->lseq && R.has_eq(s[rpis], start) && q[rpis] > 10) {
                Stat &v = getvar(M.nonins, start, string(1, R.at(start)));
                add_cnt(v, dir, tlen - rpes, q[rpis], mapq, nom);
                M.cov[start]++;
                rpis++;
                start++;
                cel--;
                rpes++;
            }
            if (rpis < rv->lseq) {
                int sumq = 0, nhq = 0, nlq = 0;
                for (int si = 0; si < cel; si++) {
                    if (s[rpis + si] == 'N') break;
                    int bq = q[rpis + si];
                    if (bq <= 12) nlq++;
                    if (nlq > 1) break;
                    sumq += bq;
                    nhq++;
                }
                if (nhq >= 1 && nhq > nlq && start >= rs && start <= re) {
                    Clip &sc = M.sc3[start];
                    for (int si = 0; si < nhq; si++) {
                        char ch = s[rpis + si];
                        sc.nt[si][ch]++;
                        add_cnt(sc.seq[si][ch], dir, nhq - si, q[rpis + si], mapq, nom);
                    }
                    add_cnt(sc, dir, cel, sumq / (double)nhq, mapq, nom);
                }
            }
        }
        rpis += cel;
        offset = 0;
        start = position;
    }

    // adjInsPos: include/VariationUtils.h:99-113 (3' rotation of an
    // all-ACGT insertion while the preceding reference base repeats it)
    int adj_ins_pos(int bi, string &ins) {
        int n = 1;
        int len = (int)ins.size();
        while (R.idx(bi) == ins[len - n]) {
            n++;
            if (n > len) n = 1;
            bi--;
        }
        if (n > 1) ins = ins.substr(len - (n - 1)) + ins.substr(0, len - (n - 1));
        return bi;
    }

    static bool all_acgt(const string &s) {
        if (s.empty()) return false;
        for (char c : s)
            if (c != 'A' && c != 'C' && c != 'G' && c != 'T') return false;
        return true;
    }

    // process_insertion: src/parseCigar.cpp:1303-1523
    int insertion(int ci, bool dir, int mapq, int nom, int position, int rlen) {
        const vector<char> &s = rv->seq;
        const uint8_t *q = rv->qual();
        if ((n_cigar > ci + 1 && cop(ci + 1) == OP_N) || (ci > 0 && cop(ci - 1) == OP_N)) {
            rpis += cel;
            return ci;
        }
        string desc(&s[rpis], cel);
        long qsum = 0;
        int qcnt = 0;
        for (int i = rpis; i < rpis + cel; i++) qsum += q[i];
        qcnt += cel;
        string ss;
        int multoffs = 0, multoffp = 0, nmoff = 0;
        if (indel_next_matched(ci)) {
            int mlen = clen_(ci + 1), indel_len = clen_(ci + 2);
            int begin = rpis + cel;
            append_segments(ci, desc, qsum, qcnt, mlen, indel_len, begin, true);
            multoffs += mlen + (cop(ci + 2) == OP_D ? indel_len : 0);
            multoffp += mlen + (cop(ci + 2) == OP_I ? indel_len : 0);
            int ci6 = n_cigar > ci + 3 ? clen_(ci + 3) : 0;
            if (ci6 != 0 && cop(ci + 3) == OP_M) {
                long qs;
                int tnm;
                offset = find_offset(start + multoffs, rpis + cel + multoffp, ci6, ss, qs, tnm);
                qsum += qs;
                qcnt += offset;
            }
            ci += 2;
        } else if (next_matched(ci)) {
            int vsn = 0;
            for (int vi = 0; vsn <= P.vext && vi < clen_(ci + 1); vi++) {
                if (s[rpis + cel + vi] == 'N') break;
                if (q[rpis + cel + vi] < P.goodq) break;
                if (R.has(start + vi)) {
                    if (s[rpis + cel + vi] != R.at(start + vi)) { offset = vi + 1; nmoff++; vsn = 0; }
                    else vsn++;
                }
            }
            if (offset != 0) {
                ss.append(&s[rpis + cel], offset);
                for (int i = rpis + cel; i < rpis + cel + offset; i++) qsum += q[i];
                qcnt += offset;
                for (int osi = 0; osi < offset; osi++) M.cov[start + osi]++;
            }
        }
        if (offset > 0) desc += "&" + ss;
        if (start - 1 >= rs && start - 1 <= re && desc.find('N') == string::npos) {
            int inspos = start - 1;
            if (all_acgt(desc)) {
                string d2 = desc;
                int bi = adj_ins_pos(start - 1, d2);
                if (rpis - 1 - (start - 1 - bi) > 0) {
                    inspos = bi;
                    desc = d2;
                }
            }
            string key = "+" + desc;
            M.inscnt[inspos][key]++;
            Stat &hv = getvar(M.ins, inspos, key);
            hv.inc_dir(dir);
            hv.cnt++;
            int tp = tp_of(rlen);
            double tmpq = (double)qsum / qcnt;
            pq_update(hv, tp, tmpq);
            hv.pmean += tp;
            hv.qmean += tmpq;
            hv.mq += mapq;
            hv.pp = tp;
            hv.pq = tmpq;
            if (tmpq >= P.goodq) hv.hi++; else hv.lo++;
            hv.nm += nom - nmoff;
            int index = rpis - 1 - (start - 1 - inspos);
            if (inspos > position && R.has_eq(s[index], inspos)) {
                // getVariationMaybe: the subtraction applies only if the key exists now
                auto it = M.nonins.find(inspos);
                if (it != M.nonins.end()) {
                    auto it2 = it->second.find(string(1, s[index]));
                    if (it2 != it->second.end()) {
                        Stat &tv = it2->second;
                        tv.cnt--;
                        dir ? tv.rev-- : tv.fwd--;
                        tv.pmean -= tp;
                        tv.qmean -= q[index];
                        tv.mq -= mapq;
                        tv.nm -= (nom - nmoff);
                        if (q[index] >= P.goodq) tv.hi--; else tv.lo--;
                    }
                }
            }
            if (ci == 1 && (cop(0) == OP_S || cop(0) == OP_H)) {
                Stat &tt = getvar(M.nonins, inspos, string(1, R.idx(inspos)));
                tt.inc_dir(dir);
                tt.cnt++;
                tt.pstd = hv.pstd;
                tt.qstd = hv.qstd;
                tt.pmean += tp;
                tt.qmean += tmpq;
                tt.mq += mapq;
                tt.pp = tp;
                tt.pq = tmpq;
                tt.nm += nom - nmoff;
                M.cov[inspos]++;
            }
        }
        rpis += cel + offset + multoffp;
        rpes += cel + offset + multoffp;
        start += offset + multoffs;
        return ci;
    }

    // process_deletion + addVariationForDeletion: src/parseCigar.cpp:1525-1727, 1036-1082
    int deletion(int ci, bool dir, int mapq, int nom, int rlen) {
        const vector<char> &s = rv->seq;
        const uint8_t *q = rv->qual();
        if ((n_cigar > ci && cop(ci + 1) == OP_N) || (ci > 1 && cop(ci - 1) == OP_N)) {
            rpis += cel;
            return ci;
        }
        string desc = "-" + std::to_string(cel);
        string app;
        uint8_t qlast = q[rpis - 1];
        long qsum = 0;
        int qcnt = 0;
        int multoffs = 0, multoffp = 0, nmoff = 0;
        if (indel_next_matched(ci)) {
            int mlen = clen_(ci + 1), indel_len = clen_(ci + 2);
            append_segments(ci, desc, qsum, qcnt, mlen, indel_len, rpis, false);
            multoffs += mlen + (cop(ci + 2) == OP_D ? indel_len : 0);
            multoffp += mlen + (cop(ci + 2) == OP_I ? indel_len : 0);
            if (next_after_num_matched(ci, 3)) {
                int vsn = 0, tn = rpis + multoffp, ts = start + multoffs + cel;
                for (int vi = 0; vsn <= P.vext && vi < clen_(ci + 3); vi++) {
                    if (s[tn + vi] == 'N') break;
                    if (q[tn + vi] < P.goodq) break;
                    if (R.has_eq('N', ts + vi)) break;
                    if (R.has(ts + vi)) {
                        if (s[tn + vi] != R.at(ts + vi)) { offset = vi + 1; nmoff++; vsn = 0; }
                        else vsn++;
                    }
                }
                if (offset != 0) {
                    app.append(&s[tn], offset);
                    for (int i = tn; i < tn + offset; i++) qsum += q[i];
                    qcnt += offset;
                }
            }
            ci += 2;
        } else if (P.local_realign && n_cigar > ci + 1 && cop(ci + 1) == OP_I) {
            int ins_len = clen_(ci + 1);
            desc += "^";
            desc.append(&s[rpis], ins_len);
            for (int i = rpis; i < rpis + ins_len; i++) qsum += q[i];
            qcnt += ins_len;
            multoffp += ins_len;
            // the reference's follow-up scan here requires op(ci+1) == M, which
            // cannot hold when op(ci+1) == I (src/parseCigar.cpp:1598-1626)
            ci += 1;
        } else if (next_matched(ci)) {
            int mlen = clen_(ci + 1), vsn = 0;
            for (int vi = 0; vsn <= P.vext && vi < mlen; vi++) {
                char sc = s[rpis + vi];
                if (sc == 'N') break;
                if (q[rpis + vi] < P.goodq) break;
                if (R.has(start + cel + vi)) {
                    char rc = R.at(start + cel + vi);
                    if (rc == 'N') break;
                    if (sc != rc) { offset = vi + 1; nmoff++; vsn = 0; }
                    else vsn++;
                }
            }
            if (offset != 0) {
                app.append(&s[rpis], offset);
                for (int i = rpis; i < rpis + offset; i++) qsum += q[i];
                qcnt += offset;
            }
        }
        if (offset > 0) desc += "&" + app;
        if (rpis + offset >= rv->lseq) {
            qsum += qlast;
            qcnt += 1;
        } else {
            uint8_t qo = q[rpis + offset];
            qsum += qlast > qo ? qlast : qo;
            qcnt += 1;
        }
        if (start >= rs && start <= re) {
            Stat &hv = getvar(M.nonins, start, desc);
            M.delcnt[start][desc]++;
            hv.inc_dir(dir);
            hv.cnt++;
            int tp = tp_of(rlen);
            double tmpq = (double)qsum / qcnt;
            pq_update(hv, tp, tmpq);
            hv.pmean += tp;
            hv.qmean += tmpq;
            hv.mq += mapq;
            hv.pp = tp;
            hv.pq = tmpq;
            hv.nm += nom - nmoff;
            if (tmpq >= P.goodq) hv.hi++; else hv.lo++;
            for (int i = 0; i < cel; i++) M.cov[start + i]++;
        }
        start += cel + offset + multoffs;
        rpis += offset + multoffp;
        rpes += offset + multoffp;
        return ci;
    }

    static bool is_mnv_key(const string &k) {  // isBEGIN_ATGC_AMP_ATGCs_END: src/parseCigar.cpp:476-495
        if (k.size() <= 2 || k[1] != '&') return false;
        auto acgt = [](char c) { return c == 'A' || c == 'C' || c == 'G' || c == 'T'; };
        if (!acgt(k[0])) return false;
        for (size_t i = 2; i < k.size(); i++)
            if (!acgt(k[i])) return false;
        return true;
    }

    // skipOverlappingReads / isReadsOverlap: src/parseCigar.cpp:180-206
    bool skip_overlapping(int position, bool dir, int mate_start, int orig_ref_len, int endpos) const {
        const ReadView &r = *rv;
        bool paired_same = (r.flag & 1) && true;  // tid == mtid for single-contig inputs
        if (P.unique_fwd && paired_same && !dir && start >= mate_start) return true;
        if (P.unique_first && (r.flag & 1) && paired_same) {
            bool ov;
            if (position >= mate_start) ov = start >= mate_start && start <= mate_start + orig_ref_len - 1;
            else ov = start >= mate_start && r.mpos + 1 <= endpos;
            if (ov) return true;
        }
        return false;
    }

    // parseCigar: src/parseCigar.cpp:497-974
    void parse(const ReadView &r) {
        rv = &r;
        vector<uint32_t> cg = r.cig;
        cigar = &cg;
        n_cigar = r.n_cigar;
        if (n_cigar <= 0) return;
        const vector<char> &s = r.seq;
        const uint8_t *q = r.qual();
        int idl = 0;
        for (int i = 0; i < n_cigar; i++)
            if (cop(i) == OP_I || cop(i) == OP_D) idl += clen_(i);
        int nom = 0;
        if (r.nm != INT32_MIN) {
            nom = r.nm - idl;
            if (nom > P.mismatch) return;
        } else if (r.flag & 4) {
            return;
        }
        bool dir = (r.flag & 16) != 0;
        int mapq = r.mapq;
        int position = r.pos + 1;
        rpis = rpes = 0;
        if (P.local_realign) {
            // CigarModifier (src/parseCigar.cpp:547-571): the rewritten CIGAR is
            // written over the record's CIGAR words (and the bytes after them when
            // it is longer); the walk reads the new count from the same address
            if (op(cg[0]) == OP_D) throw UnsupportedRead();  // the :249 pointer shift is not restated
            int nm_ = n_cigar;
            if (cg[nm_ - 1] == OP_D) nm_--;                       // whole-word compare (:251)
            if (op(cg[0]) == OP_I) cg[0] = (cg[0] & ~15u) | OP_D;  // a leading I becomes D (:253-255)
            if (cg[nm_ - 1] == OP_I) cg[nm_ - 1] = OP_D;          // whole-word compare (:256-258)
            CigarMod cm{R, s, q, r.lseq, position, cigar_string(cg, nm_)};
            const string orig = cigar_string(r.cig, r.n_cigar);
            cm.rules(idl);
            if (cm.cs != orig) {
                vector<uint32_t> nc;
                bool ok = parse_cigar_string(cm.cs, nc);
                if (!ok) parse_cigar_string(orig, nc);  // a negative length: the original CIGAR is written back
                if (nc.size() > (size_t)r.n_cigar + 3) throw UnsupportedRead();
                for (size_t k = 0; k < nc.size(); k++) cg[k] = nc[k];
                if (ok) {
                    n_cigar = (int)nc.size();
                    position = cm.position;
                }
            }
        }
        // cleanupCigar: src/parseCigar.cpp:1858-1892
        for (int pass = 0; pass < 2; pass++) {
            bool none = true;
            for (int k = 0; k < n_cigar && none; k++) {
                int c = pass == 0 ? k : n_cigar - 1 - k;
                int o = cop(c);
                if (o == OP_I) cg[c] = (cg[c] & ~15u) | OP_S;
                else if (o == 0 || o == 7 || o == 8) none = false;
            }
        }
        start = position;
        offset = 0;
        if (cop(0) == OP_S && clen_(0) >= 10 && cop(n_cigar - 1) == OP_S && clen_(n_cigar - 1) >= 10) return;
        int rlen = 0, tlen = 0;
        for (int i = 0; i < n_cigar; i++) {
            int o = cop(i);
            if (o == OP_M || o == OP_I) rlen += clen_(i);
            if (o == OP_M || o == OP_I || o == OP_S) tlen += clen_(i);
        }
        if (P.minmatch != 0 && rlen < P.minmatch) return;
        if (tlen > M.max_read_len) M.max_read_len = tlen;
        if (r.flag & 2048) return;
        int mate_start = r.mpos + 1;
        int orig_ref_len = 0;
        for (int i = 0; i < r.n_cigar; i++) {
            int o = op(cg[i]);
            if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) orig_ref_len += oplen(cg[i]);
        }
        int endpos = orig_ref_len ? r.pos + orig_ref_len : r.pos + 1;
        bool need_break = true;
        for (int ci = 0; ci < n_cigar; ++ci) {
            if (need_break && skip_overlapping(position, dir, mate_start, orig_ref_len, endpos)) break;
            need_break = false;
            int c_op = cop(ci);
            cel = clen_(ci);
            if ((ci == 0 || ci == n_cigar - 1) && c_op == OP_I) c_op = OP_S;
            if (c_op == OP_N) {  // processNotMatched: src/parseCigar.cpp:1733-1753
                start += cel;
                offset = 0;
                continue;
            }
            if (c_op == OP_S) { softclip(ci, dir, mapq, nom, position, tlen); continue; }
            if (c_op == OP_H) { offset = 0; continue; }
            if (c_op == OP_I) { offset = 0; ci = insertion(ci, dir, mapq, nom, position, rlen); continue; }
            if (c_op == OP_D) { offset = 0; ci = deletion(ci, dir, mapq, nom, rlen); continue; }
            int nmoff = 0, moffset = 0;
            for (int i = offset; i < cel; i++) {
                bool tr = trim(dir, tlen);
                char ch1 = s[rpis];
                string key(1, ch1);
                bool swd = false;
                if (ch1 == 'N') {
                    start++;
                    rpis++;
                    rpes++;
                    continue;
                }
                double qv = q[rpis];
                int qbases = 1, qibases = 0;
                string ss;
                // MNV growth: src/parseCigar.cpp:711-767
                while ((start + 1) >= rs && (start + 1) <= re && (i + 1) < cel && qv >= P.goodq &&
                       R.has_ne(s[rpis], start) && R.idx(start) != 'N') {
                    if (q[rpis + 1] < P.goodq + 5) break;
                    char nuc = s[rpis + 1];
                    if (nuc == 'N') break;
                    if (R.has_eq('N', start + 1)) break;
                    if (R.idx(start + 1) != nuc) {
                        ss += nuc;
                        qv += q[rpis + 1];
                        qbases++;
                        rpis++;
                        rpes++;
                        i++;
                        start++;
                        nmoff++;
                    } else {
                        int ssn = 0;
                        for (int ssi = 1; ssi <= P.vext; ssi++) {
                            if (i + 1 + ssi >= cel) break;
                            if (rpis + 1 + ssi < r.lseq && R.has_ne(s[rpis + 1 + ssi], start + 1 + ssi)) {
                                ssn = ssi + 1;
                                break;
                            }
                        }
                        if (ssn == 0) break;
                        if (q[rpis + ssn] < P.goodq + 5) break;
                        for (int ssi = 1; ssi <= ssn; ssi++) {
                            ss += s[rpis + ssi];
                            qv += q[rpis + ssi];
                            qbases++;
                        }
                        rpis += ssn;
                        rpes += ssn;
                        i += ssn;
                        start += ssn;
                    }
                }
                if (!ss.empty()) key = key + "&" + ss;
                int ddlen = 0;
                // complex deletion / insertion tails: src/parseCigar.cpp:779-882
                if (P.local_realign && cel - i <= P.vext && ci + 1 < n_cigar && cop(ci + 1) == OP_D && R.has(start) &&
                    (!ss.empty() || s[rpis] != R.at(start)) && q[rpis] >= P.goodq) {
                    while (i + 1 < cel) {
                        key += s[rpis + 1];
                        qv += q[rpis + 1];
                        qbases++;
                        i++;
                        rpis++;
                        rpes++;
                        start++;
                    }
                    size_t amp = key.find('&');
                    if (amp != string::npos) key.erase(amp, 1);
                    key = "-" + std::to_string(clen_(ci + 1)) + "&" + key;
                    swd = true;
                    ddlen = clen_(ci + 1);
                    ci += 1;
                    if (n_cigar > ci + 1 && cop(ci + 1) == OP_I) {
                        int nl = clen_(ci + 1);
                        key += "^";
                        key.append(&s[rpis + 1], nl);
                        for (int qi = 1; qi <= nl; qi++) {
                            qv += q[rpis + 1 + qi];
                            qibases++;
                        }
                        rpis += nl;
                        rpes += nl;
                        ci += 1;
                    }
                    if (next_after_num_matched(ci, 1)) {
                        string sq;
                        long qs;
                        int tnm;
                        int to = find_offset(start + ddlen + 1, rpis + 1, clen_(ci + 1), sq, qs, tnm);
                        if (to != 0) {
                            moffset = to;
                            nmoff += tnm;
                            key += "&" + sq;
                            // the reference adds an always-empty quality string here
                        }
                    }
                } else if (P.local_realign && cel - i <= P.vext && ci + 1 < n_cigar && cop(ci + 1) == OP_I &&
                           R.has(start) && (!ss.empty() || s[rpis] != R.at(start)) && q[rpis] >= P.goodq) {
                    while (i + 1 < cel) {
                        key += s[rpis + 1];
                        qv += q[rpis + 1];
                        qbases++;
                        i++;
                        rpis++;
                        rpes++;
                        start++;
                    }
                    size_t amp = key.find('&');
                    if (amp != string::npos) key.erase(amp, 1);
                    int nl = clen_(ci + 1);
                    key.append(&s[rpis + 1], nl);
                    key.insert((size_t)nl, "&");
                    key = "+" + key;
                    for (int qi = 1; qi <= nl; qi++) {
                        qv += q[rpis + 1 + qi];
                        qibases++;
                    }
                    rpis += nl;
                    rpes += nl;
                    ci += 1;
                    qibases--;
                    qbases++;
                }
                if (!tr) {
                    int p = start - qbases + 1;
                    if (p >= rs && p <= re) {
                        Stat &hv = getvar(M.nonins, p, key);
                        hv.inc_dir(dir);
                        if (is_mnv_key(key)) M.mnp[p][key]++;
                        hv.cnt++;
                        int tp = tp_of(rlen);
                        qv = qv / (qbases + qibases);
                        pq_update(hv, tp, qv);
                        hv.pmean += tp;
                        hv.qmean += qv;
                        hv.mq += mapq;
                        hv.pp = tp;
                        hv.pq = qv;
                        hv.nm += nom - nmoff;
                        if (qv >= P.goodq) hv.hi++; else hv.lo++;
                        for (int qi = 1; qi <= qbases; qi++) M.cov[start - qi + 1]++;
                        if (swd) {
                            M.delcnt[p][key]++;
                            for (int qi = 1; qi < ddlen; qi++) M.cov[start + qi]++;
                        }
                    }
                }
                if (swd) start += ddlen;
                if (c_op != OP_I) start++;
                if (c_op != OP_D) {
                    rpis++;
                    rpes++;
                }
            }
            if (moffset != 0) {
                offset = moffset;
                rpis += moffset;
                start += moffset;
                rpes += moffset;
            }
            if (start > re) break;
        }
    }
};

// ---------------------------------------------------------------------------
// local realigner, MNP part: VariationRealigner::adjustMNP
// (src/VariationRealigner.cpp:334-465)
// ---------------------------------------------------------------------------
// The reference iterates the per-offset base counts of a soft clip in its
// hash map's order; for the keys A,C,G,T,N that order was measured to be
// N, A, T, G, C regardless of insertion order.
int char_rank(char c) {
    switch (c) {
    case 'N': return 0;
    case 'A': return 1;
    case 'T': return 2;
    case 'G': return 3;
    case 'C': return 4;
    default: return 5 + (unsigned char)c;
    }
}

bool low_complexity(const string &seq) {  // islowcomplexseq: include/VariationUtils.h:366-395
    int len = (int)seq.size();
    if (len == 0) return true;
    int ntcnt = 0;
    for (char b : string("ATGC")) {
        int c = (int)std::count(seq.begin(), seq.end(), b);
        if (c > 0) ntcnt++;
        if (c / (double)len > 0.75) return true;
    }
    return ntcnt < 3;
}

// findconseq: include/VariationUtils.h:403-509
string consensus(Clip &sc) {
    if (!sc.cons.empty()) return sc.cons;
    int total = 0, match = 0;
    string seqq;
    bool flag = false;
    for (auto &nve : sc.nt) {
        int pos_in = nve.first;
        vector<std::pair<char, int>> nv(nve.second.begin(), nve.second.end());
        std::sort(nv.begin(), nv.end(), [](const std::pair<char, int> &a, const std::pair<char, int> &b) {
            return char_rank(a.first) < char_rank(b.first);
        });
        int maxc = 0, tt = 0;
        double maxq = 0;
        char chosen = 0;
        for (auto &e : nv) {
            tt += e.second;
            double sq = 0;
            bool has = false;
            auto it = sc.seq.find(pos_in);
            if (it != sc.seq.end()) {
                auto it2 = it->second.find(e.first);
                if (it2 != it->second.end()) { has = true; sq = it2->second.qmean; }
            }
            if (e.second > maxc || (has && sq > maxq)) {
                maxc = e.second;
                chosen = e.first;
                maxq = has ? sq : 0;  // operator[] creates an empty entry when absent
            }
        }
        if (pos_in == 3 && sc.nt.size() >= 6 && tt / (double)sc.cnt < 0.2 && tt <= 2) break;
        if ((tt - maxc > 2 || maxc <= tt - maxc) && maxc / (double)tt < 0.8) {
            if (flag) break;
            flag = true;
        }
        total += tt;
        match += maxc;
        if (chosen != 0) seqq += chosen;
    }
    string SEQ;
    int nts = (int)sc.nt.size();
    int sl = (int)seqq.size();
    if (total != 0 && match / (double)total > 0.9 && sl / 1.5 > nts - sl &&
        (sl / (double)nts > 0.8 || nts - sl < 10 || sl > 25))
        SEQ = seqq;
    else
        SEQ = " ";
    if (!SEQ.empty() && SEQ.size() > 12) {  // CONF_SEED_2
        bool a7 = SEQ.size() >= 8 && SEQ.compare(1, 7, "AAAAAAA") == 0;
        bool t7 = SEQ.size() >= 8 && SEQ.compare(1, 7, "TTTTTTT") == 0;
        if (a7 || t7) sc.used = true;
        if (low_complexity(SEQ)) sc.used = true;
    }
    sc.cons = SEQ;
    return SEQ;
}

void adj_cnt(Stat &to, const Stat &v) {  // adjCnt: include/VariationUtils.h:338-352
    to.cnt += v.cnt;
    to.extracnt += v.cnt;
    to.hi += v.hi;
    to.lo += v.lo;
    to.pmean += v.pmean;
    to.qmean += v.qmean;
    to.mq += v.mq;
    to.nm += v.nm;
    to.pstd = true;
    to.qstd = true;
    to.rev += v.rev;
    to.fwd += v.fwd;
}

// ismatchref: src/VariationRealigner.cpp:2004-2024 (MM = 3)
bool ismatchref(const string &sq, Ref &R, int position, int dir) {
    int mm = 0;
    int len = (int)sq.size();
    for (int n = 0; n < len; n++) {
        if (!R.has(position + dir * n)) return false;
        char c = dir == 1 ? sq[n] : sq[len - n - 1];
        if (c != R.idx(position + dir * n)) mm++;
    }
    return mm <= 3 && mm / (double)len < 0.15;
}

void adjust_mnp(Maps &M, Ref &R) {
    struct T { int pos; string key; int cnt; };
    vector<T> tmp;
    for (auto &pe : M.mnp)
        for (auto &ke : pe.second) tmp.push_back({pe.first, ke.first, ke.second});
    // fillAndSortTmp / CMP_tmp: src/VariationRealigner.cpp:44-58, 1362-1386
    std::sort(tmp.begin(), tmp.end(), [](const T &a, const T &b) {
        if (a.cnt != b.cnt) return a.cnt > b.cnt;
        if (a.pos != b.pos) return a.pos < b.pos;
        return a.key.compare(b.key) > 0;
    });
    for (const T &t : tmp) {
        int position = t.pos;
        const string &vn = t.key;
        auto pit = M.nonins.find(position);
        if (pit == M.nonins.end()) continue;
        std::set<string> local;  // keys of the by-value copy the reference iterates
        for (auto &e : pit->second) local.insert(e.first);
        if (!local.count(vn)) continue;
        Stat &vref = pit->second.at(vn);
        string mnt = vn;
        size_t amp = mnt.find('&');
        if (amp != string::npos) mnt.erase(amp, 1);
        int ml = (int)mnt.size();
        for (int i = 0; i < ml - 1; i++) {
            string left = mnt.substr(0, i + 1);
            if (left.size() > 1) left.insert(1, "&");
            string right = mnt.substr(i + 1);
            if (right.size() > 1) right.insert(1, "&");
            if (local.count(left)) {
                Stat &tref = pit->second.at(left);
                if (tref.cnt <= 0) continue;
                if (tref.cnt < vref.cnt && tref.pmean / tref.cnt <= i + 1) {
                    adj_cnt(vref, tref);
                    local.erase(left);
                }
            }
            auto rit = M.nonins.find(position + i + 1);
            if (rit != M.nonins.end()) {
                auto kit = rit->second.find(right);
                if (kit != rit->second.end()) {
                    Stat &tref = kit->second;
                    if (tref.cnt < 0) continue;
                    if (tref.cnt < vref.cnt) {
                        adj_cnt(vref, tref);
                        M.cov[position] += tref.cnt;
                        rit->second.erase(kit);
                    }
                }
            }
        }
        auto s3 = M.sc3.find(position);
        if (s3 != M.sc3.end() && !s3->second.used) {
            string sq = consensus(s3->second);
            if (sq.compare(0, ml, mnt) == 0 && (int)sq.size() >= ml) {
                if ((int)sq.size() == ml || ismatchref(sq.substr(ml), R, position + ml, 1)) {
                    adj_cnt(pit->second[vn], s3->second);
                    M.cov[position] += s3->second.cnt;
                    s3->second.used = true;
                }
            }
        }
        auto s5 = M.sc5.find(position + ml);
        if (s5 != M.sc5.end() && !s5->second.used) {
            string sq = consensus(s5->second);
            if (sq != " " && (int)sq.size() >= ml) {
                std::reverse(sq.begin(), sq.end());
                if (sq.substr(sq.size() - ml, ml) == mnt) {
                    if ((int)sq.size() == ml || ismatchref(sq.substr(0, sq.size() - ml), R, position - 1, -1)) {
                        adj_cnt(pit->second[vn], s5->second);
                        M.cov[position] += s5->second.cnt;
                        s5->second.used = true;
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// -k 1 indel realignment: VariationRealigner::realignIndels
// (src/VariationRealigner.cpp:467-1360) with its helpers (:1396-1990)
// ---------------------------------------------------------------------------
struct RefFail {};

string join_ref(Ref &R, int from, int to) {  // joinRef: include/VariationUtils.h:356-362 (.at throws)
    string s;
    for (int i = from; i <= to; i++) {
        if (!R.has(i)) throw RefFail();
        s += R.at(i);
    }
    return s;
}

void replace_first(string &s, const string &a, const string &b) {
    size_t p = s.find(a);
    if (p != string::npos) s.replace(p, a.size(), b);
}

struct OutOfRange {};  // std::out_of_range from string::substr (caught per candidate)

string vsub(const string &s, int idx) {  // vc_substr(str, idx): include/util.h:27-34
    // `str.length() + idx < 0` is an unsigned comparison there: too negative
    // an index wraps and substr throws
    size_t b = idx >= 0 ? (size_t)idx : s.size() + (size_t)(long long)idx;
    if (b > s.size()) throw OutOfRange();
    return s.substr(b);
}
string vsub(const string &s, int begin, int len) {  // vc_substr(str, begin, len): include/util.h:44-57
    if (begin < 0) begin = (int)(s.size() + (size_t)(long long)begin);
    if (len > 0) {
        if ((size_t)(long long)begin > s.size()) throw OutOfRange();
        return s.substr((size_t)(long long)begin, (size_t)len);
    }
    if (len == 0) return string();
    len = (int)(s.size() + (size_t)(long long)len - (size_t)(long long)begin);
    if (len < 0) return string();
    if ((size_t)(long long)begin > s.size()) throw OutOfRange();
    return s.substr((size_t)(long long)begin, (size_t)len);
}
char char_at(const string &s, int i) {  // charAt: include/util.h:171-179
    if (i < 0) {
        int k = (int)s.size() + i;
        return k < 0 ? (char)-1 : s[k];
    }
    return s[i];
}
string strip_hash_caret(const string &s) {  // regex_replace(s, "#|\\^", "")
    string o;
    for (char c : s)
        if (c != '#' && c != '^') o += c;
    return o;
}

void adj_cnt3(Stat &to, Stat &v, Stat *ref) {  // adjCnt(varToAdd, variant, referenceVar): include/VariationUtils.h:291-317
    adj_cnt(to, v);
    if (!ref) return;
    ref->cnt -= v.cnt;
    ref->hi -= v.hi;
    ref->lo -= v.lo;
    ref->pmean -= v.pmean;
    ref->qmean -= v.qmean;
    ref->mq -= v.mq;
    ref->nm -= v.nm;
    ref->rev -= v.rev;
    ref->fwd -= v.fwd;
    // correctCnt: include/VariationUtils.h:263-280
    if (ref->cnt < 0) ref->cnt = 0;
    if (ref->hi < 0) ref->hi = 0;
    if (ref->lo < 0) ref->lo = 0;
    if (ref->pmean < 0) ref->pmean = 0;
    if (ref->qmean < 0) ref->qmean = 0;
    if (ref->mq < 0) ref->mq = 0;
    if (ref->rev < 0) ref->rev = 0;
    if (ref->fwd < 0) ref->fwd = 0;
}
void correct_cnt(Stat &r) {
    if (r.cnt < 0) r.cnt = 0;
    if (r.hi < 0) r.hi = 0;
    if (r.lo < 0) r.lo = 0;
    if (r.pmean < 0) r.pmean = 0;
    if (r.qmean < 0) r.qmean = 0;
    if (r.mq < 0) r.mq = 0;
    if (r.rev < 0) r.rev = 0;
    if (r.fwd < 0) r.fwd = 0;
}

struct Mism { string seq; int pos; int end; };
struct MmResult { vector<Mism> mm; vector<int> scp; int nm = 0, misp = 0; string misnt; };

struct Realigner {
    Maps &M;
    Ref &R;
    const rvo_params &P;
    const rvo_reads *rd;
    int rs, re, chr_len;
    int max_rl;

    static Stat *maybe(map<int, KeyMap> &h, int p, char base) {  // getVariationMaybe: include/VariationUtils.h:218-239
        if (base == 0) return nullptr;
        auto it = h.find(p);
        if (it == h.end()) return nullptr;
        auto j = it->second.find(string(1, base));
        return j == it->second.end() ? nullptr : &j->second;
    }
    bool has_key(int p, const string &k) {
        auto it = M.nonins.find(p);
        return it != M.nonins.end() && it->second.count(k);
    }

    // findMM5 (:1857-1916)
    MmResult find_mm5(Ref &RR, int position, const string &wupseq) {
        string seq = strip_hash_caret(wupseq);
        MmResult r;
        int n = 0, mcnt = 0;
        string str;
        while (RR.has_ne(char_at(seq, -1 - n), position - n) && mcnt < 3) {
            str.insert(0, 1, char_at(seq, -1 - n));
            r.mm.push_back({str, position - n, 5});
            n++;
            mcnt++;
        }
        r.scp.push_back(position + 1);
        if (str.size() == 1) {
            while (RR.has_eq(char_at(seq, -1 - n), position - n)) {
                n++;
                if (n != 0) r.nm++;
            }
            if (r.nm > 1) {
                // the second scan's condition (-1 - n - 1 - n2 >= 0) never holds
                r.scp.push_back(position - n);
                auto it = M.sc5.find(position - n);
                if (it != M.sc5.end()) it->second.used = true;
            }
        }
        return r;
    }
    // findMM3 (:1919-1984)
    MmResult find_mm3(Ref &RR, int p, const string &sanpseq) {
        string seq = strip_hash_caret(sanpseq);
        MmResult r;
        int n = 0, mcnt = 0, len = (int)seq.size();
        string str;
        while (n < len && RR.has(p + n) && RR.at(p + n) == seq[n]) n++;
        r.scp.push_back(p + n);
        const int Tbp = p + n;
        while (mcnt <= 3 && n < len && RR.idx(p + n) != seq[n]) {
            str += seq[n];
            r.mm.push_back({str, Tbp, 3});
            n++;
            mcnt++;
        }
        if (str.size() == 1) {
            while (n < len && RR.has_eq(seq[n], p + n)) {
                n++;
                if (n != 0) r.nm++;
            }
            if (r.nm > 1) {
                int n2 = 0;
                while (n + n2 + 1 < len && RR.has_eq(seq[n + n2 + 1], p + n + 1 + n2)) n2++;
                if (n2 > 2 && n + n2 + 1 < len) {
                    r.scp.push_back(p + n + n2);
                    r.misp = p + n;
                    r.misnt = string(1, seq[n]);
                    auto it = M.sc3.find(p + n + n2);
                    if (it != M.sc3.end()) it->second.used = true;
                    r.nm += n2;
                } else {
                    r.scp.push_back(p + n);
                    auto it = M.sc3.find(p + n);
                    if (it != M.sc3.end()) it->second.used = true;
                }
            }
        }
        return r;
    }
    // ismatch (:1507-1546), MM = 3
    static bool ismatch(const string &seq1, const string &seq2_in, int dir) {
        string seq2 = strip_hash_caret(seq2_in);
        int mm = 0;
        for (int n = 0; n < (int)seq1.size() && n < (int)seq2.size(); n++)
            if (seq1[n] != vsub(seq2, dir * n - (dir == -1 ? 1 : 0), 1)[0]) mm++;
        return mm <= 3 && mm / (double)seq1.size() < 0.15;
    }
    // adjRefCnt (:1753-1787)
    static void adj_ref_cnt(Stat &tv, Stat *ref, int len) {
        if (!ref) return;
        double f = tv.pmean != 0 ? (tv.pmean / (double)tv.cnt - len + 1) / (tv.pmean / (double)tv.cnt) : 0;
        if (f < 0) return;
        if (f > 1) f = 1;
        ref->cnt -= (int)(f * tv.cnt);
        ref->hi -= (int)(f * tv.hi);
        ref->lo -= (int)(f * tv.lo);
        ref->pmean -= f * tv.pmean;
        ref->qmean -= f * tv.qmean;
        ref->mq -= f * tv.mq;
        ref->nm -= f * tv.nm;
        ref->rev -= (int)(f * tv.rev);
        ref->fwd -= (int)(f * tv.fwd);
        correct_cnt(*ref);
    }
    // adjRefFactor (:1794-1822)
    static void adj_ref_factor(Stat *ref, double f) {
        if (!ref) return;
        if (f > 1) f = 1;
        if (f < -1) return;
        int old = ref->cnt;
        ref->cnt -= (int)(f * ref->cnt);
        ref->hi -= (int)(f * ref->hi);
        ref->lo -= (int)(f * ref->lo);
        double fc = old != 0 ? std::abs(ref->cnt - old) / (double)old : 1;
        ref->pmean -= ref->pmean * f * fc;
        ref->qmean -= ref->qmean * f * fc;
        ref->mq -= ref->mq * f * fc;
        ref->nm -= f * ref->nm;
        ref->fwd -= (int)(f * ref->fwd);
        ref->rev -= (int)(f * ref->rev);
        correct_cnt(*ref);
    }
    // noPassingReads (:1447-1505): raw records over chr:start-end, no filters
    bool no_passing_reads(int start, int end) {
        int cnt = 0;
        const uint32_t dlenqr = ((uint32_t)(end - start) << 4) | 2u;
        int64_t lo = 0, hi = rd->n;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (rd->pos[mid] < start - 1 - 4096) lo = mid + 1; else hi = mid;
        }
        for (int64_t i = lo; i < rd->n && rd->pos[i] < end; i++) {
            const uint32_t *c = rd->cigar + rd->cig_off[i];
            int span = 0, aligned = 0;
            bool has_d = false;
            for (int k = 0; k < rd->n_cigar[i]; k++) {
                int o = c[k] & 15;
                if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) span += c[k] >> 4;
                if (o == 0 || o == 2) aligned += c[k] >> 4;
                if (c[k] == dlenqr) has_d = true;
            }
            int endpos = ((rd->flag[i] & 4) || span == 0) ? rd->pos[i] + 1 : rd->pos[i] + span;
            if (endpos <= start - 1) continue;
            if (has_d) continue;
            int rs0 = rd->pos[i] + 1, reE = rs0 + aligned;
            if (reE > end + 2 && rs0 < start - 2) cnt++;
        }
        return cnt <= 0;
    }

    struct Cand { int pos; string key; int cnt; };
    static vector<Cand> sorted(const map<int, map<string, int>> &ch) {  // fillAndSortTmp + CMP_tmp (:44-58, :1362-1386)
        vector<Cand> t;
        for (auto &pe : ch)
            for (auto &ke : pe.second) t.push_back({pe.first, ke.first, ke.second});
        std::sort(t.begin(), t.end(), [](const Cand &a, const Cand &b) {
            if (a.cnt != b.cnt) return a.cnt > b.cnt;
            if (a.pos != b.pos) return a.pos < b.pos;
            return a.key.compare(b.key) > 0;
        });
        return t;
    }
    static bool rx(const string &s, const char *pat, std::smatch &m) {
        return std::regex_search(s, m, std::regex(pat));
    }

    // realigndel (:489-775)
    void realigndel(bool with_bams, map<int, map<string, int>> dcnt_map) {
        vector<Cand> tmp = sorted(dcnt_map);
        for (const Cand &tpl : tmp) {
            try {
                const int p = tpl.pos;
                const string &vn = tpl.key;
                const int dcnt = tpl.cnt;
                Stat &vref = M.nonins[p][vn];
                int dellen = 0;
                std::smatch m;
                if (rx(vn, "^-(\\d+).*", m)) dellen = atoi(m.str(1).c_str());
                if (rx(vn, "\\^(\\d+)$", m)) dellen += atoi(m.str(1).c_str());
                string extrains, extra, inv5, inv3;
                if (rx(vn, "^-\\d+\\^([ATGNC]+)<...\\d+>([ATGNC]+)$", m)) {
                    inv5 = m.str(1);
                    inv3 = m.str(2);
                } else if (rx(vn, "^-\\d+(.*)", m)) {
                    for (char c : m.str(1))
                        if (c != '^' && c != '&' && c != '#') extra += c;
                    if (rx(vn, "\\^([ATGNC]+)", m)) extrains = m.str(1);
                }
                const int wustart = p - 200 > 1 ? p - 200 : 1;
                string wupseq = join_ref(R, wustart, p - 1) + extra;
                if (!inv3.empty()) wupseq = inv3;
                const int sanend = p + 200 > chr_len ? chr_len : p + 200;
                const int off = dellen + (int)extra.size() - (int)extrains.size();
                string sanpseq = extra + join_ref(R, p + off, sanend);
                if (!inv5.empty()) sanpseq = inv5;
                MmResult r3 = find_mm3(R, p, sanpseq);
                MmResult r5 = find_mm5(R, p + off - 1, wupseq);
                vector<Mism> mmm = r3.mm;
                mmm.insert(mmm.end(), r5.mm.begin(), r5.mm.end());
                for (Mism &mi : mmm) {
                    string mm = mi.seq;
                    if (mm.size() > 1) mm.insert(1, 1, '&');
                    const int mp = mi.pos, me = mi.end;
                    if (!has_key(mp, mm)) continue;
                    Stat &tv = M.nonins[mp][mm];
                    if (tv.cnt == 0) continue;
                    if (tv.qmean / tv.cnt < P.goodq) continue;
                    if (tv.pmean / tv.cnt > (me == 3 ? r3.nm + 4 : r5.nm + 4)) continue;
                    if (tv.cnt >= dcnt + dellen || tv.cnt / dcnt >= 8) continue;
                    if (mp > p && me == 5) {
                        double f = tv.pmean != 0 ? (mp - p) / (tv.pmean / (double)tv.cnt) : 1;
                        if (f > 1) f = 1;
                        M.cov[p] += (int)(tv.cnt * f);
                        adj_ref_cnt(tv, maybe(M.nonins, p, R.idx(p)), dellen);
                    }
                    if (mp > p && me == 3 && M.nonins.count(p) && M.nonins[p].count(string(1, R.idx(p)))) {
                        Stat *lref = &M.nonins[p][string(1, R.idx(p))];
                        adj_cnt3(vref, tv, lref);
                    } else {
                        adj_cnt(vref, tv);
                    }
                    M.nonins[mp].erase(mm);
                    if (M.nonins[mp].empty()) M.nonins.erase(mp);
                }
                if (r3.misp != 0 && r3.mm.size() == 1 && has_key(r3.misp, r3.misnt) &&
                    M.nonins[r3.misp][r3.misnt].cnt < dcnt)
                    M.nonins[r3.misp].erase(r3.misnt);
                if (r5.misp != 0 && r5.mm.size() == 1 && has_key(r5.misp, r5.misnt) &&
                    M.nonins[r5.misp][r5.misnt].cnt < dcnt)
                    M.nonins[r5.misp].erase(r5.misnt);
                for (int sc5pp : r5.scp) {
                    auto it = M.sc5.find(sc5pp);
                    if (it == M.sc5.end() || it->second.used) continue;
                    Clip &tv = it->second;
                    string seq = consensus(tv);
                    if (dcnt <= 2 && tv.cnt / dcnt > 5) continue;
                    if (seq != " " && ismatch(seq, wupseq, -1)) {
                        if (sc5pp > p) M.cov[p] += tv.cnt;
                        adj_cnt(vref, tv);
                        tv.used = true;
                    }
                }
                for (int sc3pp : r3.scp) {
                    auto it = M.sc3.find(sc3pp);
                    if (it == M.sc3.end() || it->second.used) continue;
                    Clip &tv = it->second;
                    string seq = consensus(tv);
                    if (dcnt <= 2 && tv.cnt / dcnt > 5) continue;
                    if (seq != " " && ismatch(seq, vsub(sanpseq, sc3pp - p), 1)) {
                        if (sc3pp <= p) M.cov[p] += tv.cnt;
                        Stat *lref = sc3pp <= p ? nullptr : maybe(M.nonins, p, R.idx(p));
                        adj_cnt3(vref, tv, lref);
                        tv.used = true;
                    }
                }
                const int pe = p + off;
                Stat *h = maybe(M.nonins, p, R.idx(p));
                if (with_bams && pe - p >= 5 && pe - p < max_rl - 10 && h && h->cnt != 0 &&
                    vref.cnt > 2 * h->cnt * (1 - (pe - p) / (double)max_rl) && no_passing_reads(p, pe))
                    adj_cnt3(vref, *h, h);
            } catch (const RefFail &) {
            } catch (const OutOfRange &) {
            }
        }
        for (int i = (int)tmp.size() - 1; i > 0; i--) {
            const int p = tmp[i].pos;
            const string &vn = tmp[i].key;
            if (!has_key(p, vn)) continue;
            Stat &vref = M.nonins[p][vn];
            std::smatch m;
            if (rx(vn, "(-\\d+)&[ATGC]+$", m)) {
                string tn = m.str(1);
                if (M.nonins[p].count(tn)) {
                    Stat &tref = M.nonins[p][tn];
                    if (vref.cnt < tref.cnt) {
                        adj_cnt(tref, vref);
                        M.nonins[p].erase(vn);
                    }
                }
            }
        }
    }

    // realignins (:785-1114)
    void realignins(map<int, map<string, int>> &icnt_map) {
        vector<Cand> tmp = sorted(icnt_map);
        for (const Cand &tpl : tmp) {
            try {
                const int position = tpl.pos;
                const string &vn = tpl.key;
                const int icnt = tpl.cnt;
                std::smatch m;
                string insert1;
                if (rx(vn, "^\\+([ATGC]+).*", m)) insert1 = m.str(1);
                else continue;
                string ins3;
                int inslen = (int)insert1.size();
                if (rx(vn, "<dup(\\d+)>([ATGC]+)$", m)) {
                    ins3 = m.str(2);
                    inslen += atoi(m.str(1).c_str()) + (int)ins3.size();
                }
                string extra, compm;
                if (rx(vn, ".*&([ATGC]+).*", m)) extra = m.str(1);
                if (rx(vn, "#([ATGC]+).*", m)) compm = m.str(1);
                int newdel = 0;
                if (rx(vn, "\\^(\\d+)$", m)) newdel = atoi(m.str(1).c_str());
                string tn = vn;
                if (!tn.empty() && tn[0] == '+') tn.erase(0, 1);
                replace_first(tn, "&", "");
                replace_first(tn, "#", "");
                tn = std::regex_replace(tn, std::regex("\\^\\d+$"), "", std::regex_constants::format_first_only);
                tn = std::regex_replace(tn, std::regex("\\^"), "", std::regex_constants::format_first_only);
                const int wustart = position - 150 > 1 ? position - 150 : 1;
                string wupseq = join_ref(R, wustart, position) + tn;
                int sanend = position + (int)vn.size() + 100;
                if (chr_len < sanend) sanend = chr_len;
                string sanpseq;
                MmResult r3;
                if (!ins3.empty()) {
                    int p3 = position + inslen - (int)ins3.size() + 50;
                    if ((int)ins3.size() > 50) sanpseq = vsub(ins3, 50 - (int)ins3.size());
                    sanpseq += join_ref(R, position + 1, position + 101);
                    r3 = find_mm3(R, p3 + 1, sanpseq);
                } else {
                    sanpseq = tn + join_ref(R, position + (int)extra.size() + 1 + (int)compm.size() + newdel, sanend);
                    r3 = find_mm3(R, position + 1, sanpseq);
                }
                MmResult r5 = find_mm5(R, position + (int)extra.size() + (int)compm.size() + newdel, wupseq);
                vector<Mism> mmm = r3.mm;
                mmm.insert(mmm.end(), r5.mm.begin(), r5.mm.end());
                Stat &vref = M.ins[position][vn];
                for (Mism &mi : mmm) {
                    string mb = mi.seq;
                    if (mb.size() > 1) mb = string(1, mb[0]) + "&" + mb.substr(1);
                    const int mp = mi.pos, me = mi.end;
                    if (!has_key(mp, mb)) continue;
                    Stat &var = M.nonins[mp][mb];
                    if (var.cnt == 0) continue;
                    if (var.qmean / var.cnt < P.goodq) continue;
                    if (var.pmean / var.cnt > (me == 3 ? r3.nm + 4 : r5.nm + 4)) continue;
                    if (var.cnt >= icnt + (int)insert1.size() || var.cnt / icnt >= 8) continue;
                    if (mp > position && me == 5) M.cov[position] += var.cnt;
                    if (mp > position && me == 3 && M.nonins.count(position) && R.has(position) &&
                        M.nonins[position].count(string(1, R.idx(position)))) {
                        Stat *lref = &M.nonins[position][string(1, R.idx(position))];
                        adj_cnt3(vref, var, lref);
                    } else {
                        adj_cnt(vref, var);
                    }
                    M.nonins[mp].erase(mb);
                    if (M.nonins[mp].empty()) M.nonins.erase(mp);
                }
                if (r3.misp != 0 && r3.mm.size() == 1 && has_key(r3.misp, r3.misnt) &&
                    M.nonins[r3.misp][r3.misnt].cnt < icnt)
                    M.nonins[r3.misp].erase(r3.misnt);
                if (r5.misp != 0 && r5.mm.size() == 1 && has_key(r5.misp, r5.misnt) &&
                    M.nonins[r5.misp][r5.misnt].cnt < icnt)
                    M.nonins[r5.misp].erase(r5.misnt);
                for (int sc5pp : r5.scp) {
                    auto it = M.sc5.find(sc5pp);
                    if (it == M.sc5.end()) continue;
                    Clip &tv = it->second;
                    if (tv.used) continue;
                    string seq = consensus(tv);
                    if (seq != " " && ismatch(seq, wupseq, -1)) {
                        if (sc5pp > position) M.cov[position] += tv.cnt;
                        adj_cnt(vref, tv);
                        tv.used = true;
                    }
                }
                for (int sc3pp : r3.scp) {
                    auto it = M.sc3.find(sc3pp);
                    if (it == M.sc3.end()) continue;
                    Clip &tv = it->second;
                    if (tv.used) continue;
                    string seq = consensus(tv);
                    string mseq = !ins3.empty() ? sanpseq : vsub(sanpseq, sc3pp - position - 1);
                    if (seq != " " && ismatch(seq, mseq, 1)) {
                        if (sc3pp <= position || (int)insert1.size() > tv.pmean / tv.cnt) M.cov[position] += tv.cnt;
                        Stat *lref = nullptr;
                        if (sc3pp > position && M.nonins.count(position) && R.has(position) &&
                            M.nonins[position].count(string(1, R.idx(position))))
                            lref = &M.nonins[position][string(1, R.idx(position))];
                        if ((int)insert1.size() > tv.pmean / tv.cnt) lref = nullptr;
                        adj_cnt3(vref, tv, lref);
                        tv.used = true;
                        if (insert1.size() + 1 == vn.size() && (int)insert1.size() > max_rl &&
                            sc3pp >= position + 1 + (int)insert1.size()) {
                            int flag = 0;
                            int offset = (sc3pp - position - 1) % (int)insert1.size();
                            string tvn = vn;
                            for (int si = 0; si < (int)seq.size() && si + offset < (int)insert1.size(); si++) {
                                if (vsub(seq, si, 1) != vsub(insert1, si + offset, 1)) {
                                    flag++;
                                    int shift = si + offset + 1;
                                    tvn = tvn.substr(0, shift) + vsub(seq, si, 1) + tvn.substr(shift + 1);
                                }
                            }
                            if (flag > 0) {
                                Stat moved = M.ins[position][vn];
                                M.ins[position][tvn] = moved;
                                M.ins[position].erase(vn);
                            }
                        }
                    }
                }
                if (!r3.scp.empty() && !r5.scp.empty()) {
                    int first3 = r3.scp[0], first5 = r5.scp[0];
                    if (first3 > first5 + 3 && first3 - first5 < max_rl * 0.75) {
                        if (R.has(position) && M.nonins.count(position) &&
                            M.nonins[position].count(string(1, R.idx(position))))
                            adj_ref_factor(&M.nonins[position].at(string(1, R.idx(position))),
                                           (first3 - first5 - 1) / (double)max_rl);
                        adj_ref_factor(&vref, -(first3 - first5 - 1) / (double)max_rl);
                    }
                }
            } catch (const RefFail &) {
            } catch (const OutOfRange &) {
            }
        }
        for (int i = (int)tmp.size() - 1; i > 0; i--) {
            const int p = tmp[i].pos;
            const string &vn = tmp[i].key;
            auto it = M.ins.find(p);
            if (it == M.ins.end() || !it->second.count(vn)) continue;
            Stat &vref = it->second.at(vn);
            std::smatch m;
            if (rx(vn, "(\\+[ATGC]+)&[ATGC]+$", m)) {
                string tn = m.str(1);
                if (it->second.count(tn)) {
                    Stat &tref = it->second.at(tn);
                    if (vref.cnt < tref.cnt) {
                        adj_cnt3(tref, vref, maybe(M.nonins, p, R.idx(p)));
                        it->second.erase(vn);
                    }
                }
            }
        }
    }

    // find35match (:1396-1428)
    static void find35(const string &s5, const string &s3, int &b5, int &b3, int &score) {
        b5 = b3 = score = 0;
        for (int i = 0; i < (int)s5.size() - 8; i++) {
            for (int j = 1; j < (int)s3.size() - 8; j++) {
                int nm = 0, n = 0;
                while (n + j <= (int)s3.size() && i + n <= (int)s5.size()) {
                    if (vsub(s3, -j - n, 1) != vsub(s5, i + n, 1)) nm++;
                    if (nm > 2) break;
                    n++;
                }
                if (n - nm > score && n - nm > 8 && nm / (double)n < 0.1 &&
                    (n + j >= (int)s3.size() || i + n >= (int)s5.size())) {
                    b5 = i;
                    b3 = j;
                    score = n - nm;
                    return;
                }
            }
        }
    }

    // realignlgins30 (:1119-1350); its reference map is a copy (operator[]
    // entries stay local), the nested realignins/realigndel use the shared one
    void realignlgins30() {
        Ref RL = R;
        struct T { int pos; Clip *c; int cnt; };
        vector<T> t5, t3;
        for (auto &e : M.sc5)
            if (!(e.first < rs - 5000 || e.first > re + 5000)) t5.push_back({e.first, &e.second, e.second.cnt});
        for (auto &e : M.sc3)
            if (!(e.first < rs - 5000 || e.first > re + 5000)) t3.push_back({e.first, &e.second, e.second.cnt});
        auto cmp3 = [](const T &a, const T &b) { return a.cnt != b.cnt ? a.cnt > b.cnt : a.pos < b.pos; };
        std::sort(t5.begin(), t5.end(), cmp3);
        std::sort(t3.begin(), t3.end(), cmp3);
        for (T &a : t5) {
            const int p5 = a.pos;
            Clip &sc5v = *a.c;
            const int cnt5 = a.cnt;
            if (sc5v.used) continue;
            string seq5 = consensus(sc5v);
            if (seq5.size() <= 10) continue;
            for (T &b : t3) {
                try {
                    const int p3 = b.pos;
                    Clip &sc3v = *b.c;
                    const int cnt3 = b.cnt;
                    if (sc5v.used) break;
                    if (sc3v.used) continue;
                    if (p5 - p3 > max_rl * 2.5) continue;
                    if (p3 - p5 > max_rl - 10) continue;
                    string seq3 = consensus(sc3v);
                    if (seq3.size() <= 10) continue;
                    if (!(cnt5 / (double)cnt3 >= 0.08 && cnt5 / (double)cnt3 <= 12)) continue;
                    int bp5, bp3, score;
                    find35(seq5, seq3, bp5, bp3, score);
                    if (score == 0) continue;
                    const int sm = score / 2;
                    string ins = bp3 + sm > 1 ? vsub(seq3, 0, -(bp3 + sm) + 1) : seq3;
                    if (bp5 + sm > 0) {
                        string tt = seq5.substr(0, bp5 + sm);
                        std::reverse(tt.begin(), tt.end());
                        ins += tt;
                    }
                    if (low_complexity(ins)) continue;
                    int bi = 0;
                    Stat *vref;
                    const int il = (int)ins.size();
                    if ((int)seq3.size() > il &&
                        !ismatch(seq3.substr(il), join_ref(RL, p5, p5 + (int)seq3.size() - il + 2), 1))
                        continue;
                    if ((int)seq5.size() > il &&
                        !ismatch(seq5.substr(il), join_ref(RL, p3 - ((int)seq5.size() - il) - 2, p3 - 1), -1))
                        continue;
                    if (p5 > p3) {
                        string tmp = join_ref(RL, p3, p5 - 1);
                        if (tmp.size() > ins.size()) {
                            ins = std::to_string(p3 - p5) + "^" + ins;
                            bi = p3;
                            vref = &M.nonins[p3][ins];
                        } else if (tmp.size() < ins.size()) {
                            ins = vsub(ins, 0, (int)ins.size() - (int)tmp.size()) + "&" + vsub(ins, p3 - p5);
                            ins = "+" + ins;
                            bi = p3 - 1;
                            vref = &M.ins[bi][ins];
                        } else {
                            ins = "-" + std::to_string(ins.size()) + "^" + ins;
                            bi = p3;
                            vref = &M.nonins[p3][ins];
                        }
                    } else {
                        string tmp;
                        if ((int)ins.size() <= p3 - p5) {
                            int rpt = 2, tnr = 3;
                            const int tot = p3 - p5 + (int)ins.size();
                            while ((tot / (double)tnr) / (double)ins.size() > 1) {
                                if (tot % tnr == 0) rpt++;
                                tnr++;
                            }
                            const double to = p5 + tot / (double)rpt - ins.size();
                            for (int i = p5; i < to; i++) {  // joinRef_double: include/VariationUtils.h:343-349
                                if (!RL.has(i)) throw RefFail();
                                tmp += RL.at(i);
                            }
                            ins = "+" + tmp + ins;
                        } else {
                            tmp += join_ref(RL, p5, p3 - 1);
                            if ((ins.size() - tmp.size()) % 2 == 0) {
                                int tex = (int)(ins.size() - tmp.size()) / 2;
                                ins = (tmp + vsub(ins, 0, tex)) == vsub(ins, tex) ? "+" + vsub(ins, tex) : "+" + tmp + ins;
                            } else {
                                ins = "+" + tmp + ins;
                            }
                        }
                        bi = p5 - 1;
                        vref = &M.ins[bi][ins];
                    }
                    sc3v.used = true;
                    sc5v.used = true;
                    vref->pstd = true;
                    vref->qstd = true;
                    M.cov[bi] += sc5v.cnt;
                    if (ins[0] == '+') {
                        Stat *mvref = maybe(M.nonins, bi, RL.idx(bi));
                        adj_cnt3(*vref, sc3v, mvref);
                        adj_cnt(*vref, sc5v);
                        if (p3 - p5 >= 5 && p3 - p5 < max_rl - 10 && mvref && mvref->cnt != 0 &&
                            vref->cnt > 2 * mvref->cnt && no_passing_reads(p5, p3))
                            adj_cnt3(*vref, *mvref, mvref);
                        map<int, map<string, int>> tins;
                        tins[bi][ins] = vref->cnt;
                        realignins(tins);
                    } else if (ins[0] == '-') {
                        adj_cnt3(*vref, sc3v, maybe(M.nonins, bi, RL.idx(bi)));
                        adj_cnt(*vref, sc5v);
                        map<int, map<string, int>> tdel;
                        tdel[bi][ins] = vref->cnt;
                        realigndel(false, tdel);
                    } else {
                        adj_cnt(*vref, sc3v);
                        adj_cnt(*vref, sc5v);
                    }
                    break;
                } catch (const RefFail &) {
                } catch (const OutOfRange &) {
                }
            }
        }
    }

    // realignIndels (:467-482)
    void run() {
        realigndel(true, M.delcnt);
        realignins(M.inscnt);
        realignlgins30();
    }
};

// VariationRealigner::process (src/VariationRealigner.cpp:135-161): adjustMNP
// always, the indel passes with -k 1
void realign(Maps &M, Ref &R, const rvo_params &P, const rvo_reads *rd, int rs, int re, int chr_len) {
    adjust_mnp(M, R);
    if (P.local_realign) {
        Realigner rl{M, R, P, rd, rs, re, chr_len, M.max_read_len};
        rl.run();
    }
}

// ---------------------------------------------------------------------------
// scoring: ToVarsBuilder (src/ToVarsBuilder.cpp) and Variant (include/Variant.h)
// ---------------------------------------------------------------------------
struct Var {
    string desc;
    int pc = 0, fwd = 0, rev = 0;
    string sbf = "0";
    double freq = 0, pmean = 0;
    bool pstd = false;
    double qual = 0;
    bool qstd = false;
    double mq = 0, qratio = 0, hifreq = 0, extrafreq = 0;
    int shift3 = 0;
    double msi = 0;
    int msint = 0;
    double nm = 0;
    int hicnt = 0, hicov = 0;
    string leftseq, rightseq;
    int startp = 0, endp = 0, rfc = 0, rrc = 0, tpc = 0;
    double duprate = 0;
    string genotype, varallele, refallele, vartype;
    bool filled = false;  // set when collectReferenceVariants completed for it
};

struct PosVars {
    int ref_idx = -1;  // index into all
    vector<int> vars;
    vector<Var> all;
};

int strand_bias(int f, int r, const rvo_params &P) {  // include/VariationUtils.h:511-521
    if (f + r <= 12) return f * r > 0 ? 2 : 0;
    return (f / (double)(f + r) >= P.bias && r / (double)(f + r) >= P.bias && f >= P.min_bias_reads &&
            r >= P.min_bias_reads) ? 2 : 1;
}


struct Msi { double msi; int shift3; string msint; };

// findMSI with curmsi_from_end: src/ToVarsBuilder.cpp:614-678
Msi find_msi(const string &t1, const string &t2, const string &left) {
    int nmsi = 1, shift3 = 0;
    string maxmsi;
    double msicnt = 0;
    while (nmsi <= (int)t1.size() && nmsi <= 6) {
        string msint = t1.substr(t1.size() - nmsi, nmsi);
        string mb = left + t1;
        double cur = 1.0;
        for (int i = (int)mb.size() - nmsi; i > 0; i -= nmsi) {
            if (i > nmsi && mb.compare(i - nmsi, nmsi, msint) == 0) cur += 1;
            else break;
        }
        for (int i = 0; i < (int)t2.size(); i += nmsi) {
            if (i + nmsi < (int)t2.size() && t2.compare(i, nmsi, msint) == 0) cur += 1.0;
            else break;
        }
        if (cur > msicnt) { maxmsi = msint; msicnt = cur; }
        nmsi++;
    }
    string ts = t1 + t2;
    while (shift3 < (int)t2.size() && ts[shift3] == t2[shift3]) shift3++;
    return {msicnt, shift3, maxmsi};
}


bool starts_with(const string &s, const char *p) { return s.compare(0, strlen(p), p) == 0; }

struct Scorer {
    const rvo_params &P;
    Maps &M;
    Ref &R;
    int chr_len;
    int rs, re;
    bool somatic;  // a second BAM is configured (conf->bam.hasBam2())
    map<int, PosVars> aligned;

    Scorer(const rvo_params &p, Maps &m, Ref &r, int cl, int s, int e, bool som = false)
        : P(p), M(m), R(r), chr_len(cl), rs(s), re(e), somatic(som) {}

    Var make_var(const string &k, const Stat &c, int ttcov, int hicov) {
        Var v;
        v.desc = k;
        v.pc = c.cnt;
        v.fwd = c.fwd;
        v.rev = c.rev;
        v.sbf = std::to_string(strand_bias(c.fwd, c.rev, P));
        v.freq = c.cnt / (double)ttcov;
        v.pmean = c.pmean / (double)c.cnt;
        v.pstd = c.pstd;
        v.qual = c.qmean / c.cnt;
        v.qstd = c.qstd;
        v.mq = c.mq / (double)c.cnt;
        v.qratio = c.hi / (c.lo != 0 ? (double)c.lo : 0.5);
        v.hifreq = hicov > 0 ? c.hi / (double)hicov : 0;
        v.extrafreq = c.extracnt != 0 ? c.extracnt / (double)ttcov : 0;
        v.nm = c.nm / (double)c.cnt;
        v.hicnt = c.hi;
        v.hicov = hicov;
        return v;
    }

    // ToVarsBuilder::process: src/ToVarsBuilder.cpp:97-205 (positions ascending)
    void run() {
        for (auto &pe : M.nonins) {
            int position = pe.first;
            KeyMap &vm = pe.second;
            bool has_ins = M.ins.count(position) > 0;
            if (vm.empty() && !has_ins) continue;
            auto cit = M.cov.find(position);
            if (cit == M.cov.end() || cit->second == 0) continue;
            // isTheSameVariationOnRef: src/ToVarsBuilder.cpp:213-233
            if (vm.size() == 1 && !has_ins && R.has(position) && vm.count(string(1, R.at(position))) && !P.do_pileup &&
                !somatic)
                continue;
            int tpc = cit->second;
            int hicov = 0;  // calcHicov: src/ToVarsBuilder.cpp:570-587
            for (auto &e : vm) hicov += e.second.hi;
            if (has_ins)
                for (auto &e : M.ins.at(position)) hicov += e.second.hi;
            vector<Var> var;
            // createVariant: src/ToVarsBuilder.cpp:466-536
            for (auto &e : vm) {
                const Stat &c = e.second;
                if (c.cnt == 0) continue;
                int ttcov = tpc;
                if (c.cnt > tpc && c.extracnt > 0 && c.cnt - tpc < c.extracnt) ttcov = c.cnt;
                var.push_back(make_var(e.first, c, ttcov, hicov));
            }
            // createInsertion: src/ToVarsBuilder.cpp:358-452
            if (has_ins) {
                int hic = hicov;
                for (auto &e : M.ins.at(position)) {
                    const Stat &c = e.second;
                    int ttcov = tpc;
                    if (c.cnt > tpc && c.extracnt != 0 && c.cnt - tpc < c.extracnt) ttcov = c.cnt;
                    if (ttcov < c.cnt) {
                        ttcov = c.cnt;
                        auto nc = M.cov.find(position + 1);
                        if (nc != M.cov.end() && R.has(position + 1) && ttcov < nc->second - c.cnt) {
                            ttcov = nc->second;
                            auto np = M.nonins.find(position + 1);
                            if (np != M.nonins.end()) {
                                auto nk = np->second.find(string(1, R.at(position + 1)));
                                if (nk != np->second.end()) {
                                    nk->second.fwd -= c.fwd;
                                    nk->second.rev -= c.rev;
                                }
                            }
                        }
                        tpc = ttcov;
                    }
                    if (hic < c.hi) hic = c.hi;
                    var.push_back(make_var(e.first, c, ttcov, hic));
                }
            }
            // CMP_VARI: src/ToVarsBuilder.cpp:20-26
            std::sort(var.begin(), var.end(), [](const Var &a, const Var &b) {
                double r = a.qual * a.pc - b.qual * b.pc;
                if (r < 0.00001 && r > -0.00001) return a.desc.compare(b.desc) < 0;
                return r > 0;
            });
            // collectVarsAtPosition: src/ToVarsBuilder.cpp:327-346
            PosVars pv;
            double maxfreq = 0;
            for (Var &v : var) {
                pv.all.push_back(v);
                int idx = (int)pv.all.size() - 1;
                if (R.has(position) && v.desc == string(1, R.at(position))) pv.ref_idx = idx;
                else {
                    pv.vars.push_back(idx);
                    if (v.freq > maxfreq) maxfreq = v.freq;
                }
            }
            if (!P.do_pileup && maxfreq <= P.freq && !somatic) continue;
            // only zero-count keys (and no insertion): the reference dereferences
            // a null reference variant in collectReferenceVariants
            // (src/ToVarsBuilder.cpp:737-743); such positions are left out
            if (pv.all.empty()) continue;
            try {
                collect_reference(position, tpc, pv);
            } catch (const RefFail &) {
            }
            aligned[position] = pv;
        }
    }

    // proceedVrefIsDeletion / proceedVrefIsInsertion: src/ToVarsBuilder.cpp:242-317
    Msi msi_deletion(int position, int dellen) {
        string leftseq = join_ref(R, position - 70 > 1 ? position - 70 : 1, position - 1);
        string tseq = join_ref(R, position, position + dellen + 70 > chr_len ? chr_len : position + dellen + 70);
        string a = tseq.substr(0, std::min<size_t>(dellen, tseq.size()));
        string b = (size_t)dellen <= tseq.size() ? tseq.substr(dellen) : string();
        Msi m = find_msi(a, b, leftseq);
        Msi t = find_msi(leftseq, b, "");
        if (m.msi < t.msi) { m.msi = t.msi; m.msint = t.msint; }
        if (m.msi <= m.shift3 / (double)dellen) m.msi = m.shift3 / (double)dellen;
        return m;
    }
    Msi msi_insertion(int position, const string &vn) {
        string t1 = vn.substr(1);
        string leftseq = join_ref(R, position - 50 > 1 ? position - 50 : 1, position);
        string t2 = join_ref(R, position + 1, position + 70 > chr_len ? chr_len : position + 70);
        Msi m = find_msi(t1, t2, leftseq);
        Msi t = find_msi(leftseq, t2, "");
        if (m.msi < t.msi) { m.msi = t.msi; m.msint = t.msint; }
        if (m.msi <= m.shift3 / (double)t1.size()) m.msi = m.shift3 / (double)t1.size();
        return m;
    }

    // collectReferenceVariants: src/ToVarsBuilder.cpp:730-1098 (CRISPR mode not restated)
    void collect_reference(int position, int tpc, PosVars &pv) {
        int rfc = 0, rrc = 0;
        string g1;
        Var *refv = pv.ref_idx >= 0 ? &pv.all[pv.ref_idx] : nullptr;
        if (refv && refv->freq >= P.freq) g1 = refv->desc;
        else if (!pv.vars.empty()) g1 = pv.all[pv.vars[0]].desc;
        else if (refv) g1 = refv->desc;
        if (refv) { rfc = refv->fwd; rrc = refv->rev; }
        if (starts_with(g1, "+")) g1 = "+" + std::to_string(g1.size() - 1);
        if (tpc > M.cov[position] && M.nonins.count(position + 1) && R.has(position + 1)) {
            KeyMap &n1 = M.nonins.at(position + 1);
            auto it = n1.find(string(1, R.at(position + 1)));
            if (it != n1.end()) { rfc = it->second.fwd; rrc = it->second.rev; }
        }
        if (!pv.vars.empty()) {
            for (int vi : pv.vars) {
                Var &v = pv.all[vi];
                string g2 = v.desc;
                if (starts_with(g2, "+")) g2 = "+" + std::to_string(g2.size() - 1);
                const string &vn = v.desc;
                int dellen = 0;
                if (vn.size() > 1 && vn[0] == '-' && isdigit((unsigned char)vn[1])) dellen = atoi(vn.c_str() + 1);
                int endp = position;
                if (starts_with(vn, "-")) endp = position + dellen - 1;
                string refa, vara, msint;
                int shift3 = 0;
                double msi = 0;
                int startp = position;
                if (starts_with(vn, "+")) {
                    if (vn.find('&') == string::npos && vn.find('#') == string::npos && vn.find("<dup") == string::npos) {
                        Msi m = msi_insertion(position, vn);
                        msi = m.msi; shift3 = m.shift3; msint = m.msint;
                    }
                    if (P.move_indels_3) { startp += shift3; endp += shift3; }
                    refa = R.has(position) ? string(1, R.at(position)) : "";
                    vara = refa + vn.substr(1);
                } else if (starts_with(vn, "-")) {
                    if (dellen < P.svminlen) {
                        vara = vn;
                        size_t k = 1;
                        while (k < vara.size() && isdigit((unsigned char)vara[k])) k++;
                        if (k > 1) vara.erase(0, k);
                        Msi m = msi_deletion(position, dellen);
                        msi = m.msi; shift3 = m.shift3; msint = m.msint;
                    }
                    if (vn.find('&') == string::npos && vn.find('#') == string::npos && vn.find('^') == string::npos) {
                        if (P.move_indels_3) startp += shift3;
                        if (vara != "<DEL>") vara = R.has(position - 1) ? string(1, R.at(position - 1)) : "";
                        refa = R.has(position - 1) ? string(1, R.at(position - 1)) : "";
                        startp--;
                    }
                    if (dellen < P.svminlen) refa += join_ref(R, position, position + dellen - 1);
                } else {
                    string t1 = join_ref(R, position - 30 > 1 ? position - 30 : 1, position + 1);
                    string t2 = join_ref(R, position + 2, position + 70 > chr_len ? chr_len : position + 70);
                    Msi m = find_msi(t1, t2, "");
                    msi = m.msi; shift3 = m.shift3; msint = m.msint;
                    refa = R.has(position) ? string(1, R.at(position)) : "";
                    vara = vn;
                }
                // AMP_ATGC ".*&([ATGC]+).*": the last '&' followed by a base run
                auto amp_run = [](const string &s, string &run) {
                    for (size_t k = s.size(); k-- > 0;) {
                        if (s[k] == '&' && k + 1 < s.size() && strchr("ATGC", s[k + 1]) && s[k + 1]) {
                            size_t e = k + 1;
                            while (e < s.size() && s[e] && strchr("ATGC", s[e])) e++;
                            run = s.substr(k + 1, e - k - 1);
                            return true;
                        }
                    }
                    return false;
                };
                string extra;
                if (amp_run(vn, extra)) {
                    replace_first(vara, "&", "");
                    string tch = join_ref(R, endp + 1, endp + (int)extra.size());
                    refa += tch;
                    g1 += tch;
                    endp += (int)extra.size();
                    string vextra;
                    if (amp_run(vara, vextra)) {
                        replace_first(vara, "&", "");
                        tch = join_ref(R, endp + 1, endp + (int)vextra.size());
                        refa += tch;
                        g1 += tch;
                        endp += (int)vextra.size();
                    }
                    if (starts_with(vn, "+")) {
                        refa = refa.substr(1);
                        vara = vara.substr(1);
                        startp++;
                    }
                }
                // HASH_GROUP_CARET_GROUP "#(.+)\^(.+)"
                size_t hp = vn.find('#');
                size_t cp = vn.rfind('^');
                if (hp != string::npos && cp != string::npos && cp > hp + 1 && cp + 1 < vn.size()) {
                    string mseq = vn.substr(hp + 1, cp - hp - 1);
                    string tail = vn.substr(cp + 1);
                    endp += (int)mseq.size();
                    refa += join_ref(R, endp - (int)mseq.size() + 1, endp);
                    if (!tail.empty() && isdigit((unsigned char)tail[0])) {
                        int d = atoi(tail.c_str());
                        refa += join_ref(R, endp + 1, endp + d);
                        endp += d;
                    }
                    replace_first(vara, "#", "");
                    size_t c2 = vara.find('^');
                    if (c2 != string::npos) {
                        size_t e = c2 + 1;
                        while (e < vara.size() && isdigit((unsigned char)vara[e])) e++;
                        vara.erase(c2, e - c2);
                    }
                    replace_first(g1, "#", "m");
                    replace_first(g1, "^", "i");
                    replace_first(g2, "#", "m");
                    replace_first(g2, "^", "i");
                }
                // CARET_ATGNC "\^([ATGNC]+)"
                bool caret = false;
                for (size_t k = 0; k + 1 < vn.size(); k++)
                    if (vn[k] == '^' && strchr("ATGNC", vn[k + 1]) && vn[k + 1]) { caret = true; break; }
                if (caret) {
                    replace_first(vara, "^", "");
                    replace_first(g1, "^", "i");
                    replace_first(g2, "^", "i");
                }
                v.leftseq = join_ref(R, startp - 20 < 1 ? 1 : startp - 20, startp - 1);
                v.rightseq = join_ref(R, endp + 1, endp + 20 > chr_len ? chr_len : endp + 20);
                string gt = g1 + "/" + g2;
                string gt2;
                for (char c : gt) {
                    if (c == '&' || c == '#') continue;
                    gt2 += (c == '^') ? 'i' : c;
                }
                v.msi = msi;
                v.msint = (int)msint.size();
                v.shift3 = shift3;
                v.startp = startp;
                v.endp = endp;
                v.refallele = refa;  // validateRefallele is the identity on A/C/G/T/N references
                v.varallele = vara;
                v.genotype = gt2;
                v.tpc = tpc;
                v.rfc = rfc;
                v.rrc = rrc;
                v.sbf = (refv ? refv->sbf : string("0")) + ";" + v.sbf;
                if (v.rfc < 0) v.rfc = 0;
                if (v.rrc < 0) v.rrc = 0;
                if (v.fwd < 0) v.fwd = 0;
                if (v.rev < 0) v.rev = 0;
                v.filled = true;
            }
        } else if (refv) {
            Var &v = *refv;
            v.tpc = tpc;
            v.pc = 0;
            v.freq = 0;
            v.rfc = rfc;
            v.rrc = rrc;
            v.fwd = v.rev = 0;
            v.msi = 0;
            v.msint = 0;
            v.sbf += ";0";
            v.shift3 = 0;
            v.startp = v.endp = position;
            string rb = R.has(position) ? string(1, R.at(position)) : "";
            v.refallele = rb;
            v.varallele = rb;
            v.genotype = rb + "/" + rb;
            v.leftseq = v.rightseq = "";
            v.filled = true;
        }
    }
};

// Variant::varType / isGoodVar / adjComplex: include/Variant.h:99-248
string var_type(const Var &v) {
    const string &r = v.refallele, &a = v.varallele;
    if (r.size() == 1 && a.size() == 1) return "SNV";
    if (a.size() == 5 && a[0] == '<' && a[4] == '>') return a.substr(1, 3);
    if (r.empty() || a.empty()) return "Complex";
    if (r[0] != a[0]) return "Complex";
    if (r.size() == 1 && a.size() > 1 && a.compare(0, 1, r) == 0) return "Insertion";
    if (r.size() > 1 && a.size() == 1 && r.compare(0, 1, a) == 0) return "Deletion";
    return "Complex";
}

bool good_var(const Var &v, const Var *refv, const string &type_in, const rvo_params &P) {
    if (v.refallele.empty()) return false;
    const string type = type_in.empty() ? var_type(v) : type_in;
    if (v.freq < P.freq || v.hicnt < P.minr || v.pmean < P.read_pos_filter || v.qual < P.goodq) return false;
    if (refv && refv->hicnt > P.minr && v.freq < 0.25) {
        double d = v.mq + v.refallele.size() + v.varallele.size();
        double f = (1 + d) / (refv->mq + 1);
        if ((d - 2 < 5 && refv->mq > 20) || f < 0.25) return false;
    }
    if (v.qratio < P.qratio) return false;
    if (v.freq > 0.30) return true;
    if (v.mq < P.mapq_filter) return false;
    if (v.sbf == "2;1" && v.freq < 0.20) {
        if (type.empty() || type == "SNV" || (v.refallele.size() < 3 && v.varallele.size() < 3)) return false;
    }
    return true;
}

void adj_complex(Var &v) {
    string r = v.refallele, a = v.varallele;
    if (!a.empty() && a[0] == '<') return;
    size_t n = 0;
    while (r.size() - n > 1 && a.size() - n > 1 && r[n] == a[n]) n++;
    if (n > 0) {
        v.startp += (int)n;
        v.refallele = r.substr(n);
        v.varallele = a.substr(n);
        v.leftseq += r.substr(0, n);
        v.leftseq = v.leftseq.substr(n);
    }
    r = v.refallele;
    a = v.varallele;
    size_t m = 1;
    while (r.size() > m && a.size() > m && r[r.size() - m] == a[a.size() - m]) m++;
    if (m > 1) {
        v.endp -= (int)(m - 1);
        v.refallele = r.substr(0, r.size() - (m - 1));
        v.varallele = a.substr(0, a.size() - (m - 1));
        long keep = (long)v.rightseq.size() - (long)(m - 1);
        v.rightseq = r.substr(r.size() - (m - 1)) + (keep > 0 ? v.rightseq.substr(0, keep) : string());
    }
}

string fstr(double d) { return std::to_string(d); }

// print_output_variant_simple: src/modes/simpleMode.cpp:66-142
void print_simple(string &out, const Var &v, const char *sample, const char *gene, const char *chr, int rs, int re,
                  bool fisher) {
    vector<string> c;
    c.push_back(sample);
    c.push_back(gene);
    c.push_back(chr);
    c.push_back(std::to_string(v.startp));
    c.push_back(std::to_string(v.endp));
    c.push_back(v.refallele);
    c.push_back(v.varallele);
    c.push_back(std::to_string(v.tpc));
    c.push_back(std::to_string(v.pc));
    c.push_back(std::to_string(v.rfc));
    c.push_back(std::to_string(v.rrc));
    c.push_back(std::to_string(v.fwd));
    c.push_back(std::to_string(v.rev));
    c.push_back(v.genotype.empty() ? "0" : v.genotype);
    c.push_back(fstr(v.freq));
    c.push_back(v.sbf);
    c.push_back(fstr(v.pmean));
    c.push_back(v.pstd ? "1" : "0");
    c.push_back(fstr(v.qual));
    c.push_back(v.qstd ? "1" : "0");
    if (fisher) {
        double l, r, t;
        rv_oracle_fisher(v.rfc, v.rrc, v.fwd, v.rev, &l, &r, &t);
        c.push_back(fstr(t));
        double ad = (double)(v.rfc * v.rev), bc = (double)(v.rrc * v.fwd);
        double ratio = 0.0;
        if (bc != 0 && ad != 0) ratio = ad > bc ? ad / bc : bc / ad;
        c.push_back(fstr(ratio));
    }
    c.push_back(fstr(v.mq));
    c.push_back(fstr(v.qratio));
    c.push_back(fstr(v.hifreq));
    c.push_back(fstr(v.extrafreq));
    c.push_back(std::to_string(v.shift3));
    c.push_back(fstr(v.msi));
    c.push_back(std::to_string(v.msint));
    c.push_back(v.nm > 0 ? fstr(v.nm) : "0");
    c.push_back(std::to_string(v.hicnt));
    c.push_back(std::to_string(v.hicov));
    c.push_back(v.leftseq.empty() ? "0" : v.leftseq);
    c.push_back(v.rightseq.empty() ? "0" : v.rightseq);
    c.push_back(string(chr) + ":" + std::to_string(rs) + "-" + std::to_string(re));
    c.push_back(v.vartype);
    c.push_back(fstr(v.duprate));
    c.push_back("0");
    for (size_t i = 0; i < c.size(); i++) {
        out += c[i];
        out += (i + 1 < c.size()) ? '\t' : '\n';
    }
}

// SimpleMode::output: src/modes/simpleMode.cpp:144-208
long emit_simple(string &out, Scorer &sc, const char *sample, const char *gene, const char *chr, const rvo_params &P) {
    long n = 0;
    for (auto &pe : sc.aligned) {
        int position = pe.first;
        if (position < sc.rs || position > sc.re) continue;
        PosVars &pv = pe.second;
        vector<Var *> vrefs;
        Var *refv = pv.ref_idx >= 0 ? &pv.all[pv.ref_idx] : nullptr;
        if (pv.vars.empty()) {
            if (!P.do_pileup) continue;
            if (!refv) continue;
            refv->vartype = "";
            vrefs.push_back(refv);
        } else {
            for (int vi : pv.vars) {
                Var &v = pv.all[vi];
                if (v.refallele.find('N') != string::npos) continue;
                v.vartype = var_type(v);
                if (!good_var(v, refv, v.vartype, P) && !P.do_pileup) continue;
                vrefs.push_back(&v);
            }
        }
        for (Var *v : vrefs) {
            if (v->vartype == "Complex") adj_complex(*v);
            print_simple(out, *v, sample, gene, chr, sc.rs, sc.re, P.fisher != 0);
            n++;
        }
    }
    return n;
}

// ---------------------------------------------------------------------------
// somatic mode: src/modes/somaticMode.cpp
// ---------------------------------------------------------------------------
struct Somatic {
    const rvo_params &P;
    const char *sample, *gene, *chr;
    int rs, re;
    string &o;
    long n = 0;

    // put_fisher_ext_and_odds (:130-149): two-sided p, then a float32 log ratio
    // with +0.5 pseudocounts
    void fisher_odds(int rf, int rr, int af, int ar) {
        double l, r, t;
        rv_oracle_fisher(rf, rr, af, ar, &l, &r, &t);
        o += std::to_string(t) + "\t";
        const float a = rf + 0.5, b = rr + 0.5, c = af + 0.5, d = ar + 0.5;
        const float ad = a * d, bc = b * c;
        const float ratio = std::log(ad / bc + bc / ad);
        o += std::to_string(ratio) + "\t";
    }

    void stats(const Var *v, const Var *tv) {
        if (!v) {
            for (int i = 0; i < 18; i++) o += "0\t";
            return;
        }
        auto put = [&](const string &x) { o += x; o += '\t'; };
        put(std::to_string(v->tpc));
        put(std::to_string(v->pc));
        put(std::to_string(v->rfc));
        put(std::to_string(v->rrc));
        put(std::to_string(v->fwd));
        put(std::to_string(v->rev));
        // the normal column prints the tumor genotype (:218)
        put(v->genotype.empty() ? "0" : tv->genotype);
        put(fstr(v->freq));
        put(v->sbf);
        put(fstr(v->pmean));
        put(v->pstd ? "1" : "0");
        put(fstr(v->qual));
        put(v->qstd ? "1" : "0");
        put(fstr(v->mq));
        put(fstr(v->qratio));
        put(fstr(v->hifreq));
        put(fstr(v->extrafreq));
        put(fstr(v->nm));
    }

    // print_output_variant_simple (:151-309)
    void print(const Var *beg, const Var *end, const Var *tv, const Var *nv, const string &label) {
        o += string(sample) + "\t" + gene + "\t" + chr + "\t";
        if (beg)
            o += std::to_string(beg->startp) + "\t" + std::to_string(beg->endp) + "\t" + beg->refallele + "\t" +
                 beg->varallele + "\t";
        else
            o += "0\t0\t0\t0\t";
        stats(tv, tv);
        if (P.fisher) {
            if (tv) fisher_odds(tv->rfc, tv->rrc, tv->fwd, tv->rev);
            else o += "0\t0\t";
        }
        stats(nv, tv);
        if (P.fisher) {
            if (nv) fisher_odds(nv->rfc, nv->rrc, nv->fwd, nv->rev);
            else o += "0\t0\t";
        }
        if (end)
            o += std::to_string(end->shift3) + "\t" + fstr(end->msi) + "\t" + std::to_string(end->msint) + "\t" +
                 (end->leftseq.empty() ? string("0") : end->leftseq) + "\t" +
                 (end->rightseq.empty() ? string("0") : end->rightseq) + "\t";
        else
            o += "\t\t\t\t\t";
        o += string(chr) + ":" + std::to_string(rs) + "-" + std::to_string(re) + "\t";
        o += label + "\t";
        o += (beg ? beg->vartype : string()) + "\t";
        o += (tv ? fstr(tv->duprate) : string("0")) + "\t0\t";
        o += (nv ? fstr(nv->duprate) : string("0")) + "\t0\t";
        if (P.fisher) {
            int t_tot = tv ? tv->tpc : 0, t_var = tv ? tv->pc : 0;
            int n_tot = nv ? nv->tpc : 0, n_var = nv ? nv->pc : 0;
            int tref = t_tot - t_var, rref = n_tot - n_var;
            if (tref < 0) tref = 0;
            if (rref < 0) rref = 0;
            fisher_odds(t_var, tref, n_var, rref);
            double tvaf = tv ? tv->freq : 0, nvaf = nv ? nv->freq : 0;
            o += std::to_string(std::log(std::max(tvaf, 0.0001) / std::max(nvaf, 0.0001))) + "\t";
            o += std::to_string(std::log((static_cast<float>(t_var) + 0.5) / (static_cast<float>(n_var) + 0.5))) +
                 "\t";
        }
        o += "\n";
        n++;
    }

    static Var *find(PosVars &pv, const string &desc) {
        for (int vi : pv.vars)
            if (pv.all[vi].desc == desc) return &pv.all[vi];
        return nullptr;
    }
    static Var *refv(PosVars &pv) { return pv.ref_idx >= 0 ? &pv.all[pv.ref_idx] : nullptr; }

    // Variant::isNoise (include/Variant.h:75-94): zeroes the counts of a noise variant
    bool is_noise(Var &v) {
        const double q = v.qual;
        if (((q < 4.5 || (q < 12 && !v.qstd)) && v.pc <= 3) || (q < P.goodq && v.freq < 2 * P.lofreq && v.pc <= 1)) {
            v.tpc -= v.pc;
            v.pc = 0;
            v.fwd = v.rev = 0;
            v.freq = 0;
            v.hifreq = 0;
            return true;
        }
        return false;
    }

    // determinateType (:608-633)
    string determinate(PosVars &v2, Var &std_v, Var &cmp) {
        string type;
        if (good_var(cmp, refv(v2), std_v.vartype, P)) {
            if (std_v.freq > 1 - P.lofreq && cmp.freq < 0.8 && cmp.freq > 0.2) type = "LikelyLOH";
            else if (cmp.freq < P.lofreq || cmp.pc <= 1) type = "LikelySomatic";
            else type = "Germline";
        } else {
            if (cmp.freq < P.lofreq || cmp.pc <= 1) type = "LikelySomatic";
            else type = "AFDiff";
        }
        if (is_noise(cmp) && std_v.vartype == "SNV") type = "StrongSomatic";
        return type;
    }

    // callingForOneSample (:360-380), tumor only
    void one_sample(PosVars &v1, const string &label) {
        for (int vi : v1.vars) {
            Var &v = v1.all[vi];
            v.vartype = var_type(v);
            if (!good_var(v, refv(v1), v.vartype, P)) continue;
            if (v.vartype == "Complex") adj_complex(v);
            print(&v, &v, &v, nullptr, label);
        }
    }

    // printVariationsFromFirstSample (:405-530)
    void first_sample(PosVars &v1, PosVars &v2) {
        size_t k = 0;
        while (k < v1.vars.size() && good_var(v1.all[v1.vars[k]], refv(v1), v1.all[v1.vars[k]].vartype, P)) {
            Var &vref = v1.all[v1.vars[k]];
            vref.vartype = var_type(vref);
            if (vref.vartype == "Complex") adj_complex(vref);
            Var *v2nt = find(v2, vref.desc);
            if (v2nt) {
                string type = determinate(v2, vref, *v2nt);
                print(&vref, v2nt, &vref, v2nt, type);
            } else {
                // sample 1 only; combineAnalysis (:639-735) needs a '<' in the
                // description, which no key of this pipeline has
                Var shown;
                const Var *vfp;
                if (!v2.vars.empty()) {
                    const Var &v2r = v2.all[v2.vars[0]];
                    shown.tpc = v2r.tpc;
                    shown.rfc = v2r.rfc;
                    shown.rrc = v2r.rrc;
                    vfp = &shown;
                } else {
                    vfp = refv(v2);
                }
                print(&vref, &vref, &vref, vfp, "StrongSomatic");
            }
            k++;
        }
        if (k > 0 || v2.vars.empty()) return;
        for (int vi : v2.vars) {
            Var &v2var = v2.all[vi];
            v2var.vartype = var_type(v2var);
            if (!good_var(v2var, refv(v2), v2var.vartype, P)) continue;
            Var *v1nt = find(v1, v2var.desc);
            if (v1nt) {
                string type = v1nt->freq < P.lofreq ? "LikelyLOH" : "Germline";
                if (v2var.vartype == "Complex") adj_complex(*v1nt);
                v1nt->vartype = var_type(*v1nt);
                print(v1nt, &v2var, v1nt, &v2var, type);
            } else {
                const Var *v1var = v1.vars.empty() ? nullptr : &v1.all[v1.vars[0]];
                const Var *v1ref = refv(v1);
                Var shown;
                shown.tpc = v1var ? v1var->tpc : 0;
                shown.rfc = v1ref ? v1ref->fwd : 0;
                shown.rrc = v1ref ? v1ref->rev : 0;
                shown.genotype = v1var ? v1var->genotype : (v1ref ? v1ref->desc + "/" + v1ref->desc : "N/N");
                if (v2var.vartype == "Complex") adj_complex(v2var);
                print(&v2var, &v2var, &shown, &v2var, "StrongLOH");
            }
        }
    }

    // printVariationsFromSecondSample (:537-600)
    void second_sample(PosVars &v1, PosVars &v2) {
        for (int vi : v2.vars) {
            Var &v2var = v2.all[vi];
            v2var.vartype = var_type(v2var);
            if (!good_var(v2var, refv(v2), v2var.vartype, P)) continue;
            Var *v1nt = find(v1, v2var.desc);
            if (v1nt) v1nt->pc = 0;
            const Var *vfp = refv(v1);
            if (v2var.vartype == "Complex") adj_complex(v2var);
            print(&v2var, &v2var, vfp, &v2var, "StrongLOH");
        }
    }

    // SomaticMode::output (:311-353): positions of the first BAM only
    void run(Scorer &t, Scorer &nrm) {
        for (auto &pe : t.aligned) {
            int position = pe.first;
            if (position < rs || position > re) continue;
            PosVars &v1 = pe.second;
            auto it = nrm.aligned.find(position);
            if (it == nrm.aligned.end()) {
                if (!v1.vars.empty()) one_sample(v1, "SampleSpecific");
                continue;
            }
            PosVars &v2 = it->second;
            if (v1.vars.empty() && v2.vars.empty()) continue;
            if (!v1.vars.empty()) first_sample(v1, v2);
            else second_sample(v1, v2);
        }
    }
};

// ---------------------------------------------------------------------------
// record iteration: sam_itr_querys + RecordPreprocessor::next_record
// (src/recordPreprocessor.cpp:101-180)
// ---------------------------------------------------------------------------
void load_read(const rvo_reads *rd, int64_t i, ReadView &r) {
    r.pos = rd->pos[i];
    r.mpos = rd->mpos[i];
    r.nm = rd->nm[i];
    r.flag = rd->flag[i];
    r.mapq = rd->mapq[i];
    r.lseq = rd->l_qseq[i];
    r.n_cigar = rd->n_cigar[i];
    const uint8_t *s4 = rd->seq4 + rd->base_off[i];
    const uint8_t *q = rd->qual + rd->base_off[i];
    r.seq.assign(r.lseq + 8, 0);
    for (int k = 0; k < r.lseq; k++) r.seq[k] = kNt16[s4[k] & 15];
    // the bytes that follow the CIGAR in a BAM record: packed bases, then quals
    vector<uint8_t> tail;
    for (int k = 0; k < r.lseq; k += 2)
        tail.push_back((uint8_t)(((s4[k] & 15) << 4) | (k + 1 < r.lseq ? (s4[k + 1] & 15) : 0)));
    uint8_t before_qual = tail.empty() ? 0 : tail.back();
    for (int k = 0; k < r.lseq; k++) tail.push_back(q[k]);
    while (tail.size() < 32) tail.push_back(0);
    r.cig.assign(rd->cigar + rd->cig_off[i], rd->cigar + rd->cig_off[i] + r.n_cigar);
    for (int w = 0; w < 4; w++) {
        uint32_t v = 0;
        memcpy(&v, &tail[4 * w], 4);
        r.cig.push_back(v);
    }
    r.qual_buf.assign(r.lseq + 9, 0);
    r.qual_buf[0] = before_qual;
    memcpy(r.qual_buf.data() + 1, q, r.lseq);
}

int ref_span(const rvo_reads *rd, int64_t i) {
    int len = 0;
    const uint32_t *c = rd->cigar + rd->cig_off[i];
    for (int k = 0; k < rd->n_cigar[i]; k++) {
        int o = c[k] & 15;
        if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) len += c[k] >> 4;
    }
    return len;
}

void run_pileup(const rvo_reads *rd, const rvo_params &P, int rs, int re, int chr_len, Maps &M, Ref &R) {
    // reads overlapping [rs-1, re) in 0-based half-open coordinates, file order
    int64_t lo = 0, hi = rd->n;
    while (lo < hi) {  // first read with pos >= rs - 1 - max_span
        int64_t mid = (lo + hi) / 2;
        if (rd->pos[mid] < rs - 1 - 4096) lo = mid + 1; else hi = mid;
    }
    Walker W(P, M, R, rs, re, chr_len);
    std::set<string> dups;
    int first_match = 0;
    ReadView r;
    for (int64_t i = lo; i < rd->n && rd->pos[i] < re; i++) {
        int span = ref_span(rd, i);
        int endpos = ((rd->flag[i] & 4) || span == 0) ? rd->pos[i] + 1 : rd->pos[i] + span;
        if (endpos <= rs - 1) continue;
        uint16_t fl = rd->flag[i];
        if (fl & P.samfilter) continue;
        if (rd->mapq[i] < P.min_mapq) continue;
        if (rd->l_qseq[i] == 1) continue;
        if (P.dedup) {
            int a = rd->pos[i] + 1, m = rd->mpos[i] + 1;
            if (a != first_match) dups.clear();
            string mref = (fl & 1) ? "=" : "*";
            if (m < 10) {
                string k = std::to_string(a) + "-" + mref + "-" + std::to_string(m);
                if (dups.count(k)) continue;
                dups.insert(k);
                first_match = a;
            } else if ((fl & 1) && (fl & 4)) {
                string k = std::to_string(a) + "-";
                const uint32_t *c = rd->cigar + rd->cig_off[i];
                for (int q = 0; q < rd->n_cigar[i]; q++) k += std::to_string(c[q] >> 4) + "MIDNSHP=XB"[c[q] & 15];
                if (dups.count(k)) continue;
                dups.insert(k);
                first_match = a;
            }
        }
        load_read(rd, i, r);
        W.parse(r);
    }
}

void fmt_stat(string &o, const char *tag, int pos, const string &key, const Stat &v) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s\t%d\t%s\t%d\t%d\t%d\t%.17g\t%.17g\t%.17g\t%.17g\t%d\t%d\t%d\t%d\t%d\t%.17g\t%d\n", tag,
             pos, key.c_str(), v.cnt, v.fwd, v.rev, v.pmean, v.qmean, v.mq, v.nm, v.lo, v.hi, (int)v.pstd, (int)v.qstd,
             v.pp, v.pq, v.extracnt);
    o += buf;
}

void dump_maps(string &o, const char *pfx, Maps &M, bool full) {
    string t;
    char buf[64];
    if (full) {
        snprintf(buf, sizeof buf, "%s_ML\t%d\n", pfx, M.max_read_len);
        o += buf;
    }
    for (auto &pe : M.nonins)
        for (auto &ke : pe.second) fmt_stat(o, (string(pfx) + "N").c_str(), pe.first, ke.first, ke.second);
    for (auto &pe : M.ins)
        for (auto &ke : pe.second) fmt_stat(o, (string(pfx) + "I").c_str(), pe.first, ke.first, ke.second);
    for (auto &ce : M.cov) {
        snprintf(buf, sizeof buf, "%sC\t%d\t%d\n", pfx, ce.first, ce.second);
        o += buf;
    }
    if (!full) return;
    for (int side = 0; side < 2; side++) {
        auto &mm = side == 0 ? M.sc5 : M.sc3;
        string tag = string(pfx) + (side == 0 ? "S5" : "S3");
        for (auto &se : mm) {
            fmt_stat(o, tag.c_str(), se.first, "*", se.second);
            for (auto &ne : se.second.nt) {
                vector<char> cs;
                for (auto &c : ne.second) cs.push_back(c.first);
                std::sort(cs.begin(), cs.end());
                for (char c : cs) {
                    char key[64];
                    snprintf(key, sizeof key, "%d:%c:%d", ne.first, c, ne.second.at(c));
                    fmt_stat(o, tag.c_str(), se.first, key, se.second.seq.at(ne.first).at(c));
                }
            }
        }
    }
    auto cnts = [&](const char *tg, map<int, map<string, int>> &mm) {
        for (auto &pe : mm)
            for (auto &ke : pe.second) {
                o += string(pfx) + tg + "\t" + std::to_string(pe.first) + "\t" + ke.first + "\t" +
                     std::to_string(ke.second) + "\n";
            }
    };
    cnts("CI", M.inscnt);
    cnts("CD", M.delcnt);
    cnts("MN", M.mnp);
}

void dump_variants(string &o, Scorer &sc) {
    char buf[2048];
    for (auto &pe : sc.aligned) {
        PosVars &pv = pe.second;
        auto one = [&](const char *kind, const Var &v) {
            snprintf(buf, sizeof buf,
                     "V\t%d\t%s\t%s\t%d\t%d\t%d\t%s\t%.17g\t%.17g\t%d\t%.17g\t%d\t%.17g\t%.17g\t%.17g\t%.17g\t%d\t%.17g"
                     "\t%d\t%.17g\t%d\t%d\t%s\t%s\t%d\t%d\t%d\t%d\t%d\t%s\t%s\t%s\n",
                     pe.first, kind, v.desc.c_str(), v.pc, v.fwd, v.rev, v.sbf.c_str(), v.freq, v.pmean, (int)v.pstd,
                     v.qual, (int)v.qstd, v.mq, v.qratio, v.hifreq, v.extrafreq, v.shift3, v.msi, v.msint, v.nm,
                     v.hicnt, v.hicov, v.leftseq.c_str(), v.rightseq.c_str(), v.startp, v.endp, v.rfc, v.rrc, v.tpc,
                     v.genotype.c_str(), v.refallele.c_str(), v.varallele.c_str());
            o += buf;
        };
        if (pv.ref_idx >= 0) one("ref", pv.all[pv.ref_idx]);
        for (int vi : pv.vars) one("var", pv.all[vi]);
    }
}

void setup_ref(Ref &R, const char *ref, int clen, int rs, int re, const rvo_params &P) {
    R.contig = ref;
    R.clen = clen;
    int ext = P.ref_extension, x = P.extend_nt;
    R.lo = rs - x - ext < 1 ? 1 : rs - x - ext;
    int seq_end = re + x + ext > clen ? clen : re + x + ext;
    R.hi = seq_end - 17;
}

}  // namespace

extern "C" {

void rvo_default_params(rvo_params *p) {
    memset(p, 0, sizeof *p);
    p->goodq = 22.5;
    p->vext = 2;
    p->mismatch = 8;
    p->local_realign = 1;
    p->freq = 0.01;
    p->minr = 2;
    p->read_pos_filter = 5;
    p->qratio = 1.5;
    p->mapq_filter = 0;
    p->min_mapq = 0;
    p->lofreq = 0.05;
    p->bias = 0.05;
    p->min_bias_reads = 2;
    p->samfilter = 0x504;
    p->ref_extension = 1200;
    p->svminlen = 1000;
}

int rvo_run_region(const rvo_reads *reads, const char *ref, int contig_len, const char *chr, int start, int end,
                   const char *sample, const rvo_params *p, const char *stages, char **out, size_t *out_len) {
    Maps M;
    Ref R;
    setup_ref(R, ref, contig_len, start, end, *p);
    try {
        run_pileup(reads, *p, start, end, contig_len, M, R);
    } catch (const UnsupportedRead &) {
        const char *msg = "ERROR unsupported read (leading D or a CIGAR rewrite longer than the record allows)\n";
        *out = strdup(msg);
        *out_len = strlen(msg);
        return -5;
    }
    string o;
    if (strchr(stages, 'P')) dump_maps(o, "P", M, true);
    realign(M, R, *p, reads, start, end, contig_len);
    if (strchr(stages, 'R')) dump_maps(o, "R", M, false);
    Scorer sc(*p, M, R, contig_len, start, end);
    sc.run();
    if (strchr(stages, 'V')) dump_variants(o, sc);
    if (strchr(stages, 'O')) emit_simple(o, sc, sample, chr, chr, *p);
    *out = (char *)malloc(o.size() + 1);
    memcpy(*out, o.data(), o.size());
    (*out)[o.size()] = 0;
    *out_len = o.size();
    return 0;
}

long rvo_run_regions(const rvo_reads *reads, const char *ref, int contig_len, const char *chr, const int32_t *starts,
                     const int32_t *ends, int n_regions, const char *sample, const rvo_params *p, int threads,
                     char **out, size_t *out_len) {
    vector<string> per(n_regions);
    vector<long> cnt(n_regions, 0);
#pragma omp parallel for schedule(dynamic) num_threads(threads > 0 ? threads : 1)
    for (int i = 0; i < n_regions; i++) {
        Maps M;
        Ref R;
        setup_ref(R, ref, contig_len, starts[i], ends[i], *p);
        run_pileup(reads, *p, starts[i], ends[i], contig_len, M, R);
        realign(M, R, *p, reads, starts[i], ends[i], contig_len);
        Scorer sc(*p, M, R, contig_len, starts[i], ends[i]);
        sc.run();
        cnt[i] = emit_simple(per[i], sc, sample, chr, chr, *p);
    }
    string o;
    long n = 0;
    for (int i = 0; i < n_regions; i++) { o += per[i]; n += cnt[i]; }
    *out = (char *)malloc(o.size() + 1);
    memcpy(*out, o.data(), o.size());
    (*out)[o.size()] = 0;
    *out_len = o.size();
    return n;
}

// SomaticMode::process / one_region_run_somt (src/modes/somaticMode.cpp:83-127):
// the tumor (first BAM) and the normal run the same per-region pipeline on a
// shared reference window, then the two variant sets are classified.
static long somatic_region(const rvo_reads *tumor, const rvo_reads *normal, const char *ref, int contig_len,
                           const char *chr, int start, int end, const char *sample, const rvo_params &P,
                           const char *stages, string &o) {
    Maps MT, MN;
    Ref R;
    setup_ref(R, ref, contig_len, start, end, P);
    run_pileup(tumor, P, start, end, contig_len, MT, R);
    realign(MT, R, P, tumor, start, end, contig_len);
    Scorer st(P, MT, R, contig_len, start, end, true);
    st.run();
    run_pileup(normal, P, start, end, contig_len, MN, R);
    realign(MN, R, P, normal, start, end, contig_len);
    Scorer sn(P, MN, R, contig_len, start, end, true);
    sn.run();
    if (strchr(stages, 'V')) {
        string a, b;
        dump_variants(a, st);
        dump_variants(b, sn);
        for (size_t i = 0; i < a.size(); i++) o += (i == 0 || a[i - 1] == '\n') && a[i] == 'V' ? "VT" : string(1, a[i]);
        for (size_t i = 0; i < b.size(); i++) o += (i == 0 || b[i - 1] == '\n') && b[i] == 'V' ? "VN" : string(1, b[i]);
    }
    if (!strchr(stages, 'O')) return 0;
    Somatic so{P, sample, chr, chr, start, end, o};
    so.run(st, sn);
    return so.n;
}

int rvo_run_somatic(const rvo_reads *tumor, const rvo_reads *normal, const char *ref, int contig_len, const char *chr,
                    int start, int end, const char *sample, const rvo_params *p, const char *stages, char **out,
                    size_t *out_len) {
    string o;
    somatic_region(tumor, normal, ref, contig_len, chr, start, end, sample, *p, stages, o);
    *out = (char *)malloc(o.size() + 1);
    memcpy(*out, o.data(), o.size());
    (*out)[o.size()] = 0;
    *out_len = o.size();
    return 0;
}

long rvo_run_somatic_regions(const rvo_reads *tumor, const rvo_reads *normal, const char *ref, int contig_len,
                             const char *chr, const int32_t *starts, const int32_t *ends, int n_regions,
                             const char *sample, const rvo_params *p, int threads, char **out, size_t *out_len) {
    vector<string> per(n_regions);
    vector<long> cnt(n_regions, 0);
#pragma omp parallel for schedule(dynamic) num_threads(threads > 0 ? threads : 1)
    for (int i = 0; i < n_regions; i++)
        cnt[i] = somatic_region(tumor, normal, ref, contig_len, chr, starts[i], ends[i], sample, *p, "O", per[i]);
    string o;
    long n = 0;
    for (int i = 0; i < n_regions; i++) { o += per[i]; n += cnt[i]; }
    *out = (char *)malloc(o.size() + 1);
    memcpy(*out, o.data(), o.size());
    (*out)[o.size()] = 0;
    *out_len = o.size();
    return n;
}

void rvo_free(char *p) { free(p); }

double rvo_fisher(int n11, int n12, int n21, int n22, double *left, double *right, double *two) {
    return rv_oracle_fisher(n11, n12, n21, n22, left, right, two);
}
}
