// Allele strings, hard filter and complex-variant trimming of called
// variants (declarations and reference citations in rv_records.h).
#include "rv_records.h"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace rv {
namespace recs {

const char kBases[4] = {'A', 'C', 'G', 'T'};

// findMSI with curmsi_from_end (src/ToVarsBuilder.cpp:614-678)
Msi find_msi(const std::string &t1, const std::string &t2, const std::string &left) {
    int nmsi = 1, shift3 = 0;
    std::string best;
    double best_cnt = 0;
    std::string both = left + t1;
    while (nmsi <= (int)t1.size() && nmsi <= 6) {
        std::string unit = t1.substr(t1.size() - nmsi, nmsi);
        double cur = 1.0;
        for (int i = (int)both.size() - nmsi; i > 0; i -= nmsi) {
            if (i > nmsi && both.compare(i - nmsi, nmsi, unit) == 0) cur += 1;
            else break;
        }
        for (int i = 0; i < (int)t2.size(); i += nmsi) {
            if (i + nmsi < (int)t2.size() && t2.compare(i, nmsi, unit) == 0) cur += 1.0;
            else break;
        }
        if (cur > best_cnt) { best = unit; best_cnt = cur; }
        nmsi++;
    }
    std::string ts = t1 + t2;
    while (shift3 < (int)t2.size() && ts[shift3] == t2[shift3]) shift3++;
    return {best_cnt, shift3, best};
}

std::string join(const RefWin &R, int from, int to) {
    if (from > to) return std::string();
    if (!R.has(from) || !R.has(to)) throw NoRef();  // the window is one contiguous range
    return std::string(R.ref->data() + (from - 1), (size_t)(to - from + 1));
}

// joinRef's failure condition without building the string
void join_check(const RefWin &R, int from, int to) {
    if (from <= to && (!R.has(from) || !R.has(to))) throw NoRef();
}

void repl_first(std::string &s, const std::string &a, const std::string &b) {
    size_t p = s.find(a);
    if (p != std::string::npos) s.replace(p, a.size(), b);
}


// last '&' followed by an A/C/G/T run (the ".*&([ATGC]+).*" search)
bool amp_tail(const std::string &s, std::string &run) {
    for (size_t k = s.size(); k-- > 0;) {
        if (s[k] == '&' && k + 1 < s.size() && strchr("ATGC", s[k + 1]) && s[k + 1]) {
            size_t e = k + 1;
            while (e < s.size() && s[e] && strchr("ATGC", s[e])) e++;
            run = s.substr(k + 1, e - k - 1);
            return true;
        }
    }
    return false;
}

// collectReferenceVariants for one variant.  With full == false (a variant
// the device pre-screen rules out of the output) only what can affect later
// variants of the position is done: the genotype-1 edits and the
// reference-window checks whose failure ends the position.
void describe(RecVar &v, std::string &g1, int position, const RefWin &R, const rv_params &P, bool full) {
    std::string g2 = v.desc;
    if (starts(g2, '+')) g2 = "+" + std::to_string(g2.size() - 1);
    const std::string &vn = v.desc;
    int dellen = 0;
    if (vn.size() > 1 && vn[0] == '-' && isdigit((unsigned char)vn[1])) dellen = atoi(vn.c_str() + 1);
    int endp = position, startp = position, shift3 = 0;
    if (starts(vn, '-')) endp = position + dellen - 1;
    std::string refa, vara, unit;
    double msi = 0;
    int L = R.len;
    if (starts(vn, '+')) {
        if (vn.find('&') == std::string::npos && vn.find('#') == std::string::npos && vn.find("<dup") == std::string::npos) {
            if (!full) {
                join_check(R, position - 50 > 1 ? position - 50 : 1, position);
                join_check(R, position + 1, position + 70 > L ? L : position + 70);
            } else {
            std::string t1 = vn.substr(1);
            std::string left = join(R, position - 50 > 1 ? position - 50 : 1, position);
            std::string t2 = join(R, position + 1, position + 70 > L ? L : position + 70);
            Msi a = find_msi(t1, t2, left), b = find_msi(left, t2, "");
            if (a.msi < b.msi) { a.msi = b.msi; a.unit = b.unit; }
            if (a.msi <= a.shift3 / (double)t1.size()) a.msi = a.shift3 / (double)t1.size();
            msi = a.msi; shift3 = a.shift3; unit = a.unit;
            }
        }
        if (P.move_indels_3) { startp += shift3; endp += shift3; }
        refa = R.has(position) ? std::string(1, R.at(position)) : "";
        vara = refa + vn.substr(1);
    } else if (starts(vn, '-')) {
        if (dellen < P.svminlen) {
            vara = vn;
            size_t k = 1;
            while (k < vara.size() && isdigit((unsigned char)vara[k])) k++;
            if (k > 1) vara.erase(0, k);
            if (!full) {
                join_check(R, position - 70 > 1 ? position - 70 : 1, position - 1);
                join_check(R, position, position + dellen + 70 > L ? L : position + dellen + 70);
            } else {
            std::string left = join(R, position - 70 > 1 ? position - 70 : 1, position - 1);
            std::string ts = join(R, position, position + dellen + 70 > L ? L : position + dellen + 70);
            std::string a1 = ts.substr(0, std::min<size_t>(dellen, ts.size()));
            std::string a2 = (size_t)dellen <= ts.size() ? ts.substr(dellen) : std::string();
            Msi a = find_msi(a1, a2, left), b = find_msi(left, a2, "");
            if (a.msi < b.msi) { a.msi = b.msi; a.unit = b.unit; }
            if (a.msi <= a.shift3 / (double)dellen) a.msi = a.shift3 / (double)dellen;
            msi = a.msi; shift3 = a.shift3; unit = a.unit;
            }
        }
        if (vn.find('&') == std::string::npos && vn.find('#') == std::string::npos && vn.find('^') == std::string::npos) {
            if (P.move_indels_3) startp += shift3;
            if (vara != "<DEL>") vara = R.has(position - 1) ? std::string(1, R.at(position - 1)) : "";
            refa = R.has(position - 1) ? std::string(1, R.at(position - 1)) : "";
            startp--;
        }
        if (dellen < P.svminlen) refa += join(R, position, position + dellen - 1);
    } else {
        if (!full) {
            join_check(R, position - 30 > 1 ? position - 30 : 1, position + 1);
            join_check(R, position + 2, position + 70 > L ? L : position + 70);
        } else {
            std::string t1 = join(R, position - 30 > 1 ? position - 30 : 1, position + 1);
            std::string t2 = join(R, position + 2, position + 70 > L ? L : position + 70);
            Msi a = find_msi(t1, t2, "");
            msi = a.msi; shift3 = a.shift3; unit = a.unit;
        }
        refa = R.has(position) ? std::string(1, R.at(position)) : "";
        vara = vn;
    }
    std::string extra;
    if (amp_tail(vn, extra)) {
        repl_first(vara, "&", "");
        std::string tch = join(R, endp + 1, endp + (int)extra.size());
        refa += tch;
        g1 += tch;
        endp += (int)extra.size();
        std::string vextra;
        if (amp_tail(vara, vextra)) {
            repl_first(vara, "&", "");
            tch = join(R, endp + 1, endp + (int)vextra.size());
            refa += tch;
            g1 += tch;
            endp += (int)vextra.size();
        }
        if (starts(vn, '+')) {
            refa = refa.substr(1);
            vara = vara.substr(1);
            startp++;
        }
    }
    size_t hp = vn.find('#'), cp = vn.rfind('^');
    if (hp != std::string::npos && cp != std::string::npos && cp > hp + 1 && cp + 1 < vn.size()) {
        std::string mseq = vn.substr(hp + 1, cp - hp - 1), tail = vn.substr(cp + 1);
        endp += (int)mseq.size();
        refa += join(R, endp - (int)mseq.size() + 1, endp);
        if (!tail.empty() && isdigit((unsigned char)tail[0])) {
            int d = atoi(tail.c_str());
            refa += join(R, endp + 1, endp + d);
            endp += d;
        }
        repl_first(vara, "#", "");
        size_t c2 = vara.find('^');
        if (c2 != std::string::npos) {
            size_t e = c2 + 1;
            while (e < vara.size() && isdigit((unsigned char)vara[e])) e++;
            vara.erase(c2, e - c2);
        }
        repl_first(g1, "#", "m");
        repl_first(g1, "^", "i");
        repl_first(g2, "#", "m");
        repl_first(g2, "^", "i");
    }
    for (size_t k = 0; k + 1 < vn.size(); k++) {
        if (vn[k] == '^' && vn[k + 1] && strchr("ATGNC", vn[k + 1])) {
            repl_first(vara, "^", "");
            repl_first(g1, "^", "i");
            repl_first(g2, "^", "i");
            break;
        }
    }
    if (!full) {
        join_check(R, startp - 20 < 1 ? 1 : startp - 20, startp - 1);
        join_check(R, endp + 1, endp + 20 > L ? L : endp + 20);
        return;  // not emitted: no record fields needed
    }
    v.leftseq = join(R, startp - 20 < 1 ? 1 : startp - 20, startp - 1);
    v.rightseq = join(R, endp + 1, endp + 20 > L ? L : endp + 20);
    std::string gt;
    for (char c : g1 + "/" + g2) {
        if (c == '&' || c == '#') continue;
        gt += c == '^' ? 'i' : c;
    }
    v.msi = msi;
    v.msint = (int)unit.size();
    v.shift3 = shift3;
    v.startp = startp;
    v.endp = endp;
    v.refallele = refa;
    v.varallele = vara;
    v.genotype = gt;
    v.filled = true;
}

std::string var_type(const RecVar &v) {
    const std::string &r = v.refallele, &a = v.varallele;
    if (r.size() == 1 && a.size() == 1) return "SNV";
    if (a.size() == 5 && a[0] == '<' && a[4] == '>') return a.substr(1, 3);
    if (r.empty() || a.empty()) return "Complex";
    if (r[0] != a[0]) return "Complex";
    if (r.size() == 1 && a.size() > 1 && a[0] == r[0]) return "Insertion";
    if (r.size() > 1 && a.size() == 1 && r[0] == a[0]) return "Deletion";
    return "Complex";
}

bool good_var(const RecVar &v, const CandVar *ref, const rv_params &P, const std::string &type_in) {
    const CandVar &c = *v.c;
    if (v.refallele.empty()) return false;
    const std::string type = type_in.empty() ? var_type(v) : type_in;
    if (c.freq < P.freq || c.hicnt < P.minr || c.pmean < P.read_pos_filter || c.qual < P.goodq) return false;
    if (ref && ref->hicnt > P.minr && c.freq < 0.25) {
        double d = c.mq + v.refallele.size() + v.varallele.size();
        double f = (1 + d) / (ref->mq + 1);
        if ((d - 2 < 5 && ref->mq > 20) || f < 0.25) return false;
    }
    if (c.qratio < P.qratio) return false;
    if (c.freq > 0.30) return true;
    if (c.mq < P.mapq_filter) return false;
    if (v.sbf == "2;1" && c.freq < 0.20) {
        if (type.empty() || type == "SNV" || (v.refallele.size() < 3 && v.varallele.size() < 3)) return false;
    }
    return true;
}

void adj_complex(RecVar &v) {
    std::string r = v.refallele, a = v.varallele;
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
        v.rightseq = r.substr(r.size() - (m - 1)) + (keep > 0 ? v.rightseq.substr(0, keep) : std::string());
    }
}

}  // namespace recs
}  // namespace rv
