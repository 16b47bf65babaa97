// Hand-written matchers for the allele-key patterns the -k 1 realigner reads
// (src/VariationRealigner.cpp realigndel :489-775, realignins :785-1117; the
// patterns of include/patterns.h), and its soft-clip pairing scan find35match
// (:1396-1428).  Each matcher gives the same result as the std::regex
// (ECMAScript) search it replaces, without the regex engine: the keys are
// short, their grammar is fixed (digits, bases, '&' '#' '^' '+' '-' '<' '>';
// never a line break, so '.' matches any character here), and the realigner
// runs these on every candidate allele.
#pragma once
#include <cstddef>
#include <string>

namespace rv {
namespace keymatch {

inline bool is_digit(char c) { return c >= '0' && c <= '9'; }
inline bool is_atgc(char c) { return c == 'A' || c == 'T' || c == 'G' || c == 'C'; }
inline bool is_atgnc(char c) { return is_atgc(c) || c == 'N'; }

// end of the run of characters satisfying `pred` starting at i
template <class Pred>
inline size_t run_end(const std::string &s, size_t i, Pred pred) {
    while (i < s.size() && pred(s[i])) i++;
    return i;
}

// ^-\d+\^([ATGNC]+)<...\d+>([ATGNC]+)$
inline bool inv(const std::string &s, std::string &g1, std::string &g2) {
    if (s.empty() || s[0] != '-') return false;
    size_t i = run_end(s, 1, is_digit);
    if (i == 1 || i >= s.size() || s[i] != '^') return false;
    size_t j = run_end(s, i + 1, is_atgnc);
    if (j == i + 1 || j >= s.size() || s[j] != '<') return false;
    size_t k = j + 4;  // '<' and three characters
    if (k > s.size()) return false;
    size_t d = run_end(s, k, is_digit);
    if (d == k || d >= s.size() || s[d] != '>') return false;
    size_t e = run_end(s, d + 1, is_atgnc);
    if (e == d + 1 || e != s.size()) return false;
    g1 = s.substr(i + 1, j - i - 1);
    g2 = s.substr(d + 1);
    return true;
}

// ^-\d+(.*)   (group 1: everything after the digit run)
inline bool del_rest(const std::string &s, std::string &g1) {
    if (s.empty() || s[0] != '-') return false;
    size_t i = run_end(s, 1, is_digit);
    if (i == 1) return false;
    g1 = s.substr(i);
    return true;
}

// search \^([ATGNC]+): the first '^' followed by a base, its maximal base run
inline bool caret_bases(const std::string &s, std::string &g1) {
    for (size_t i = 0; i + 1 < s.size(); i++)
        if (s[i] == '^' && is_atgnc(s[i + 1])) {
            g1 = s.substr(i + 1, run_end(s, i + 1, is_atgnc) - i - 1);
            return true;
        }
    return false;
}

// search (-\d+)&[ATGC]+$   (group 1)
inline bool del_amp_tail(const std::string &s, std::string &g1) {
    for (size_t i = 0; i < s.size(); i++) {
        if (s[i] != '-') continue;
        size_t j = run_end(s, i + 1, is_digit);
        if (j == i + 1 || j >= s.size() || s[j] != '&') continue;
        size_t e = run_end(s, j + 1, is_atgc);
        if (e == j + 1 || e != s.size()) continue;
        g1 = s.substr(i, j - i);
        return true;
    }
    return false;
}

// ^\+([ATGC]+).*
inline bool ins_lead(const std::string &s, std::string &g1) {
    if (s.size() < 2 || s[0] != '+' || !is_atgc(s[1])) return false;
    g1 = s.substr(1, run_end(s, 1, is_atgc) - 1);
    return true;
}

// search <dup(\d+)>([ATGC]+)$
inline bool dup_tail(const std::string &s, std::string &g1, std::string &g2) {
    for (size_t i = 0; i + 4 <= s.size(); i++) {
        if (s.compare(i, 4, "<dup") != 0) continue;
        size_t d = run_end(s, i + 4, is_digit);
        if (d == i + 4 || d >= s.size() || s[d] != '>') continue;
        size_t e = run_end(s, d + 1, is_atgc);
        if (e == d + 1 || e != s.size()) continue;
        g1 = s.substr(i + 4, d - i - 4);
        g2 = s.substr(d + 1);
        return true;
    }
    return false;
}

// .*&([ATGC]+).*   (greedy: the last '&' followed by a base; its maximal run)
inline bool last_amp_bases(const std::string &s, std::string &g1) {
    for (size_t k = s.size(); k-- > 0;)
        if (s[k] == '&' && k + 1 < s.size() && is_atgc(s[k + 1])) {
            g1 = s.substr(k + 1, run_end(s, k + 1, is_atgc) - k - 1);
            return true;
        }
    return false;
}

// search #([ATGC]+).*   (the first '#' followed by a base; its maximal run)
inline bool hash_bases(const std::string &s, std::string &g1) {
    for (size_t i = 0; i + 1 < s.size(); i++)
        if (s[i] == '#' && is_atgc(s[i + 1])) {
            g1 = s.substr(i + 1, run_end(s, i + 1, is_atgc) - i - 1);
            return true;
        }
    return false;
}

// search \^(\d+)$   (a '^' whose suffix is all digits; its index, or npos)
inline size_t caret_num_tail(const std::string &s) {
    size_t d = s.size();
    while (d > 0 && is_digit(s[d - 1])) d--;
    if (d == s.size() || d == 0 || s[d - 1] != '^') return std::string::npos;
    return d - 1;
}

// search (\+[ATGC]+)&[ATGC]+$   (group 1)
inline bool ins_amp_tail(const std::string &s, std::string &g1) {
    for (size_t i = 0; i + 1 < s.size(); i++) {
        if (s[i] != '+' || !is_atgc(s[i + 1])) continue;
        size_t j = run_end(s, i + 1, is_atgc);
        if (j >= s.size() || s[j] != '&') continue;
        size_t e = run_end(s, j + 1, is_atgc);
        if (e == j + 1 || e != s.size()) continue;
        g1 = s.substr(i, j - i);
        return true;
    }
    return false;
}

// find35match (:1396-1428): the first start (i, j), in the reference's
// order, from which s5 read forwards and s3 read backwards agree over more
// than 8 bases with at most two mismatches (one past the end of s5 counts
// as a mismatch; the reference's substr calls never throw inside these
// bounds).  b5, b3, score = that start and its matched length, or 0, 0, 0.
// The device pass k_find35 runs the same loops.
inline void find35(const std::string &s5, const std::string &s3, int &b5, int &b3, int &score) {
    b5 = b3 = score = 0;
    const int l5 = (int)s5.size(), l3 = (int)s3.size();
    for (int i = 0; i < l5 - 8; i++) {
        for (int j = 1; j < l3 - 8; j++) {
            int nm = 0, n = 0;
            while (n + j <= l3 && i + n <= l5) {
                if (i + n == l5 || s3[l3 - j - n] != s5[i + n]) nm++;
                if (nm > 2) break;
                n++;
            }
            if (n - nm > 8 && nm / (double)n < 0.1 && (n + j >= l3 || i + n >= l5)) {
                b5 = i;
                b3 = j;
                score = n - nm;
                return;
            }
        }
    }
}

}  // namespace keymatch
}  // namespace rv
