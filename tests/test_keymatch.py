"""The realigner's hand-written key matchers (rabbitvar_gb300/csrc/rv_keymatch.h)
against what they replace, on the CPU: each matcher against the std::regex
search of the pattern the reference uses (src/VariationRealigner.cpp
:489-1117, include/patterns.h) on random keys of the allele-key alphabet.
The find35match restatement the realigner's device pass mirrors is checked
by the GPU tests (the -k 1 golden cases) against the reference's output."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

DRIVER = r'''
#include <cstdio>
#include <random>
#include <regex>
#include <string>
#include "rv_keymatch.h"
using namespace rv::keymatch;
using std::string;

int main() {
    std::mt19937_64 rng(12345);
    const string alpha = "ACGTNACGTACGT-+&#^<>0123456789dupinv";
    const std::regex r_inv("^-\\d+\\^([ATGNC]+)<...\\d+>([ATGNC]+)$"), r_rest("^-\\d+(.*)"),
        r_caret("\\^([ATGNC]+)"), r_dtail("(-\\d+)&[ATGC]+$"), r_ins1("^\\+([ATGC]+).*"),
        r_dup("<dup(\\d+)>([ATGC]+)$"), r_extra(".*&([ATGC]+).*"), r_compm("#([ATGC]+).*"),
        r_newdel("\\^(\\d+)$"), r_itail("(\\+[ATGC]+)&[ATGC]+$");
    const char *pre[] = {"-", "+", "-12", "+AC", "-3^", "-4^ACG<inv12>", "+TT&", "-2&", "+A#", "<dup3>", ""};
    long bad = 0, n = 0;
    for (int it = 0; it < 200000; it++) {
        string s = pre[rng() % 11];
        int len = (int)(rng() % 14);
        for (int k = 0; k < len; k++) s += alpha[rng() % alpha.size()];
        std::smatch m;
        auto chk = [&](bool mine, bool want, const string &x, const string &y) {
            n++;
            if (mine != want || (want && x != y)) {
                if (bad < 10) printf("MISMATCH %s\n", s.c_str());
                bad++;
            }
        };
        { string g1, g2; bool w = std::regex_search(s, m, r_inv); bool me = inv(s, g1, g2);
          chk(me, w, g1 + "|" + g2, w ? m.str(1) + "|" + m.str(2) : ""); }
        { string g; bool w = std::regex_search(s, m, r_rest); chk(del_rest(s, g), w, g, w ? m.str(1) : ""); }
        { string g; bool w = std::regex_search(s, m, r_caret); chk(caret_bases(s, g), w, g, w ? m.str(1) : ""); }
        { string g; bool w = std::regex_search(s, m, r_dtail); chk(del_amp_tail(s, g), w, g, w ? m.str(1) : ""); }
        { string g; bool w = std::regex_search(s, m, r_ins1); chk(ins_lead(s, g), w, g, w ? m.str(1) : ""); }
        { string g1, g2; bool w = std::regex_search(s, m, r_dup); bool me = dup_tail(s, g1, g2);
          chk(me, w, g1 + "|" + g2, w ? m.str(1) + "|" + m.str(2) : ""); }
        { string g; bool w = std::regex_search(s, m, r_extra); chk(last_amp_bases(s, g), w, g, w ? m.str(1) : ""); }
        { string g; bool w = std::regex_search(s, m, r_compm); chk(hash_bases(s, g), w, g, w ? m.str(1) : ""); }
        { bool w = std::regex_search(s, m, r_newdel); size_t p = caret_num_tail(s);
          chk(p != string::npos, w, p != string::npos ? s.substr(p + 1) : "", w ? m.str(1) : ""); }
        { string g; bool w = std::regex_search(s, m, r_itail); chk(ins_amp_tail(s, g), w, g, w ? m.str(1) : ""); }
    }
    printf("%ld %ld\n", n, bad);
    return 0;
}
'''


def test_key_matchers_match_the_regex_searches(tmp_path):
    src = tmp_path / "keymatch_driver.cpp"
    exe = tmp_path / "keymatch_driver"
    src.write_text(DRIVER)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "rabbitvar_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    n, bad = map(int, out[-2].split())
    assert bad == 0, out[:10]
    assert n == 2_000_000
