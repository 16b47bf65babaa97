// Allele strings and hard filter of one called variant, shared by the simple
// and somatic record writers: the allele-string part of
// ToVarsBuilder::collectReferenceVariants (src/ToVarsBuilder.cpp:730-1098,
// findMSI :614-678, proceedVrefIs* :242-317) and Variant::varType /
// isGoodVar / adjComplex (include/Variant.h:99-248).
#pragma once

#include <charconv>
#include <cmath>
#include <cstdio>
#include <string>

#include "rv_ctx.h"

namespace rv {
namespace recs {

extern const char kBases[4];

// The reference window of a region: positions ws..we (1-based) of the contig.
struct RefWin {
    const std::string *ref;
    int ws, we, len;
    bool has(int p) const { return p >= ws && p <= we; }
    char at(int p) const { return has(p) ? (*ref)[p - 1] : 0; }
};

struct Msi { double msi; int shift3; std::string unit; };
struct NoRef {};

struct RecVar {
    const CandVar *c;
    std::string desc;
    std::string sbf;
    int startp = 0, endp = 0, shift3 = 0, msint = 0;
    double msi = 0;
    std::string leftseq, rightseq, genotype, refallele, varallele, vartype;
    bool filled = false;
    bool vartype_fixed = false;   // pileup mode's reference-allele record (type "")
};

Msi find_msi(const std::string &t1, const std::string &t2, const std::string &left);

// collectReferenceVariants for one variant; throws NoRef where the reference's
// joinRef would throw.  With full == false only what can affect later variants
// of the position is done (the genotype-1 edits and the window checks).
void describe(RecVar &v, std::string &g1, int position, const RefWin &R, const rv_params &P, bool full);
std::string var_type(const RecVar &v);
// Variant::isGoodVar; an empty `type` means the variant's own varType()
bool good_var(const RecVar &v, const CandVar *ref, const rv_params &P, const std::string &type);
void adj_complex(RecVar &v);
// printf("%f") and printf("%lld") appended to o: std::to_chars gives the
// same correctly rounded digits as printf; non-finite values go through
// snprintf for its exact spelling
inline void put_f6(std::string &o, double d) {
    char b[352];
    if (!std::isfinite(d)) {
        snprintf(b, sizeof b, "%f", d);
        o += b;
        return;
    }
    auto r = std::to_chars(b, b + sizeof b, d, std::chars_format::fixed, 6);
    if (r.ec != std::errc()) {
        snprintf(b, sizeof b, "%f", d);
        o += b;
        return;
    }
    o.append(b, r.ptr);
}
inline void put_int(std::string &o, long long x) {
    char b[24];
    auto r = std::to_chars(b, b + sizeof b, x);
    o.append(b, r.ptr);
}
inline bool starts(const std::string &s, char c) { return !s.empty() && s[0] == c; }

}  // namespace recs
}  // namespace rv
