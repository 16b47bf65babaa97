// Somatic mode on the host: the tumor/normal classification and the
// 63-column records of SomaticMode (src/modes/somaticMode.cpp).
//
// Both samples come from their own context, scored with the same region
// list.  rv_score_pair has already made every position that can produce a
// record available in both samples: positions where either sample has an
// allele passing the numeric part of isGoodVar, with all alleles of the
// position (and its reference allele) as CandVars.  What is left here is
// string work and the per-position label logic; the three Fisher tests of
// every record run on the device in one batch once the tables are known
// (Variant::isNoise can change the counts of the normal allele first).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "rv_ctx.h"
#include "rv_pool.h"
#include "rv_records.h"

namespace rv {

using namespace recs;

namespace {

// One allele of one sample at one position: a mutable copy of its numbers
// (isNoise and the somatic writer change them) and its description.
struct SVar {
    CandVar c;
    RecVar r;
    const RecVar &rec() {
        r.c = &c;
        return r;
    }
};

struct SPos {
    int region = 0, pos = 0;
    bool has_ref = false;
    SVar ref;
    std::vector<SVar> vars;  // CMP_VARI order
};

std::string key_of(const rv_ctx *ctx, const CandVar &c) {
    if (c.key_len < 0) return std::string(1, kBases[c.key_off & 3]);
    return std::string((const char *)ctx->h_arena.data() + c.key_off, (size_t)c.key_len);
}

// The Vars of one position after collectVarsAtPosition and
// collectReferenceVariants (src/ToVarsBuilder.cpp:327-346, 730-1098).
void build_position(const rv_ctx *ctx, const CandVar *const *g, size_t n, SPos &sp) {
    const rv_params &P = ctx->params;
    sp.region = g[0]->region;
    sp.pos = g[0]->pos;
    const Region &Rg = ctx->regions[sp.region];
    RefWin R{&ctx->ref_host, Rg.ws, Rg.we, ctx->ref_len};
    for (size_t i = 0; i < n; i++) {
        SVar v;
        v.c = *g[i];
        v.r.desc = key_of(ctx, v.c);
        if (v.c.kind == 0) {
            sp.ref = v;
            sp.has_ref = true;
        } else {
            sp.vars.push_back(std::move(v));
        }
    }
    const int position = sp.pos;
    const std::string refdesc = sp.has_ref ? sp.ref.r.desc : std::string();
    if (!sp.vars.empty()) {
        std::string g1;
        if (sp.has_ref && sp.ref.c.freq >= P.freq) g1 = refdesc;
        else g1 = sp.vars[0].r.desc;
        if (!g1.empty() && g1[0] == '+') g1 = "+" + std::to_string(g1.size() - 1);
        size_t done = 0;
        try {
            for (; done < sp.vars.size(); done++) {
                SVar &v = sp.vars[done];
                v.r.c = &v.c;
                describe(v.r, g1, position, R, P, true);
                v.r.sbf = (sp.has_ref ? std::to_string(sp.ref.c.bias) : std::string("0")) + ";" +
                          std::to_string(v.c.bias);
                // adjustVariantCounts (src/ToVarsBuilder.cpp:543-566)
                v.c.rfc = std::max(0, v.c.rfc);
                v.c.rrc = std::max(0, v.c.rrc);
                v.c.fwd = std::max(0, v.c.fwd);
                v.c.rev = std::max(0, v.c.rev);
            }
        } catch (const NoRef &) {
            // joinRef threw: this and the later alleles keep what createVariant
            // gave them (src/ToVarsBuilder.cpp:183-186)
        }
        for (size_t k = done; k < sp.vars.size(); k++) {
            SVar &v = sp.vars[k];
            v.r = RecVar();
            v.r.desc = key_of(ctx, v.c);
            v.r.sbf = std::to_string(v.c.bias);
            v.c.tpc = 0;
            v.c.rfc = v.c.rrc = 0;
        }
        if (sp.has_ref) {  // the reference allele keeps createVariant's fields only
            sp.ref.r.sbf = std::to_string(sp.ref.c.bias);
            sp.ref.c.tpc = 0;
            sp.ref.c.rfc = sp.ref.c.rrc = 0;
        }
    } else if (sp.has_ref) {  // only reference reads: :1063-1088
        SVar &v = sp.ref;
        v.c.pc = 0;
        v.c.freq = 0;
        v.c.fwd = v.c.rev = 0;
        v.r.sbf = std::to_string(v.c.bias) + ";0";
        v.r.startp = v.r.endp = position;
        std::string rb = R.has(position) ? std::string(1, R.at(position)) : std::string();
        v.r.refallele = rb;
        v.r.varallele = rb;
        v.r.genotype = rb + "/" + rb;
        v.r.filled = true;
    }
}

// a `new Variant()` the writer fills with a few fields
SVar blank() {
    SVar v;
    memset(&v.c, 0, sizeof v.c);
    v.r.sbf = "0";
    return v;
}

struct Rec {
    int region = 0;
    bool has_beg = false, has_end = false, has_t = false, has_n = false;
    SVar beg, end, t, n;
    std::string label;
};

struct Classifier {
    const rv_params &P;
    std::vector<Rec> &out;

    static SVar *find(SPos &sp, const std::string &desc) {
        for (SVar &v : sp.vars)
            if (v.r.desc == desc) return &v;
        return nullptr;
    }
    static const CandVar *refc(SPos &sp) { return sp.has_ref ? &sp.ref.c : nullptr; }

    bool good(SVar &v, SPos &sp, const std::string &type) { return good_var(v.rec(), refc(sp), P, type); }

    void emit(int region, const SVar *beg, const SVar *end, const SVar *t, const SVar *n, const char *label) {
        Rec r;
        r.region = region;
        if (beg) { r.has_beg = true; r.beg = *beg; }
        if (end) { r.has_end = true; r.end = *end; }
        if (t) { r.has_t = true; r.t = *t; }
        if (n) { r.has_n = true; r.n = *n; }
        r.label = label;
        out.push_back(std::move(r));
    }

    // Variant::isNoise (include/Variant.h:75-94)
    bool is_noise(SVar &v) {
        const double q = v.c.qual;
        if (((q < 4.5 || (q < 12 && !v.c.qstd)) && v.c.pc <= 3) ||
            (q < P.goodq && v.c.freq < 2 * P.lofreq && v.c.pc <= 1)) {
            v.c.tpc -= v.c.pc;
            v.c.pc = 0;
            v.c.fwd = v.c.rev = 0;
            v.c.freq = 0;
            v.c.hifreq = 0;
            return true;
        }
        return false;
    }

    // determinateType (somaticMode.cpp:608-633)
    const char *determinate(SPos &v2, SVar &std_v, SVar &cmp) {
        const char *type;
        if (good(cmp, v2, std_v.r.vartype)) {
            if (std_v.c.freq > 1 - P.lofreq && cmp.c.freq < 0.8 && cmp.c.freq > 0.2) type = "LikelyLOH";
            else if (cmp.c.freq < P.lofreq || cmp.c.pc <= 1) type = "LikelySomatic";
            else type = "Germline";
        } else {
            if (cmp.c.freq < P.lofreq || cmp.c.pc <= 1) type = "LikelySomatic";
            else type = "AFDiff";
        }
        if (is_noise(cmp) && std_v.r.vartype == "SNV") type = "StrongSomatic";
        return type;
    }

    // callingForOneSample (:360-380) for a tumor position the normal lacks
    void one_sample(SPos &v1) {
        for (SVar &v : v1.vars) {
            v.r.vartype = var_type(v.rec());
            if (!good(v, v1, v.r.vartype)) continue;
            if (v.r.vartype == "Complex") adj_complex(v.r);
            emit(v1.region, &v, &v, &v, nullptr, "SampleSpecific");
        }
    }

    // printVariationsFromFirstSample (:405-530)
    void first_sample(SPos &v1, SPos &v2) {
        size_t k = 0;
        while (k < v1.vars.size() && good(v1.vars[k], v1, v1.vars[k].r.vartype)) {
            SVar &vref = v1.vars[k];
            vref.r.vartype = var_type(vref.rec());
            if (vref.r.vartype == "Complex") adj_complex(vref.r);
            SVar *v2nt = find(v2, vref.r.desc);
            if (v2nt) {
                const char *type = determinate(v2, vref, *v2nt);
                emit(v1.region, &vref, v2nt, &vref, v2nt, type);
            } else {
                // combineAnalysis (:639-735) runs only for descriptions with a
                // '<', which this pipeline never produces
                SVar shown = blank();
                const SVar *vfp;
                if (!v2.vars.empty()) {
                    const SVar &v2r = v2.vars[0];
                    shown.c.tpc = v2r.c.tpc;
                    shown.c.rfc = v2r.c.rfc;
                    shown.c.rrc = v2r.c.rrc;
                    vfp = &shown;
                } else {
                    vfp = v2.has_ref ? &v2.ref : nullptr;
                }
                emit(v1.region, &vref, &vref, &vref, vfp, "StrongSomatic");
            }
            k++;
        }
        if (k > 0 || v2.vars.empty()) return;
        for (SVar &v2var : v2.vars) {
            v2var.r.vartype = var_type(v2var.rec());
            if (!good(v2var, v2, v2var.r.vartype)) continue;
            SVar *v1nt = find(v1, v2var.r.desc);
            if (v1nt) {
                const char *type = v1nt->c.freq < P.lofreq ? "LikelyLOH" : "Germline";
                if (v2var.r.vartype == "Complex") adj_complex(v1nt->r);
                v1nt->r.vartype = var_type(v1nt->rec());
                emit(v1.region, v1nt, &v2var, v1nt, &v2var, type);
            } else {
                const SVar *v1var = v1.vars.empty() ? nullptr : &v1.vars[0];
                SVar shown = blank();
                shown.c.tpc = v1var ? v1var->c.tpc : 0;
                shown.c.rfc = v1.has_ref ? v1.ref.c.fwd : 0;
                shown.c.rrc = v1.has_ref ? v1.ref.c.rev : 0;
                shown.r.genotype = v1var ? v1var->r.genotype
                                         : (v1.has_ref ? v1.ref.r.desc + "/" + v1.ref.r.desc : std::string("N/N"));
                if (v2var.r.vartype == "Complex") adj_complex(v2var.r);
                emit(v1.region, &v2var, &v2var, &shown, &v2var, "StrongLOH");
            }
        }
    }

    // printVariationsFromSecondSample (:537-600): the tumor has no variant here
    void second_sample(SPos &v1, SPos &v2) {
        for (SVar &v2var : v2.vars) {
            v2var.r.vartype = var_type(v2var.rec());
            if (!good(v2var, v2, v2var.r.vartype)) continue;
            const SVar *vfp = v1.has_ref ? &v1.ref : nullptr;
            if (v2var.r.vartype == "Complex") adj_complex(v2var.r);
            emit(v1.region, &v2var, &v2var, vfp, &v2var, "StrongLOH");
        }
    }
};

// CandVars of a context grouped by (region, position), CMP_VARI order within
void group(const rv_ctx *ctx, std::vector<const CandVar *> &order, std::vector<std::pair<size_t, size_t>> &groups) {
    order.resize(ctx->h_cand.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = &ctx->h_cand[i];
    std::sort(order.begin(), order.end(), [](const CandVar *a, const CandVar *b) {
        if (a->region != b->region) return a->region < b->region;
        if (a->pos != b->pos) return a->pos < b->pos;
        return a->rank < b->rank;
    });
    groups.clear();
    for (size_t i = 0; i < order.size();) {
        size_t j = i;
        while (j < order.size() && order[j]->region == order[i]->region && order[j]->pos == order[i]->pos) j++;
        groups.push_back({i, j});
        i = j;
    }
}

void put_stats(std::string &o, const Rec &r, const SVar *v) {
    if (!v) {
        for (int i = 0; i < 18; i++) o += "0\t";
        return;
    }
    auto I = [&](long long x) { put_int(o, x); o += '\t'; };
    auto F = [&](double x) { put_f6(o, x); o += '\t'; };
    const CandVar &c = v->c;
    I(c.tpc);
    I(c.pc);
    I(c.rfc);
    I(c.rrc);
    I(c.fwd);
    I(c.rev);
    // the normal column prints the tumor allele's genotype (:218)
    o += v->r.genotype.empty() ? std::string("0") : r.t.r.genotype;
    o += '\t';
    F(c.freq);
    o += v->r.sbf;
    o += '\t';
    F(c.pmean);
    o += c.pstd ? "1\t" : "0\t";
    F(c.qual);
    o += c.qstd ? "1\t" : "0\t";
    F(c.mq);
    F(c.qratio);
    F(c.hifreq);
    F(c.extrafreq);
    F(c.nm);
}

// put_fisher_ext_and_odds (:130-149): the p-value, then a float32 log ratio
// with +0.5 pseudocounts
void put_fisher(std::string &o, double p, const int32_t *t) {
    put_f6(o, p);
    o += '\t';
    const float a = t[0] + 0.5, bb = t[1] + 0.5, c = t[2] + 0.5, d = t[3] + 0.5;
    const float ad = a * d, bc = bb * c;
    const float ratio = std::log(ad / bc + bc / ad);
    put_f6(o, (double)ratio);
    o += '\t';
}

}  // namespace

rv_status host_format_somatic(rv_ctx *t, rv_ctx *n, const char *sample, const char *gene) {
    PhaseTimer pt("format_somatic");
    const rv_params &P = t->params;
    std::vector<const CandVar *> to, no;
    std::vector<std::pair<size_t, size_t>> tg, ng;
    parallel_for(2, [&](int64_t k) {
        if (k == 0) group(t, to, tg);
        else group(n, no, ng);
    });
    pt.lap("group");
    // positions are independent: classify them on host threads, keeping order
    const int64_t kMinPos = 64;
    std::vector<std::vector<Rec>> part(chunks_for((int64_t)tg.size(), kMinPos));
    parallel_chunks((int64_t)tg.size(), kMinPos, [&](int64_t k, int64_t a, int64_t b) {
        Classifier C{P, part[k]};
        for (size_t gi = (size_t)a; gi < (size_t)b; gi++) {
            SPos v1;
            build_position(t, &to[tg[gi].first], tg[gi].second - tg[gi].first, v1);
            auto key = std::make_pair(v1.region, v1.pos);
            auto it = std::lower_bound(ng.begin(), ng.end(), key, [&](const std::pair<size_t, size_t> &g,
                                                                      const std::pair<int, int> &k2) {
                return std::make_pair(no[g.first]->region, no[g.first]->pos) < k2;
            });
            bool has2 = it != ng.end() && no[it->first]->region == v1.region && no[it->first]->pos == v1.pos;
            if (!has2) {
                if (!v1.vars.empty()) C.one_sample(v1);
                continue;
            }
            SPos v2;
            build_position(n, &no[it->first], it->second - it->first, v2);
            if (v1.vars.empty() && v2.vars.empty()) continue;
            if (!v1.vars.empty()) C.first_sample(v1, v2);
            else C.second_sample(v1, v2);
        }
    });
    pt.lap("classify");
    std::vector<Rec> recs;
    size_t nrec = 0;
    for (auto &pv : part) nrec += pv.size();
    recs.reserve(nrec);
    for (auto &pv : part)
        for (auto &r : pv) recs.push_back(std::move(r));
    // the three Fisher tables of every record, tested on the device
    std::vector<int32_t> tab;
    std::vector<double> p2;
    if (P.fisher && !recs.empty()) {
        tab.resize(recs.size() * 12);
        for (size_t i = 0; i < recs.size(); i++) {
            const Rec &r = recs[i];
            int32_t *x = &tab[12 * i];
            const CandVar *tc = r.has_t ? &r.t.c : nullptr, *nc = r.has_n ? &r.n.c : nullptr;
            int32_t z[4] = {0, 0, 0, 0};
            const int32_t a[4] = {tc ? tc->rfc : 0, tc ? tc->rrc : 0, tc ? tc->fwd : 0, tc ? tc->rev : 0};
            const int32_t b[4] = {nc ? nc->rfc : 0, nc ? nc->rrc : 0, nc ? nc->fwd : 0, nc ? nc->rev : 0};
            int t_tot = tc ? tc->tpc : 0, t_var = tc ? tc->pc : 0, n_tot = nc ? nc->tpc : 0, n_var = nc ? nc->pc : 0;
            const int32_t c[4] = {t_var, std::max(0, t_tot - t_var), n_var, std::max(0, n_tot - n_var)};
            memcpy(x, tc ? a : z, 16);
            memcpy(x + 4, nc ? b : z, 16);
            memcpy(x + 8, c, 16);
        }
        p2.resize(recs.size() * 3);
        rv_status s = device_fisher(t, tab.data(), (int64_t)recs.size() * 3, p2.data());
        if (s) return s;
    }
    pt.lap("fisher");
    const Region *regs = t->regions.data();
    std::vector<std::string> texts(chunks_for((int64_t)recs.size(), 64));
    parallel_chunks((int64_t)recs.size(), 64, [&](int64_t k, int64_t i0, int64_t i1) {
    std::string &o = texts[k];
    o.reserve((size_t)(i1 - i0) * 640);
    char b[96];
    for (size_t i = (size_t)i0; i < (size_t)i1; i++) {
        const Rec &r = recs[i];
        o += sample;
        o += '\t';
        o += gene;
        o += '\t';
        o += t->chr;
        o += '\t';
        if (r.has_beg) {
            put_int(o, r.beg.r.startp);
            o += '\t';
            put_int(o, r.beg.r.endp);
            o += '\t';
            o += r.beg.r.refallele + "\t" + r.beg.r.varallele + "\t";
        } else {
            o += "0\t0\t0\t0\t";
        }
        put_stats(o, r, r.has_t ? &r.t : nullptr);
        if (P.fisher) {
            if (r.has_t) put_fisher(o, p2[3 * i], &tab[12 * i]);
            else o += "0\t0\t";
        }
        put_stats(o, r, r.has_n ? &r.n : nullptr);
        if (P.fisher) {
            if (r.has_n) put_fisher(o, p2[3 * i + 1], &tab[12 * i + 4]);
            else o += "0\t0\t";
        }
        if (r.has_end) {
            put_int(o, r.end.r.shift3);
            o += '\t';
            put_f6(o, r.end.r.msi);
            o += '\t';
            put_int(o, r.end.r.msint);
            o += '\t';
            o += (r.end.r.leftseq.empty() ? std::string("0") : r.end.r.leftseq) + "\t";
            o += (r.end.r.rightseq.empty() ? std::string("0") : r.end.r.rightseq) + "\t";
        } else {
            o += "\t\t\t\t\t";
        }
        snprintf(b, sizeof b, "%s:%d-%d\t", t->chr.c_str(), regs[r.region].start, regs[r.region].end);
        o += b;
        o += r.label + "\t";
        o += (r.has_beg ? r.beg.r.vartype : std::string()) + "\t";
        o += r.has_t ? "0.000000\t0\t" : "0\t0\t";  // duprate, sv
        o += r.has_n ? "0.000000\t0\t" : "0\t0\t";
        if (P.fisher) {
            put_fisher(o, p2[3 * i + 2], &tab[12 * i + 8]);
            double tvaf = r.has_t ? r.t.c.freq : 0, nvaf = r.has_n ? r.n.c.freq : 0;
            put_f6(o, std::log(std::max(tvaf, 0.0001) / std::max(nvaf, 0.0001)));
            o += '\t';
            int t_var = r.has_t ? r.t.c.pc : 0, n_var = r.has_n ? r.n.c.pc : 0;
            put_f6(o, std::log((static_cast<float>(t_var) + 0.5) / (static_cast<float>(n_var) + 0.5)));
            o += '\t';
        }
        o += '\n';
    }
    });
    t->text.clear();
    size_t tl = 0;
    for (auto &x : texts) tl += x.size();
    t->text.reserve(tl);
    for (auto &x : texts) t->text += x;
    t->n_records = (int64_t)recs.size();
    t->h_records.clear();
    pt.lap("text");
    if (pt.on) fprintf(stderr, "trace format_somatic sizes cand_t %zu cand_n %zu positions %zu records %zu\n",
                       t->h_cand.size(), n->h_cand.size(), tg.size(), recs.size());
    return RV_OK;
}

}  // namespace rv
