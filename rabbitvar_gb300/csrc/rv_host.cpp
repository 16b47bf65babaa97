// Host side of librvgpu that works on strings and on the few keys the local
// realigner touches:
//   * host_realign_mnp: VariationRealigner::adjustMNP
//     (src/VariationRealigner.cpp:334-465) over the device-built maps;
//   * host_format_records: the allele-string part of
//     ToVarsBuilder::collectReferenceVariants (src/ToVarsBuilder.cpp:730-1098,
//     findMSI :614-678, proceedVrefIs* :242-317), Variant::varType /
//     isGoodVar / adjComplex (include/Variant.h:99-248) and
//     print_output_variant_simple (src/modes/simpleMode.cpp:66-142);
//   * host_export_maps: the pileup-boundary maps as text.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "rv_ctx.h"
#include "rv_mirror.h"
#include "rv_pool.h"
#include "rv_records.h"

namespace rv {

using namespace recs;

namespace {

#define HCUDA(call)                                                        \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return RV_ERR_CUDA;                                            \
        }                                                                  \
    } while (0)

constexpr uint32_t FC_PDIFF = 1u << 30, FC_QDIFF = 1u << 31;

}  // namespace

// Measured iteration order of the reference's hash map over soft-clip
// bases (N, A, T, G, C), which decides ties in the consensus.
static int clip_rank(char c) {
    switch (c) {
    case 'N': return 0;
    case 'A': return 1;
    case 'T': return 2;
    case 'G': return 3;
    case 'C': return 4;
    default: return 5 + (unsigned char)c;
    }
}

bool is_mnv(const std::string &k) {
    if (k.size() <= 2 || k[1] != '&') return false;
    auto b = [](char c) { return c == 'A' || c == 'C' || c == 'G' || c == 'T'; };
    if (!b(k[0])) return false;
    for (size_t i = 2; i < k.size(); i++)
        if (!b(k[i])) return false;
    return true;
}


// findconseq: include/VariationUtils.h:403-509, over the per-offset base
// counts sorted by (offset, clip_rank); sets `used` where the reference marks
// a low-complexity consensus as used
std::string consensus_of(const std::vector<NtCount> &nt, int agg_cnt, bool &used) {
    int nts = 0;
    for (size_t i = 0; i < nt.size(); i++)
        if (i == 0 || nt[i].idx != nt[i - 1].idx) nts++;
    int total = 0, match = 0;
    std::string seqq;
    bool flag = false;
    for (size_t i = 0; i < nt.size();) {
        size_t j = i;
        while (j < nt.size() && nt[j].idx == nt[i].idx) j++;
        int maxc = 0, tt = 0;
        double maxq = 0;
        char chosen = 0;
        for (size_t k = i; k < j; k++) {
            tt += nt[k].cnt;
            if (nt[k].cnt > maxc || nt[k].q > maxq) {
                maxc = nt[k].cnt;
                chosen = nt[k].ch;
                maxq = nt[k].q;
            }
        }
        if (nt[i].idx == 3 && nts >= 6 && tt / (double)agg_cnt < 0.2 && tt <= 2) break;
        if ((tt - maxc > 2 || maxc <= tt - maxc) && maxc / (double)tt < 0.8) {
            if (flag) break;
            flag = true;
        }
        total += tt;
        match += maxc;
        if (chosen != 0) seqq += chosen;
        i = j;
    }
    const int sl = (int)seqq.size();
    std::string out;
    if (total != 0 && match / (double)total > 0.9 && sl / 1.5 > nts - sl &&
        (sl / (double)nts > 0.8 || nts - sl < 10 || sl > 25))
        out = seqq;
    else
        out = " ";
    if (out.size() > 12) {
        bool a7 = out.compare(1, 7, "AAAAAAA") == 0, t7 = out.compare(1, 7, "TTTTTTT") == 0;
        if (a7 || t7) used = true;
        int len = (int)out.size(), kinds = 0;
        bool low = false;
        for (char b : std::string("ATGC")) {
            int c = (int)std::count(out.begin(), out.end(), b);
            if (c > 0) kinds++;
            if (c / (double)len > 0.75) low = true;
        }
        if (low || kinds < 3) used = true;
    }
    return out;
}

void sort_nt(std::vector<NtCount> &nt) {
    std::sort(nt.begin(), nt.end(), [](const NtCount &a, const NtCount &b) {
        if (a.idx != b.idx) return a.idx < b.idx;
        return clip_rank(a.ch) < clip_rank(b.ch);
    });
}

std::string clip_consensus(HClip &sc) {
    if (!sc.cons.empty()) return sc.cons;
    std::vector<NtCount> nt;
    for (auto &nve : sc.nt)
        for (auto &e : nve.second) nt.push_back({nve.first, e.first, e.second.first, e.second.second});
    sort_nt(nt);
    sc.cons = consensus_of(nt, sc.agg.cnt, sc.used);
    return sc.cons;
}

void add_into(HVar &to, const HVar &v) {  // adjCnt: include/VariationUtils.h:338-352
    to.cnt += v.cnt;
    to.extracnt += v.cnt;
    to.hi += v.hi;
    to.lo += v.lo;
    to.tp += v.tp;
    to.q += v.q;
    to.mq += v.mq;
    to.nm += v.nm;
    to.fwd += v.fwd;
    to.rev += v.rev;
    to.pstd = to.qstd = true;
    to.force_std = true;
    to.dirty = true;
}

static bool matches_ref(const std::string &s, const RefWin &R, int position, int dir) {  // ismatchref, MM = 3
    int mm = 0, n = (int)s.size();
    for (int k = 0; k < n; k++) {
        int p = position + dir * k;
        if (!R.has(p)) return false;
        char c = dir == 1 ? s[k] : s[n - k - 1];
        if (c != R.at(p)) mm++;
    }
    return mm <= 3 && mm / (double)n < 0.15;
}

std::string slot_key(const rv_ctx *ctx, const Slot &s) {
    if (s.klen == 0 || (size_t)s.koff + s.klen > ctx->h_arena.size()) return std::string();
    return std::string((const char *)ctx->h_arena.data() + s.koff, s.klen);
}

rv_status fetch_slots(rv_ctx *ctx, std::vector<Slot> &slots, std::vector<uint32_t> &idx) {
    DevState st = ctx->state();
    unsigned int *d_n = nullptr;
    uint32_t *d_idx = nullptr;
    Slot *d_out = nullptr;
    HCUDA(cudaMalloc((void **)&d_n, 4));
    HCUDA(cudaMemset(d_n, 0, 4));
    HCUDA(cudaMalloc((void **)&d_idx, ctx->hash_cap * 4));
    launch_compact_slots(st, d_idx, d_n, ctx->stream);
    unsigned int n = 0;
    HCUDA(cudaMemcpyAsync(&n, d_n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaStreamSynchronize(ctx->stream));
    idx.resize(n);
    slots.resize(n);
    if (n) {
        HCUDA(cudaMalloc((void **)&d_out, (size_t)n * sizeof(Slot)));
        launch_gather_slots(ctx->d_slots, d_idx, n, d_out, ctx->stream);
        HCUDA(cudaMemcpyAsync(slots.data(), d_out, (size_t)n * sizeof(Slot), cudaMemcpyDeviceToHost, ctx->stream));
        HCUDA(cudaMemcpyAsync(idx.data(), d_idx, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    unsigned long long used = 0;
    HCUDA(cudaMemcpyAsync(&used, ctx->d_counters + 8, 8, cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaStreamSynchronize(ctx->stream));
    used = std::min<unsigned long long>(used, ctx->arena_cap);
    ctx->h_arena.resize(used);
    if (used) HCUDA(cudaMemcpy(ctx->h_arena.data(), ctx->d_arena, used, cudaMemcpyDeviceToHost));
    cudaFree(d_n);
    cudaFree(d_idx);
    if (d_out) cudaFree(d_out);
    return RV_OK;
}

rv_status fetch_cells(rv_ctx *ctx, const std::vector<int64_t> &cells, std::vector<CellView> &out) {
    out.resize(cells.size());
    if (cells.empty()) return RV_OK;
    int64_t *d_c = nullptr;
    CellView *d_v = nullptr;
    HCUDA(cudaMalloc((void **)&d_c, cells.size() * 8));
    HCUDA(cudaMalloc((void **)&d_v, cells.size() * sizeof(CellView)));
    HCUDA(cudaMemcpyAsync(d_c, cells.data(), cells.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    launch_gather_cells(ctx->state(), d_c, (int64_t)cells.size(), d_v, ctx->stream);
    HCUDA(cudaMemcpyAsync(out.data(), d_v, cells.size() * sizeof(CellView), cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(d_c);
    cudaFree(d_v);
    return RV_OK;
}

HVar from_cell(const CellView &v, int b, int64_t cell) {
    HVar h;
    h.fwd = (int)v.fwd[b];
    h.rev = (int)v.rev[b];
    h.cnt = h.fwd + h.rev;
    h.hi = (int)v.hi[b];
    h.lo = h.cnt - h.hi;
    h.tp = (double)(int)v.tp[b];
    h.q = (double)(int)v.q[b];
    h.mq = (double)(int)v.mq[b];
    h.nm = (double)v.nm[b];
    h.pstd = (v.first[b] & FC_PDIFF) != 0;
    h.qstd = (v.first[b] & FC_QDIFF) != 0;
    h.cell = cell;
    h.base = b;
    return h;
}

HVar from_slot(const Slot &s, int64_t slot) {
    HVar h;
    h.fwd = s.fwd;
    h.rev = s.rev;
    h.cnt = s.fwd + s.rev;
    h.hi = s.hi;
    h.lo = s.lo;
    h.extracnt = s.extracnt;
    h.q = s.q_sum;
    if (s.flags & SF_OVR) {
        double d[3];
        memcpy(&d[0], &s.tp_sum, 8);
        memcpy(&d[1], &s.mq_sum, 8);
        memcpy(&d[2], &s.nm_sum, 8);
        h.cnt = s.first_tp;
        h.tp = d[0];
        h.mq = d[1];
        h.nm = d[2];
        h.pstd = (s.flags & SF_PDIFF) != 0;
        h.qstd = (s.flags & SF_QDIFF) != 0;
    } else {
        h.tp = (double)s.tp_sum;
        h.mq = (double)s.mq_sum;
        h.nm = (double)s.nm_sum;
        h.pstd = (s.flags & (SF_PDIFF | SF_FORCE_STD)) != 0;
        h.qstd = (s.flags & (SF_QDIFF | SF_FORCE_STD)) != 0;
    }
    h.erased = (s.flags & SF_ERASED) != 0;
    h.slot = slot;
    return h;
}


// Slots named by a device index list, copied to the host.
rv_status pull_slots(rv_ctx *ctx, unsigned int n, std::vector<Slot> &slots, std::vector<uint32_t> &idx) {
    slots.resize(n);
    idx.resize(n);
    if (!n) return RV_OK;
    rv_status st = ensure(ctx, ctx->d_tmp_slots, ctx->cap_tmp_slots, n);
    if (st) return st;
    launch_gather_slots(ctx->d_slots, ctx->d_tmp_idx, n, ctx->d_tmp_slots, ctx->stream);
    ctx->kernels++;
    HCUDA(cudaMemcpyAsync(slots.data(), ctx->d_tmp_slots, (size_t)n * sizeof(Slot), cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaMemcpyAsync(idx.data(), ctx->d_tmp_idx, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaStreamSynchronize(ctx->stream));
    ctx->io_d2h += (int64_t)n * (int64_t)(sizeof(Slot) + 4);
    return RV_OK;
}

rv_status pull_arena(rv_ctx *ctx) {
    unsigned long long used = 0;
    HCUDA(cudaMemcpyAsync(&used, ctx->d_counters + 8, 8, cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaStreamSynchronize(ctx->stream));
    used = std::min<unsigned long long>(used, ctx->arena_cap);
    ctx->h_arena.resize(used);
    if (used) {
        HCUDA(cudaMemcpyAsync(ctx->h_arena.data(), ctx->d_arena, used, cudaMemcpyDeviceToHost, ctx->stream));
        HCUDA(cudaStreamSynchronize(ctx->stream));
    }
    return RV_OK;
}

rv_status host_realign_mnp(rv_ctx *ctx) {
    rv_status st;
    if ((st = ensure(ctx, ctx->d_tmp_idx, ctx->cap_tmp_idx, (size_t)ctx->hash_cap))) return st;
    size_t one = 0;
    if (!ctx->d_tmp_n) HCUDA(cudaMalloc((void **)&ctx->d_tmp_n, 16));
    (void)one;
    HCUDA(cudaMemsetAsync(ctx->d_tmp_n, 0, 4, ctx->stream));
    DevState ds = ctx->state();
    launch_select_mnv(ds, ctx->d_tmp_idx, ctx->d_tmp_n, ctx->stream);
    ctx->kernels++;
    unsigned int n_mnv = 0;
    HCUDA(cudaMemcpyAsync(&n_mnv, ctx->d_tmp_n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    HCUDA(cudaStreamSynchronize(ctx->stream));
    if (n_mnv == 0) return RV_OK;
    std::vector<Slot> mslots;
    std::vector<uint32_t> midx;
    if ((st = pull_slots(ctx, n_mnv, mslots, midx))) return st;
    if ((st = pull_arena(ctx))) return st;
    struct Mnp { int region, pos; std::string key; int cnt; };
    std::vector<Mnp> mnps;
    for (const Slot &s : mslots) mnps.push_back({s.region, s.pos, slot_key(ctx, s), s.obs});
    // positions whose keys the MNP merge may read or change
    std::set<std::pair<int, int>> need;
    std::set<std::tuple<int, int, int>> need_clip;  // region, pos, side (5 or 3)
    for (const Mnp &m : mnps) {
        int len = (int)m.key.size() - 1;
        for (int k = 0; k < len; k++) need.insert({m.region, m.pos + k});
        need_clip.insert({m.region, m.pos, 3});
        need_clip.insert({m.region, m.pos + len, 5});
    }
    std::set<std::pair<int, int>> all_pos(need.begin(), need.end());
    for (auto &c : need_clip) all_pos.insert({std::get<0>(c), std::get<1>(c)});
    std::vector<int64_t> cells;
    std::vector<std::pair<int, int>> cell_pos;
    for (auto &np : all_pos) {
        const Region &R = ctx->regions[np.first];
        if (np.second < R.clo || np.second > R.chi) continue;
        cells.push_back(R.cell_base + (np.second - R.clo));
        cell_pos.push_back(np);
    }
    std::vector<CellView> cv(cells.size());
    std::vector<Slot> slots;
    std::vector<uint32_t> sidx;
    if (!cells.empty()) {
        if ((st = ensure(ctx, ctx->d_tmp_cells, ctx->cap_tmp_cells, cells.size()))) return st;
        CellView *dv = (CellView *)ctx->d_tmp_views;
        size_t capv = ctx->cap_tmp_views;
        if ((st = ensure(ctx, dv, capv, cells.size()))) return st;
        ctx->d_tmp_views = dv;
        ctx->cap_tmp_views = capv;
        HCUDA(cudaMemcpyAsync(ctx->d_tmp_cells, cells.data(), cells.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
        launch_gather_cells(ds, ctx->d_tmp_cells, (int64_t)cells.size(), dv, ctx->stream);
        ctx->kernels++;
        HCUDA(cudaMemcpyAsync(cv.data(), dv, cells.size() * sizeof(CellView), cudaMemcpyDeviceToHost, ctx->stream));
        HCUDA(cudaMemsetAsync(ctx->d_tmp_n, 0, 4, ctx->stream));
        launch_gather_lists(ds, ctx->d_tmp_cells, (int64_t)cells.size(), ctx->d_tmp_idx, ctx->d_tmp_n,
                            (unsigned int)ctx->cap_tmp_idx, ctx->stream);
        ctx->kernels++;
        unsigned int nl = 0;
        HCUDA(cudaMemcpyAsync(&nl, ctx->d_tmp_n, 4, cudaMemcpyDeviceToHost, ctx->stream));
        HCUDA(cudaStreamSynchronize(ctx->stream));
        if (nl > ctx->cap_tmp_idx) { ctx->err = "realigner gather overflow"; return RV_ERR_CAPACITY; }
        if ((st = pull_slots(ctx, nl, slots, sidx))) return st;
    }
    // mirror of the touched part of the maps
    std::map<std::pair<int, int>, std::map<std::string, HVar>> vars;
    std::map<std::pair<int, int>, int64_t> cell_of_pos;
    for (size_t i = 0; i < cells.size(); i++) {
        cell_of_pos[cell_pos[i]] = cells[i];
        if (!need.count(cell_pos[i])) continue;
        auto &m = vars[cell_pos[i]];
        for (int b = 0; b < 4; b++) {
            bool exist = (cv[i].kflags >> b) & 1, erased = (cv[i].kflags >> (4 + b)) & 1;
            if (exist && !erased) m[std::string(1, kBases[b])] = from_cell(cv[i], b, cells[i]);
        }
    }
    std::map<std::tuple<int, int, int>, HClip> clips;
    for (size_t i = 0; i < slots.size(); i++) {
        const Slot &s = slots[i];
        if (s.kind == KIND_NONINS && need.count({s.region, s.pos}) && !(s.flags & SF_ERASED)) {
            vars[{s.region, s.pos}][slot_key(ctx, s)] = from_slot(s, sidx[i]);
        } else if (s.kind == KIND_SC3 || s.kind == KIND_SC5) {
            auto key = std::make_tuple((int)s.region, (int)s.pos, s.kind == KIND_SC3 ? 3 : 5);
            if (need_clip.count(key)) clips[key].agg = from_slot(s, sidx[i]);
        } else if (s.kind == KIND_SC3_SEQ || s.kind == KIND_SC5_SEQ) {
            auto key = std::make_tuple((int)s.region, (int)s.pos, s.kind == KIND_SC3_SEQ ? 3 : 5);
            if (!need_clip.count(key)) continue;
            std::string k = slot_key(ctx, s);
            if (k.size() != 3) continue;
            int idx = (uint8_t)k[0] | ((uint8_t)k[1] << 8);
            clips[key].nt[idx][k[2]] = {s.obs, s.q_sum};
        }
    }
    // fillAndSortTmp / CMP_tmp (src/VariationRealigner.cpp:44-58, 1362-1386), per region
    std::sort(mnps.begin(), mnps.end(), [](const Mnp &a, const Mnp &b) {
        if (a.region != b.region) return a.region < b.region;
        if (a.cnt != b.cnt) return a.cnt > b.cnt;
        if (a.pos != b.pos) return a.pos < b.pos;
        return a.key.compare(b.key) > 0;
    });
    std::vector<Patch> patches;
    auto add_cov = [&](int region, int pos, int n) {
        auto it = cell_of_pos.find({region, pos});
        if (it == cell_of_pos.end()) return;
        Patch p;
        memset(&p, 0, sizeof p);
        p.type = 3;
        p.target = it->second;
        p.cov_add = n;
        patches.push_back(p);
    };
    for (const Mnp &m : mnps) {
        const Region &Rg = ctx->regions[m.region];
        RefWin R{&ctx->ref_host, Rg.ws, Rg.we, ctx->ref_len};
        auto pit = vars.find({m.region, m.pos});
        if (pit == vars.end() || !pit->second.count(m.key)) continue;
        std::set<std::string> local;
        for (auto &e : pit->second) local.insert(e.first);
        HVar &vref = pit->second.at(m.key);
        std::string mnt = m.key;
        mnt.erase(mnt.find('&'), 1);
        int ml = (int)mnt.size();
        for (int i = 0; i < ml - 1; i++) {
            std::string left = mnt.substr(0, i + 1), right = mnt.substr(i + 1);
            if (left.size() > 1) left.insert(1, "&");
            if (right.size() > 1) right.insert(1, "&");
            if (local.count(left)) {
                HVar &tref = pit->second.at(left);
                if (tref.cnt <= 0) continue;
                if (tref.cnt < vref.cnt && tref.tp / tref.cnt <= i + 1) {
                    add_into(vref, tref);
                    local.erase(left);
                }
            }
            auto rit = vars.find({m.region, m.pos + i + 1});
            if (rit != vars.end()) {
                auto kit = rit->second.find(right);
                if (kit != rit->second.end()) {
                    HVar &tref = kit->second;
                    if (tref.cnt < 0) continue;
                    if (tref.cnt < vref.cnt) {
                        add_into(vref, tref);
                        add_cov(m.region, m.pos, tref.cnt);
                        Patch p;
                        memset(&p, 0, sizeof p);
                        if (tref.slot >= 0) { p.type = 1; p.target = tref.slot; }
                        else { p.type = 2; p.target = tref.cell; p.base = tref.base; }
                        patches.push_back(p);
                        rit->second.erase(kit);
                    }
                }
            }
        }
        auto s3 = clips.find(std::make_tuple(m.region, m.pos, 3));
        if (s3 != clips.end() && !s3->second.used) {
            std::string sq = clip_consensus(s3->second);
            if ((int)sq.size() >= ml && sq.compare(0, ml, mnt) == 0 &&
                ((int)sq.size() == ml || matches_ref(sq.substr(ml), R, m.pos + ml, 1))) {
                add_into(vref, s3->second.agg);
                add_cov(m.region, m.pos, s3->second.agg.cnt);
                s3->second.used = true;
            }
        }
        auto s5 = clips.find(std::make_tuple(m.region, m.pos + ml, 5));
        if (s5 != clips.end() && !s5->second.used) {
            std::string sq = clip_consensus(s5->second);
            if (sq != " " && (int)sq.size() >= ml) {
                std::reverse(sq.begin(), sq.end());
                if (sq.compare(sq.size() - ml, ml, mnt) == 0 &&
                    ((int)sq.size() == ml || matches_ref(sq.substr(0, sq.size() - ml), R, m.pos - 1, -1))) {
                    add_into(vref, s5->second.agg);
                    add_cov(m.region, m.pos, s5->second.agg.cnt);
                    s5->second.used = true;
                }
            }
        }
    }
    for (auto &pe : vars)
        for (auto &ke : pe.second) {
            const HVar &h = ke.second;
            if (!h.dirty || h.slot < 0) continue;
            Patch p;
            memset(&p, 0, sizeof p);
            p.type = 0;
            p.target = h.slot;
            p.fwd = h.fwd;
            p.rev = h.rev;
            p.hi = h.hi;
            p.lo = h.lo;
            p.extracnt = h.extracnt;
            p.tp_sum = (long long)llround(h.tp);
            p.mq_sum = (long long)llround(h.mq);
            p.nm_sum = (long long)llround(h.nm);
            p.q_sum = h.q;
            p.flags_or = h.force_std ? (int)SF_FORCE_STD : 0;
            patches.push_back(p);
        }
    return apply_patches(ctx, patches, std::string());
}

rv_status apply_patches(rv_ctx *ctx, const std::vector<Patch> &patches, const std::string &keys) {
    if (patches.empty()) return RV_OK;
    rv_status st;
    if ((st = ensure(ctx, ctx->d_patches, ctx->cap_patches, patches.size()))) return st;
    const uint8_t *d_keys = nullptr;
    if (!keys.empty()) {
        if ((st = ensure(ctx, ctx->d_patch_keys, ctx->cap_patch_keys, keys.size()))) return st;
        HCUDA(cudaMemcpyAsync(ctx->d_patch_keys, keys.data(), keys.size(), cudaMemcpyHostToDevice, ctx->stream));
        d_keys = ctx->d_patch_keys;
    }
    HCUDA(cudaMemcpyAsync(ctx->d_patches, patches.data(), patches.size() * sizeof(Patch), cudaMemcpyHostToDevice,
                          ctx->stream));
    ctx->io_h2d += (int64_t)(patches.size() * sizeof(Patch) + keys.size());
    launch_apply_patches(ctx->state(), ctx->d_patches, (int64_t)patches.size(), d_keys, ctx->stream);
    ctx->kernels++;
    HCUDA(cudaStreamSynchronize(ctx->stream));
    return RV_OK;
}

// ---------------------------------------------------------------------------
// records
// ---------------------------------------------------------------------------

// Text and numeric records of the candidate positions [g0, g1) of `groups`.
static void format_groups(const rv_ctx *ctx, const std::vector<const CandVar *> &order,
                          const std::vector<std::pair<size_t, size_t>> &groups, size_t g0, size_t g1,
                          const char *sample, const char *gene, std::string &text,
                          std::vector<rv_site_record> &recs, uint8_t *emitted) {
    const rv_params &P = ctx->params;
    const std::string &chr = ctx->chr;
    for (size_t gi = g0; gi < g1; gi++) {
        size_t i = groups[gi].first, j = groups[gi].second;
        const Region &Rg = ctx->regions[order[i]->region];
        RefWin R{&ctx->ref_host, Rg.ws, Rg.we, ctx->ref_len};
        int position = order[i]->pos;
        const CandVar *ref = nullptr;
        std::vector<RecVar> vs;
        vs.reserve(j - i);
        for (size_t k = i; k < j; k++) {
            const CandVar *c = order[k];
            if (c->kind == 0) { ref = c; continue; }
            RecVar v;
            v.c = c;
            if (c->key_len < 0) v.desc = std::string(1, kBases[c->key_off & 3]);
            else v.desc.assign((const char *)ctx->h_arena.data() + c->key_off, c->key_len);
            vs.push_back(std::move(v));
        }
        std::string refdesc = ref ? std::string(1, R.at(position)) : "";
        std::string g1s;
        if (ref && ref->freq >= P.freq) g1s = refdesc;
        else if (!vs.empty()) g1s = vs[0].desc;
        else g1s = refdesc;
        if (starts(g1s, '+')) g1s = "+" + std::to_string(g1s.size() - 1);
        const bool pileup = ctx->dp.do_pileup != 0 && ctx->dp.dataset_min == 0;
        try {
            for (RecVar &v : vs) {
                describe(v, g1s, position, R, P, v.c->pass != 0 || pileup);
                v.sbf = std::string(ref ? std::to_string(ref->bias) : std::string("0")) + ";" + std::to_string(v.c->bias);
            }
        } catch (const NoRef &) {
            // the reference's joinRef throws here; the position keeps the
            // variants described so far (src/ToVarsBuilder.cpp:183-186)
        }
        std::string reg = chr + ":" + std::to_string(Rg.start) + "-" + std::to_string(Rg.end);
        if (ctx->dp.dataset_min > 0) {
            // candidate-set scoring keeps positions the -f gate drops
            // (src/ToVarsBuilder.cpp:170-175): apply it here
            double maxfreq = 0;
            for (RecVar &v : vs) maxfreq = std::max(maxfreq, v.c->freq);
            if (maxfreq <= P.freq) continue;
        }
        // pileup mode, a position without variants: its reference allele
        // (collectReferenceVariants, src/ToVarsBuilder.cpp:1063-1091: no
        // variant reads, genotype ref/ref, no flanks, empty type)
        RecVar refrec;
        if (pileup && vs.empty() && ref) {
            refrec.c = ref;
            refrec.filled = true;
            refrec.startp = refrec.endp = position;
            refrec.refallele = refrec.varallele = refdesc;
            refrec.genotype = refdesc + "/" + refdesc;
            refrec.shift3 = 0;
            refrec.msi = 0;
            refrec.msint = 0;
            refrec.sbf = std::to_string(ref->bias) + ";0";
            refrec.vartype_fixed = true;
            vs.push_back(refrec);
        }
        for (RecVar &v : vs) {
            if (!v.filled || (!v.c->pass && !pileup)) continue;
            const bool ref_only = v.vartype_fixed;
            if (!ref_only) {
                if (v.refallele.find('N') != std::string::npos) continue;
                v.vartype = var_type(v);
                if (!good_var(v, ref, P, v.vartype) && !pileup) continue;
                if (v.vartype == "Complex") adj_complex(v);
            }
            const CandVar &c = *v.c;
            // adjustVariantCounts (src/ToVarsBuilder.cpp:543-566): negative counts print as 0
            const int rfc = std::max(0, c.rfc), rrc = std::max(0, c.rrc);
            const int afwd = ref_only ? 0 : std::max(0, c.fwd), arev = ref_only ? 0 : std::max(0, c.rev);
            auto add = [&](const std::string &x, bool last = false) {
                text += x;
                text += last ? '\n' : '\t';
            };
            auto addi = [&](long long x) { put_int(text, x); text += '\t'; };
            auto addf = [&](double x) { put_f6(text, x); text += '\t'; };
            add(sample);
            add(gene);
            add(chr);
            addi(v.startp);
            addi(v.endp);
            add(v.refallele);
            add(v.varallele);
            addi(c.tpc);
            addi(ref_only ? 0 : c.pc);
            addi(rfc);
            addi(rrc);
            addi(afwd);
            addi(arev);
            add(v.genotype.empty() ? "0" : v.genotype);
            addf(ref_only ? 0.0 : c.freq);
            add(v.sbf);
            addf(c.pmean);
            add(c.pstd ? "1" : "0");
            addf(c.qual);
            add(c.qstd ? "1" : "0");
            if (P.fisher) {
                addf(c.fisher_p);
                addf(c.fisher_ratio);
            }
            addf(c.mq);
            addf(c.qratio);
            addf(c.hifreq);
            addf(c.extrafreq);
            addi(v.shift3);
            addf(v.msi);
            addi(v.msint);
            if (c.nm > 0) addf(c.nm); else add("0");
            addi(c.hicnt);
            addi(c.hicov);
            add(v.leftseq.empty() ? "0" : v.leftseq);
            add(v.rightseq.empty() ? "0" : v.rightseq);
            add(reg);
            add(v.vartype);
            addf(0.0);
            add("0", true);
            rv_site_record r;
            memset(&r, 0, sizeof r);
            r.region = c.region;
            r.position = position;
            r.start = v.startp;
            r.end = v.endp;
            r.total_cov = c.tpc;
            r.var_cov = ref_only ? 0 : c.pc;
            r.ref_fwd = rfc;
            r.ref_rev = rrc;
            r.alt_fwd = afwd;
            r.alt_rev = arev;
            r.freq = ref_only ? 0.0 : c.freq;
            r.pmean = c.pmean;
            r.qual = c.qual;
            r.mapq = c.mq;
            r.qratio = c.qratio;
            r.hifreq = c.hifreq;
            r.extrafreq = c.extrafreq;
            r.msi = v.msi;
            r.nm = c.nm;
            r.pstd = c.pstd;
            r.qstd = c.qstd;
            r.shift3 = v.shift3;
            r.msint = v.msint;
            r.hicnt = c.hicnt;
            r.hicov = c.hicov;
            r.fisher_p = c.fisher_p;
            r.fisher_ratio = c.fisher_ratio;
            recs.push_back(r);
            if (emitted) emitted[v.c - ctx->h_cand.data()] = 1;
        }
    }
}

rv_status host_format_records(rv_ctx *ctx, const char *sample, const char *gene, uint8_t *emitted) {
    std::vector<const CandVar *> order(ctx->h_cand.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = &ctx->h_cand[i];
    std::sort(order.begin(), order.end(), [](const CandVar *a, const CandVar *b) {
        if (a->region != b->region) return a->region < b->region;
        if (a->pos != b->pos) return a->pos < b->pos;
        return a->rank < b->rank;
    });
    std::vector<std::pair<size_t, size_t>> groups;
    for (size_t i = 0; i < order.size();) {
        size_t j = i;
        while (j < order.size() && order[j]->region == order[i]->region && order[j]->pos == order[i]->pos) j++;
        groups.push_back({i, j});
        i = j;
    }
    // candidate positions are independent: split them over host threads
    const int64_t nt = chunks_for((int64_t)groups.size(), 64);
    std::vector<std::string> texts(nt);
    std::vector<std::vector<rv_site_record>> recs(nt);
    parallel_chunks((int64_t)groups.size(), 64, [&](int64_t t, int64_t a, int64_t b) {
        format_groups(ctx, order, groups, (size_t)a, (size_t)b, sample, gene, texts[t], recs[t], emitted);
    });
    ctx->text.clear();
    ctx->h_records.clear();
    for (int t = 0; t < nt; t++) {
        ctx->text += texts[t];
        ctx->h_records.insert(ctx->h_records.end(), recs[t].begin(), recs[t].end());
    }
    ctx->n_records = (int64_t)ctx->h_records.size();
    return RV_OK;
}

// ---------------------------------------------------------------------------
// map export (pileup boundary) in the oracle's line format
// ---------------------------------------------------------------------------
rv_status host_export_maps(rv_ctx *ctx, int region, const char *stages) {
    const Region &Rg = ctx->regions[region];
    std::vector<Slot> slots;
    std::vector<uint32_t> sidx;
    rv_status st = fetch_slots(ctx, slots, sidx);
    if (st) return st;
    std::vector<int64_t> cells;
    for (int p = Rg.clo; p <= Rg.chi; p++) cells.push_back(Rg.cell_base + (p - Rg.clo));
    std::vector<CellView> cv;
    if ((st = fetch_cells(ctx, cells, cv))) return st;
    // max read length of the region
    Region Rd;
    HCUDA(cudaMemcpy(&Rd, ctx->d_regions + region, sizeof(Region), cudaMemcpyDeviceToHost));
    bool realigned = strchr(stages, 'R') != nullptr;
    const char *pfx = realigned ? "R" : "P";
    char buf[640];
    std::string &o = ctx->dump;
    o.clear();
    if (!realigned) {
        snprintf(buf, sizeof buf, "P_ML\t%d\n", Rd.max_read_len);
        o += buf;
    }
    auto line = [&](const char *tag, int pos, const std::string &key, const HVar &v) {
        snprintf(buf, sizeof buf, "%s\t%d\t%s\t%d\t%d\t%d\t%.17g\t%.17g\t%.17g\t%.17g\t%d\t%d\t%d\t%d\t%d\t%.17g\t%d\n", tag,
                 pos, key.c_str(), v.cnt, v.fwd, v.rev, v.tp, v.q, v.mq, v.nm, v.lo, v.hi, (int)v.pstd, (int)v.qstd, 0,
                 0.0, v.extracnt);
        o += buf;
    };
    std::map<int, std::map<std::string, HVar>> nonins, ins;
    std::map<int, std::pair<HVar, std::map<int, std::map<char, HVar>>>> sc[2];
    std::map<int, std::map<std::string, int>> cnt_i, cnt_d, cnt_m;
    std::map<int, int> cov;
    for (size_t i = 0; i < cells.size(); i++) {
        int p = Rg.clo + (int)i;
        for (int b = 0; b < 4; b++) {
            bool exist = (cv[i].kflags >> b) & 1, erased = (cv[i].kflags >> (4 + b)) & 1;
            if (exist && !(realigned && erased)) nonins[p][std::string(1, kBases[b])] = from_cell(cv[i], b, cells[i]);
        }
        if (cv[i].cov) cov[p] = (int)cv[i].cov;
    }
    for (size_t i = 0; i < slots.size(); i++) {
        const Slot &s = slots[i];
        if (s.region != region) continue;
        std::string k = slot_key(ctx, s);
        HVar h = from_slot(s, sidx[i]);
        if (realigned && h.erased) continue;
        switch (s.kind) {
        case KIND_NONINS:
            nonins[s.pos][k] = h;
            if (is_mnv(k)) cnt_m[s.pos][k] = s.obs;
            if (starts(k, '-')) cnt_d[s.pos][k] = s.obs;
            break;
        case KIND_INS:
            ins[s.pos][k] = h;
            cnt_i[s.pos][k] = s.obs;
            break;
        case KIND_SC5: case KIND_SC3:
            sc[s.kind == KIND_SC3][s.pos].first = h;
            break;
        case KIND_SC5_SEQ: case KIND_SC3_SEQ: {
            if (k.size() != 3) break;
            int idx = (uint8_t)k[0] | ((uint8_t)k[1] << 8);
            HVar hv = h;
            hv.extracnt = s.obs;  // nt count rides along
            sc[s.kind == KIND_SC3_SEQ][s.pos].second[idx][k[2]] = hv;
            break;
        }
        default: break;
        }
    }
    std::string tN = std::string(pfx) + "N", tI = std::string(pfx) + "I";
    for (auto &pe : nonins)
        for (auto &ke : pe.second) line(tN.c_str(), pe.first, ke.first, ke.second);
    for (auto &pe : ins)
        for (auto &ke : pe.second) line(tI.c_str(), pe.first, ke.first, ke.second);
    for (auto &ce : cov) {
        snprintf(buf, sizeof buf, "%sC\t%d\t%d\n", pfx, ce.first, ce.second);
        o += buf;
    }
    if (!realigned) {
        for (int side = 0; side < 2; side++) {
            const char *tag = side == 0 ? "PS5" : "PS3";
            for (auto &se : sc[side]) {
                line(tag, se.first, "*", se.second.first);
                for (auto &ie : se.second.second)
                    for (auto &che : ie.second) {
                        HVar v = che.second;
                        int ntc = v.extracnt;
                        v.extracnt = 0;
                        char key[64];
                        snprintf(key, sizeof key, "%d:%c:%d", ie.first, che.first, ntc);
                        line(tag, se.first, key, v);
                    }
            }
        }
        auto cnts = [&](const char *tg, std::map<int, std::map<std::string, int>> &m) {
            for (auto &pe : m)
                for (auto &ke : pe.second) {
                    snprintf(buf, sizeof buf, "%s\t%d\t%s\t%d\n", tg, pe.first, ke.first.c_str(), ke.second);
                    o += buf;
                }
        };
        cnts("PCI", cnt_i);
        cnts("PCD", cnt_d);
        cnts("PMN", cnt_m);
    }
    return RV_OK;
}

}  // namespace rv
