// The local realigner of -k 1 over the device-built maps, on the host:
// VariationRealigner::adjustMNP (src/VariationRealigner.cpp:334-465) followed
// by realignIndels (:467-1360: realigndel :489-775, realignins :785-1114,
// realignlgins30 :1119-1350, with findMM3/findMM5 :1857-1984, ismatch
// :1507-1546, adjRefCnt :1753-1787, adjRefFactor :1794-1822, noPassingReads
// :1447-1505, find35match :1396-1428).
//
// Each region runs over a lazily filled mirror of its maps: a position's
// keys are read from the fetched cells and slots the first time the
// realigner touches it, and a snapshot is kept.  At the end the mirror is
// diffed against the snapshots and the differences go back to the device as
// patches: realigned statistics (SF_OVR slots; a single-base key that
// changes moves from its cell to a slot), erased keys, new keys, removed
// position entries and coverage additions.  The score kernel reads the
// patched maps.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <deque>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rv_keymatch.h"
#include "rv_mirror.h"
#include "rv_pool.h"

namespace rv {

namespace {

#define HCUDA(call)                                                        \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return RV_ERR_CUDA;                                            \
        }                                                                  \
    } while (0)

using std::string;

// Reference window of a region with the insert-on-lookup behaviour of the
// reference's map: operator[] on a position outside the window stores base 0
// there, and the position counts as present afterwards.
struct PRef {
    const string *ref = nullptr;
    int ws = 1, we = 0;
    std::set<int> phantom;
    bool has(int p) const { return (p >= ws && p <= we) || phantom.count(p); }
    char at(int p) const { return (p >= ws && p <= we) ? (*ref)[p - 1] : 0; }
    char idx(int p) {
        if (p >= ws && p <= we) return (*ref)[p - 1];
        phantom.insert(p);
        return 0;
    }
    bool has_eq(char c, int p) const { return has(p) && at(p) == c; }
    bool has_ne(char c, int p) const { return has(p) && at(p) != c; }
};

struct RefFail {};     // joinRef's .at() on a missing position
struct OutOfRange {};  // std::out_of_range from substr

string join_ref(const PRef &R, int from, int to) {  // joinRef: include/VariationUtils.h:356-362
    string s;
    for (int i = from; i <= to; i++) {
        if (!R.has(i)) throw RefFail();
        s += R.at(i);
    }
    return s;
}

// vc_substr (include/util.h:27-57): negative indices count from the end; the
// length test there is unsigned, so too negative an index throws
string vsub(const string &s, int idx) {
    size_t b = idx >= 0 ? (size_t)idx : s.size() + (size_t)(long long)idx;
    if (b > s.size()) throw OutOfRange();
    return s.substr(b);
}
string vsub(const string &s, int begin, int len) {
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
string drop_hash_caret(const string &s) {
    string o;
    for (char c : s)
        if (c != '#' && c != '^') o += c;
    return o;
}
void replace_first(string &s, const string &a, const string &b) {
    size_t p = s.find(a);
    if (p != string::npos) s.replace(p, a.size(), b);
}
bool low_complexity(const string &seq) {  // islowcomplexseq: include/VariationUtils.h:366-395
    int len = (int)seq.size();
    if (len == 0) return true;
    int kinds = 0;
    for (char b : string("ATGC")) {
        int c = (int)std::count(seq.begin(), seq.end(), b);
        if (c > 0) kinds++;
        if (c / (double)len > 0.75) return true;
    }
    return kinds < 3;
}

void clamp_counts(HVar &r) {  // correctCnt: include/VariationUtils.h:263-280
    if (r.cnt < 0) r.cnt = 0;
    if (r.hi < 0) r.hi = 0;
    if (r.lo < 0) r.lo = 0;
    if (r.tp < 0) r.tp = 0;
    if (r.q < 0) r.q = 0;
    if (r.mq < 0) r.mq = 0;
    if (r.rev < 0) r.rev = 0;
    if (r.fwd < 0) r.fwd = 0;
}
// adjCnt(varToAdd, variant, referenceVar): include/VariationUtils.h:291-317
void add_sub(HVar &to, const HVar &v, HVar *ref) {
    add_into(to, v);
    if (!ref) return;
    ref->cnt -= v.cnt;
    ref->hi -= v.hi;
    ref->lo -= v.lo;
    ref->tp -= v.tp;
    ref->q -= v.q;
    ref->mq -= v.mq;
    ref->nm -= v.nm;
    ref->rev -= v.rev;
    ref->fwd -= v.fwd;
    clamp_counts(*ref);
}

bool same_stats(const HVar &a, const HVar &b) {
    return a.cnt == b.cnt && a.fwd == b.fwd && a.rev == b.rev && a.hi == b.hi && a.lo == b.lo &&
           a.extracnt == b.extracnt && a.tp == b.tp && a.q == b.q && a.mq == b.mq && a.nm == b.nm &&
           a.pstd == b.pstd && a.qstd == b.qstd;
}

// ---------------------------------------------------------------------------
// batch-wide mirror (pinned host copies, read-only while the regions run):
// the cells, and every cell's keys flattened in list order
// ---------------------------------------------------------------------------
struct Mirror {
    rv_ctx *ctx = nullptr;
    const uint32_t *fwd, *rev, *hi, *tp, *q, *mq, *first;
    const int32_t *nm;
    const uint8_t *kflags;
    const uint32_t *off = nullptr;   // n_cells + 1
    const Slot *slots = nullptr;     // off[n_cells]
    const uint32_t *sidx = nullptr;  // hash slot index of each
    const uint32_t *cmeta = nullptr; // per clip aggregate: its device-computed consensus (k_clip_consensus)
    const uint8_t *cons = nullptr;
    std::vector<Region> regions;     // device copies (max_read_len)

    string key(uint32_t i) const { return slot_key(ctx, slots[i]); }
    HVar cell_var(int64_t c, int b) const {
        HVar h;
        const int64_t g = 4 * c + b;
        h.fwd = (int)fwd[g];
        h.rev = (int)rev[g];
        h.cnt = h.fwd + h.rev;
        h.hi = (int)hi[g];
        h.lo = h.cnt - h.hi;
        h.tp = (double)(int)tp[g];
        h.q = (double)(int)q[g];
        h.mq = (double)(int)mq[g];
        h.nm = (double)nm[g];
        h.pstd = (first[g] & (1u << 30)) != 0;
        h.qstd = (first[g] & (1u << 31)) != 0;
        h.cell = c;
        h.base = b;
        return h;
    }
};

// One position of nonInsertionVariants or insertionVariants.
struct PosMap {
    bool present = false;
    std::map<string, HVar> keys;
};

// ---------------------------------------------------------------------------
// one region
// ---------------------------------------------------------------------------
struct RegionRealigner {
    Mirror &mir;
    rv_ctx *ctx;
    const rv_params &P;
    int region;
    Region Rg;
    int max_rl;
    int chr_len;
    PRef R;
    std::map<int, PosMap> nonins, ins, nonins0, ins0;
    std::map<int, int> cov_add;
    struct Clip {
        HClip c;
        int64_t cell = -1;  // the clip's per-offset counts are in this cell's list
        int64_t agg = -1;   // list index of the aggregate
        int seq_kind = 0;
        bool loaded = false;
    };
    // The soft-clip aggregates by position (the reference's position-keyed
    // maps, filled in position order by load_lists): an index per position
    // of the region's cell range into a deque (stable references), and the
    // filled positions in ascending order for the walks over all of them.
    struct ClipMap {
        int lo = 0;
        std::vector<int32_t> idx;  // per position from lo: index into clips, -1 = absent
        std::deque<Clip> clips;
        std::vector<int> pos;      // position of each clip, ascending
        void init(int clo, int chi) {
            lo = clo;
            idx.assign((size_t)std::max(0, chi - clo + 1), -1);
            clips.clear();
            pos.clear();
        }
        Clip &insert(int p) {
            int32_t &k = idx[(size_t)(p - lo)];
            if (k < 0) {
                k = (int32_t)clips.size();
                clips.emplace_back();
                pos.push_back(p);
            }
            return clips[(size_t)k];
        }
        Clip *find(int p) {
            const int64_t i = (int64_t)p - lo;
            if (i < 0 || i >= (int64_t)idx.size() || idx[(size_t)i] < 0) return nullptr;
            return &clips[(size_t)idx[(size_t)i]];
        }
    };
    ClipMap sc5, sc3;

    RegionRealigner(Mirror &m, rv_ctx *c, int r)
        : mir(m), ctx(c), P(c->params), region(r), Rg(m.regions[r]), max_rl(m.regions[r].max_read_len),
          chr_len(c->ref_len) {
        R.ref = &ctx->ref_host;
        R.ws = Rg.ws;
        R.we = Rg.we;
    }

    bool in_cells(int p) const { return p >= Rg.clo && p <= Rg.chi; }
    int64_t cell_of(int p) const { return Rg.cell_base + (p - Rg.clo); }

    PosMap &N(int p) {
        auto it = nonins.find(p);
        if (it != nonins.end()) return it->second;
        PosMap &m = nonins[p];
        if (in_cells(p)) {
            const int64_t c = cell_of(p);
            const int exist = mir.kflags[c] & 15, erased = (mir.kflags[c] >> 4) & 15;
            if (exist) m.present = true;
            for (int b = 0; b < 4; b++)
                if (((exist & ~erased) >> b) & 1) m.keys[string(1, "ACGT"[b])] = mir.cell_var(c, b);
            for (uint32_t i = mir.off[c]; i < mir.off[c + 1]; i++) {
                if (mir.slots[i].kind != KIND_NONINS) continue;
                m.present = true;
                HVar h = from_slot(mir.slots[i], mir.sidx[i]);
                if (!h.erased) m.keys[mir.key(i)] = h;
            }
        }
        nonins0[p] = m;
        return m;
    }
    PosMap &I(int p) {
        auto it = ins.find(p);
        if (it != ins.end()) return it->second;
        PosMap &m = ins[p];
        if (in_cells(p)) {
            const int64_t c = cell_of(p);
            for (uint32_t i = mir.off[c]; i < mir.off[c + 1]; i++) {
                if (mir.slots[i].kind != KIND_INS) continue;
                m.present = true;
                HVar h = from_slot(mir.slots[i], mir.sidx[i]);
                if (!h.erased) m.keys[mir.key(i)] = h;
            }
        }
        ins0[p] = m;
        return m;
    }
    bool has_key(int p, const string &k) {
        PosMap &m = N(p);
        return m.present && m.keys.count(k);
    }
    // map operator[] on position and key
    HVar &nget(int p, const string &k) {
        PosMap &m = N(p);
        m.present = true;
        return m.keys[k];
    }
    HVar &iget(int p, const string &k) {
        PosMap &m = I(p);
        m.present = true;
        return m.keys[k];
    }
    // erase a key; drop the position entry when it becomes empty
    void nerase_drop(int p, const string &k) {
        PosMap &m = N(p);
        m.present = true;  // operator[] before erase
        m.keys.erase(k);
        if (m.keys.empty()) m.present = false;
    }
    // getVariationMaybe: include/VariationUtils.h:218-239
    HVar *maybe(int p, char base) {
        if (base == 0) return nullptr;
        PosMap &m = N(p);
        if (!m.present) return nullptr;
        auto j = m.keys.find(string(1, base));
        return j == m.keys.end() ? nullptr : &j->second;
    }
    // nonInsertionVariants.count(p) && [p].count(k)
    HVar *nfind(int p, const string &k) {
        PosMap &m = N(p);
        if (!m.present) return nullptr;
        auto j = m.keys.find(k);
        return j == m.keys.end() ? nullptr : &j->second;
    }

    Clip *clip(ClipMap &sc, int p) { return sc.find(p); }
    double *prof = nullptr;  // per-region phase times (trace)
    const string &consensus(Clip &k) {
        if (!k.loaded && k.agg >= 0 && (mir.cmeta[k.agg] >> 31)) {
            // computed on the device; the low-complexity mark applies now, at
            // the first use, as in the reference
            k.loaded = true;
            const uint32_t m = mir.cmeta[k.agg];
            k.c.cons.assign((const char *)mir.cons + mir.off[k.cell] + ((m >> 16) & 0x3FFFu), m & 0xFFFFu);
            if (m & (1u << 30)) k.c.used = true;
        }
        if (!k.loaded) {
            auto t0 = std::chrono::steady_clock::now();
            k.loaded = true;
            std::vector<NtCount> nt;
            if (k.cell >= 0)
                for (uint32_t i = mir.off[k.cell]; i < mir.off[k.cell + 1]; i++) {
                    const Slot &s = mir.slots[i];
                    if (s.kind != k.seq_kind || s.klen != 3 || (size_t)s.koff + 3 > ctx->h_arena.size()) continue;
                    const uint8_t *kb = ctx->h_arena.data() + s.koff;
                    nt.push_back({kb[0] | (kb[1] << 8), (char)kb[2], s.obs, s.q_sum});
                }
            sort_nt(nt);
            k.c.cons = consensus_of(nt, k.c.agg.cnt, k.c.used);
            if (prof) prof[6] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        return k.c.cons;
    }
    // The consensus string of a clip without the side effect consensus() has
    // at its first use (the low-complexity mark); the string itself does not
    // depend on when it is computed.
    string peek_consensus(Clip &k) {
        if (k.loaded) return k.c.cons;
        if (k.agg >= 0 && (mir.cmeta[k.agg] >> 31)) {
            const uint32_t m = mir.cmeta[k.agg];
            return string((const char *)mir.cons + mir.off[k.cell] + ((m >> 16) & 0x3FFFu), m & 0xFFFFu);
        }
        std::vector<NtCount> nt;
        if (k.cell >= 0)
            for (uint32_t i = mir.off[k.cell]; i < mir.off[k.cell + 1]; i++) {
                const Slot &s = mir.slots[i];
                if (s.kind != k.seq_kind || s.klen != 3 || (size_t)s.koff + 3 > ctx->h_arena.size()) continue;
                const uint8_t *kb = ctx->h_arena.data() + s.koff;
                nt.push_back({kb[0] | (kb[1] << 8), (char)kb[2], s.obs, s.q_sum});
            }
        sort_nt(nt);
        bool unused = false;
        return consensus_of(nt, k.c.agg.cnt, unused);
    }
    void add_cov(int p, int n) { cov_add[p] += n; }

    // one pass over the region's key lists: the soft-clip aggregates, and
    // the MNV / deletion / insertion counts the passes iterate
    // (VariationData's mnp, positionToDeletionCount, positionToInsertionCount)
    void load_lists(std::map<int, std::map<string, int>> &mnp, std::map<int, std::map<string, int>> &delcnt,
                    std::map<int, std::map<string, int>> &inscnt) {
        const uint8_t *arena = ctx->h_arena.data();
        const size_t arena_n = ctx->h_arena.size();
        sc5.init(Rg.clo, Rg.chi);
        sc3.init(Rg.clo, Rg.chi);
        for (int p = Rg.clo; p <= Rg.chi; p++) {
            const int64_t c = cell_of(p);
            const uint32_t e = mir.off[c + 1];
            for (uint32_t i = mir.off[c]; i < e; i++) {
                const Slot &s = mir.slots[i];
                if (s.kind == KIND_SC5 || s.kind == KIND_SC3) {
                    Clip &k = (s.kind == KIND_SC3 ? sc3 : sc5).insert(p);
                    k.c.agg = from_slot(s, mir.sidx[i]);
                    k.cell = c;
                    k.agg = i;
                    k.seq_kind = s.kind == KIND_SC3 ? KIND_SC3_SEQ : KIND_SC5_SEQ;
                    continue;
                }
                if ((s.kind != KIND_NONINS && s.kind != KIND_INS) || s.obs <= 0) continue;
                if (s.kind == KIND_NONINS) {
                    // only MNV ("X&Y...") and deletion keys are counted
                    if (s.klen == 0 || (size_t)s.koff + s.klen > arena_n) continue;
                    const uint8_t k0 = arena[s.koff];
                    if (k0 != '-' && !(s.klen > 2 && arena[s.koff + 1] == '&')) continue;
                }
                string k = mir.key(i);
                if (s.kind == KIND_INS) inscnt[p][k] = s.obs;
                else if (is_mnv(k)) mnp[p][k] = s.obs;
                else if (!k.empty() && k[0] == '-') delcnt[p][k] = s.obs;
            }
        }
    }

    // ------------------------------------------------------------------
    // adjustMNP (src/VariationRealigner.cpp:334-465)
    // ------------------------------------------------------------------
    void adjust_mnp(const std::map<int, std::map<string, int>> &mnp) {
        struct T { int pos; string key; int cnt; };
        std::vector<T> tmp;
        for (auto &pe : mnp)
            for (auto &ke : pe.second) tmp.push_back({pe.first, ke.first, ke.second});
        std::sort(tmp.begin(), tmp.end(), [](const T &a, const T &b) {
            if (a.cnt != b.cnt) return a.cnt > b.cnt;
            if (a.pos != b.pos) return a.pos < b.pos;
            return a.key.compare(b.key) > 0;
        });
        for (const T &t : tmp) {
            const int position = t.pos;
            const string &vn = t.key;
            PosMap &pm = N(position);
            if (!pm.present) continue;
            std::set<string> local;  // keys of the by-value copy the reference iterates
            for (auto &e : pm.keys) local.insert(e.first);
            if (!local.count(vn)) continue;
            HVar &vref = pm.keys.at(vn);
            string mnt = vn;
            size_t amp = mnt.find('&');
            if (amp != string::npos) mnt.erase(amp, 1);
            const int ml = (int)mnt.size();
            for (int i = 0; i < ml - 1; i++) {
                string left = mnt.substr(0, i + 1), right = mnt.substr(i + 1);
                if (left.size() > 1) left.insert(1, "&");
                if (right.size() > 1) right.insert(1, "&");
                if (local.count(left)) {
                    HVar &tref = pm.keys.at(left);
                    if (tref.cnt <= 0) continue;
                    if (tref.cnt < vref.cnt && tref.tp / tref.cnt <= i + 1) {
                        add_into(vref, tref);
                        local.erase(left);
                    }
                }
                PosMap &rm = N(position + i + 1);
                if (rm.present) {
                    auto kit = rm.keys.find(right);
                    if (kit != rm.keys.end()) {
                        HVar &tref = kit->second;
                        if (tref.cnt < 0) continue;
                        if (tref.cnt < vref.cnt) {
                            add_into(vref, tref);
                            add_cov(position, tref.cnt);
                            rm.keys.erase(kit);
                        }
                    }
                }
            }
            Clip *s3 = clip(sc3, position);
            if (s3 && !s3->c.used) {
                string sq = consensus(*s3);
                if (sq.compare(0, ml, mnt) == 0 && (int)sq.size() >= ml &&
                    ((int)sq.size() == ml || ismatchref(sq.substr(ml), position + ml, 1))) {
                    add_into(pm.keys[vn], s3->c.agg);
                    add_cov(position, s3->c.agg.cnt);
                    s3->c.used = true;
                }
            }
            Clip *s5 = clip(sc5, position + ml);
            if (s5 && !s5->c.used) {
                string sq = consensus(*s5);
                if (sq != " " && (int)sq.size() >= ml) {
                    std::reverse(sq.begin(), sq.end());
                    if (sq.substr(sq.size() - ml, ml) == mnt &&
                        ((int)sq.size() == ml || ismatchref(sq.substr(0, sq.size() - ml), position - 1, -1))) {
                        add_into(pm.keys[vn], s5->c.agg);
                        add_cov(position, s5->c.agg.cnt);
                        s5->c.used = true;
                    }
                }
            }
        }
    }
    // ismatchref: src/VariationRealigner.cpp:2004-2024 (MM = 3)
    bool ismatchref(const string &sq, int position, int dir) {
        int mm = 0, len = (int)sq.size();
        for (int n = 0; n < len; n++) {
            if (!R.has(position + dir * n)) return false;
            char c = dir == 1 ? sq[n] : sq[len - n - 1];
            if (c != R.idx(position + dir * n)) mm++;
        }
        return mm <= 3 && mm / (double)len < 0.15;
    }

    // ------------------------------------------------------------------
    // indel passes
    // ------------------------------------------------------------------
    struct Mism { string seq; int pos; int end; };
    struct MmResult { std::vector<Mism> mm; std::vector<int> scp; int nm = 0, misp = 0; string misnt; };

    // findMM5 (:1857-1916)
    MmResult find_mm5(int position, const string &wupseq) {
        string seq = drop_hash_caret(wupseq);
        MmResult r;
        int n = 0, mcnt = 0;
        string str;
        while (R.has_ne(char_at(seq, -1 - n), position - n) && mcnt < 3) {
            str.insert(0, 1, char_at(seq, -1 - n));
            r.mm.push_back({str, position - n, 5});
            n++;
            mcnt++;
        }
        r.scp.push_back(position + 1);
        if (str.size() == 1) {
            while (R.has_eq(char_at(seq, -1 - n), position - n)) {
                n++;
                if (n != 0) r.nm++;
            }
            if (r.nm > 1) {
                // the reference's second scan (-1 - n - 1 - n2 >= 0) never runs
                r.scp.push_back(position - n);
                if (Clip *k = clip(sc5, position - n)) k->c.used = true;
            }
        }
        return r;
    }
    // findMM3 (:1919-1984)
    MmResult find_mm3(int p, const string &sanpseq) {
        string seq = drop_hash_caret(sanpseq);
        MmResult r;
        int n = 0, mcnt = 0, len = (int)seq.size();
        string str;
        while (n < len && R.has(p + n) && R.at(p + n) == seq[n]) n++;
        r.scp.push_back(p + n);
        const int tbp = p + n;
        while (mcnt <= 3 && n < len && R.idx(p + n) != seq[n]) {
            str += seq[n];
            r.mm.push_back({str, tbp, 3});
            n++;
            mcnt++;
        }
        if (str.size() == 1) {
            while (n < len && R.has_eq(seq[n], p + n)) {
                n++;
                if (n != 0) r.nm++;
            }
            if (r.nm > 1) {
                int n2 = 0;
                while (n + n2 + 1 < len && R.has_eq(seq[n + n2 + 1], p + n + 1 + n2)) n2++;
                if (n2 > 2 && n + n2 + 1 < len) {
                    r.scp.push_back(p + n + n2);
                    r.misp = p + n;
                    r.misnt = string(1, seq[n]);
                    if (Clip *k = clip(sc3, p + n + n2)) k->c.used = true;
                    r.nm += n2;
                } else {
                    r.scp.push_back(p + n);
                    if (Clip *k = clip(sc3, p + n)) k->c.used = true;
                }
            }
        }
        return r;
    }
    // ismatch (:1507-1546), MM = 3
    static bool ismatch(const string &seq1, const string &seq2_in, int dir) {
        string seq2 = drop_hash_caret(seq2_in);
        int mm = 0;
        const int l2 = (int)seq2.size();
        for (int n = 0; n < (int)seq1.size() && n < l2; n++)
            if (seq1[n] != seq2[dir == 1 ? n : l2 - 1 - n]) mm++;
        return mm <= 3 && mm / (double)seq1.size() < 0.15;
    }
    // adjRefCnt (:1753-1787)
    static void adj_ref_cnt(const HVar &tv, HVar *ref, int len) {
        if (!ref) return;
        double f = tv.tp != 0 ? (tv.tp / (double)tv.cnt - len + 1) / (tv.tp / (double)tv.cnt) : 0;
        if (f < 0) return;
        if (f > 1) f = 1;
        ref->cnt -= (int)(f * tv.cnt);
        ref->hi -= (int)(f * tv.hi);
        ref->lo -= (int)(f * tv.lo);
        ref->tp -= f * tv.tp;
        ref->q -= f * tv.q;
        ref->mq -= f * tv.mq;
        ref->nm -= f * tv.nm;
        ref->rev -= (int)(f * tv.rev);
        ref->fwd -= (int)(f * tv.fwd);
        clamp_counts(*ref);
    }
    // adjRefFactor (:1794-1822)
    static void adj_ref_factor(HVar *ref, double f) {
        if (!ref) return;
        if (f > 1) f = 1;
        if (f < -1) return;
        int old = ref->cnt;
        ref->cnt -= (int)(f * ref->cnt);
        ref->hi -= (int)(f * ref->hi);
        ref->lo -= (int)(f * ref->lo);
        double fc = old != 0 ? std::abs(ref->cnt - old) / (double)old : 1;
        ref->tp -= ref->tp * f * fc;
        ref->q -= ref->q * f * fc;
        ref->mq -= ref->mq * f * fc;
        ref->nm -= f * ref->nm;
        ref->fwd -= (int)(f * ref->fwd);
        ref->rev -= (int)(f * ref->rev);
        clamp_counts(*ref);
    }
    // noPassingReads (:1447-1505): the batch's records over start..end, unfiltered
    bool no_passing_reads(int start, int end) {
        const rv_ctx *c = ctx;
        int cnt = 0;
        const uint32_t dlen = ((uint32_t)(end - start) << 4) | 2u;
        const int64_t n = c->hb_n;
        const int32_t *pos = c->hb_pos;
        int64_t lo = std::lower_bound(pos, pos + n, start - 1 - 4096) - pos;
        for (int64_t i = lo; i < n && pos[i] < end; i++) {
            const uint32_t *cg = c->hb_cigar + c->hb_cigoff[i];
            int span = 0, aligned = 0;
            bool has_d = false;
            for (int k = 0; k < c->hb_ncig[i]; k++) {
                int o = cg[k] & 15;
                if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) span += (int)(cg[k] >> 4);
                if (o == 0 || o == 2) aligned += (int)(cg[k] >> 4);
                if (cg[k] == dlen) has_d = true;
            }
            int endpos = ((c->hb_flag[i] & 4) || span == 0) ? pos[i] + 1 : pos[i] + span;
            if (endpos <= start - 1) continue;
            if (has_d) continue;
            int rs0 = pos[i] + 1, re0 = rs0 + aligned;
            if (re0 > end + 2 && rs0 < start - 2) cnt++;
        }
        return cnt <= 0;
    }

    struct Cand { int pos; string key; int cnt; };
    static std::vector<Cand> sorted(const std::map<int, std::map<string, int>> &ch) {  // CMP_tmp (:1362-1386)
        std::vector<Cand> t;
        for (auto &pe : ch)
            for (auto &ke : pe.second) t.push_back({pe.first, ke.first, ke.second});
        std::sort(t.begin(), t.end(), [](const Cand &a, const Cand &b) {
            if (a.cnt != b.cnt) return a.cnt > b.cnt;
            if (a.pos != b.pos) return a.pos < b.pos;
            return a.key.compare(b.key) > 0;
        });
        return t;
    }

    // the leading number of a key ("-12..." -> 12), or -1
    static int lead_num(const string &s, size_t from) {
        size_t i = from;
        int v = 0;
        bool any = false;
        while (i < s.size() && s[i] >= '0' && s[i] <= '9') { v = v * 10 + (s[i] - '0'); i++; any = true; }
        return any ? v : -1;
    }
    static bool all_bases(const string &s, const char *alphabet) {
        if (s.empty()) return false;
        for (char c : s)
            if (!strchr(alphabet, c)) return false;
        return true;
    }
    // "^<digits>" at the end of the key: the digits, or -1
    static int tail_caret_num(const string &s) {
        size_t i = s.size();
        while (i > 0 && s[i - 1] >= '0' && s[i - 1] <= '9') i--;
        if (i == s.size() || i == 0 || s[i - 1] != '^') return -1;
        return atoi(s.c_str() + i);
    }

    // realigndel (:489-775)
    void realigndel(bool with_reads, const std::map<int, std::map<string, int>> &dcnt_map) {
        std::vector<Cand> tmp = sorted(dcnt_map);
        for (const Cand &tpl : tmp) {
            try {
                const int p = tpl.pos;
                const string &vn = tpl.key;
                const int dcnt = tpl.cnt;
                HVar &vref = nget(p, vn);
                int dellen = 0;
                if (vn.size() > 1 && vn[0] == '-') {
                    int d = lead_num(vn, 1);
                    if (d >= 0) dellen = d;
                }
                int tc = tail_caret_num(vn);
                if (tc >= 0) dellen += tc;
                string extrains, extra, inv5, inv3, rest;
                // ^-\d+\^([ATGNC]+)<...\d+>([ATGNC]+)$, else ^-\d+(.*) and \^([ATGNC]+)
                if (keymatch::inv(vn, inv5, inv3)) {
                } else if (keymatch::del_rest(vn, rest)) {
                    for (char c : rest)
                        if (c != '^' && c != '&' && c != '#') extra += c;
                    keymatch::caret_bases(vn, extrains);
                }
                const int wustart = p - 200 > 1 ? p - 200 : 1;
                string wupseq = join_ref(R, wustart, p - 1) + extra;
                if (!inv3.empty()) wupseq = inv3;
                const int sanend = p + 200 > chr_len ? chr_len : p + 200;
                const int off = dellen + (int)extra.size() - (int)extrains.size();
                string sanpseq = extra + join_ref(R, p + off, sanend);
                if (!inv5.empty()) sanpseq = inv5;
                MmResult r3 = find_mm3(p, sanpseq);
                MmResult r5 = find_mm5(p + off - 1, wupseq);
                std::vector<Mism> mmm = r3.mm;
                mmm.insert(mmm.end(), r5.mm.begin(), r5.mm.end());
                for (Mism &mi : mmm) {
                    string mm = mi.seq;
                    if (mm.size() > 1) mm.insert(1, 1, '&');
                    const int mp = mi.pos, me = mi.end;
                    if (!has_key(mp, mm)) continue;
                    HVar &tv = N(mp).keys.at(mm);
                    if (tv.cnt == 0) continue;
                    if (tv.q / tv.cnt < P.goodq) continue;
                    if (tv.tp / tv.cnt > (me == 3 ? r3.nm + 4 : r5.nm + 4)) continue;
                    if (tv.cnt >= dcnt + dellen || tv.cnt / dcnt >= 8) continue;
                    if (mp > p && me == 5) {
                        double f = tv.tp != 0 ? (mp - p) / (tv.tp / (double)tv.cnt) : 1;
                        if (f > 1) f = 1;
                        add_cov(p, (int)(tv.cnt * f));
                        char b = R.idx(p);
                        adj_ref_cnt(tv, maybe(p, b), dellen);
                    }
                    HVar *lref = nullptr;
                    if (mp > p && me == 3 && N(p).present) {
                        char b = R.idx(p);
                        lref = nfind(p, string(1, b));
                    }
                    if (lref) add_sub(vref, tv, lref);
                    else add_into(vref, tv);
                    nerase_drop(mp, mm);
                }
                if (r3.misp != 0 && r3.mm.size() == 1 && has_key(r3.misp, r3.misnt) &&
                    N(r3.misp).keys.at(r3.misnt).cnt < dcnt)
                    N(r3.misp).keys.erase(r3.misnt);
                if (r5.misp != 0 && r5.mm.size() == 1 && has_key(r5.misp, r5.misnt) &&
                    N(r5.misp).keys.at(r5.misnt).cnt < dcnt)
                    N(r5.misp).keys.erase(r5.misnt);
                for (int sc5pp : r5.scp) {
                    Clip *k = clip(sc5, sc5pp);
                    if (!k || k->c.used) continue;
                    string seq = consensus(*k);
                    if (dcnt <= 2 && k->c.agg.cnt / dcnt > 5) continue;
                    if (seq != " " && ismatch(seq, wupseq, -1)) {
                        if (sc5pp > p) add_cov(p, k->c.agg.cnt);
                        add_into(vref, k->c.agg);
                        k->c.used = true;
                    }
                }
                for (int sc3pp : r3.scp) {
                    Clip *k = clip(sc3, sc3pp);
                    if (!k || k->c.used) continue;
                    string seq = consensus(*k);
                    if (dcnt <= 2 && k->c.agg.cnt / dcnt > 5) continue;
                    if (seq != " " && ismatch(seq, vsub(sanpseq, sc3pp - p), 1)) {
                        if (sc3pp <= p) add_cov(p, k->c.agg.cnt);
                        HVar *lref = nullptr;
                        if (sc3pp > p) {
                            char b = R.idx(p);
                            lref = maybe(p, b);
                        }
                        add_sub(vref, k->c.agg, lref);
                        k->c.used = true;
                    }
                }
                const int pe = p + off;
                char b = R.idx(p);
                HVar *h = maybe(p, b);
                if (with_reads && pe - p >= 5 && pe - p < max_rl - 10 && h && h->cnt != 0 &&
                    vref.cnt > 2 * h->cnt * (1 - (pe - p) / (double)max_rl) && no_passing_reads(p, pe))
                    add_sub(vref, *h, h);
            } catch (const RefFail &) {
            } catch (const OutOfRange &) {
            }
        }
        for (int i = (int)tmp.size() - 1; i > 0; i--) {
            const int p = tmp[i].pos;
            const string &vn = tmp[i].key;
            if (!has_key(p, vn)) continue;
            HVar &vref = N(p).keys.at(vn);
            string tn;
            if (keymatch::del_amp_tail(vn, tn)) {  // (-\d+)&[ATGC]+$
                auto &keys = N(p).keys;
                auto t = keys.find(tn);
                if (t != keys.end() && vref.cnt < t->second.cnt) {
                    add_into(t->second, vref);
                    keys.erase(vn);
                }
            }
        }
    }

    // realignins (:785-1114)
    void realignins(const std::map<int, std::map<string, int>> &icnt_map) {
        std::vector<Cand> tmp = sorted(icnt_map);
        for (const Cand &tpl : tmp) {
            try {
                const int position = tpl.pos;
                const string &vn = tpl.key;
                const int icnt = tpl.cnt;
                string insert1;
                if (!keymatch::ins_lead(vn, insert1)) continue;  // ^\+([ATGC]+).*
                string ins3, dupn;
                int inslen = (int)insert1.size();
                if (keymatch::dup_tail(vn, dupn, ins3))  // <dup(\d+)>([ATGC]+)$
                    inslen += atoi(dupn.c_str()) + (int)ins3.size();
                string extra, compm;
                keymatch::last_amp_bases(vn, extra);  // .*&([ATGC]+).*
                keymatch::hash_bases(vn, compm);      // #([ATGC]+).*
                int newdel = 0;
                const size_t nd = keymatch::caret_num_tail(vn);  // \^(\d+)$
                if (nd != string::npos) newdel = atoi(vn.c_str() + nd + 1);
                string tn = vn;
                if (!tn.empty() && tn[0] == '+') tn.erase(0, 1);
                replace_first(tn, "&", "");
                replace_first(tn, "#", "");
                // the first \^\d+$, then the first \^, removed
                const size_t cn = keymatch::caret_num_tail(tn);
                if (cn != string::npos) tn.erase(cn);
                const size_t c1 = tn.find('^');
                if (c1 != string::npos) tn.erase(c1, 1);
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
                    r3 = find_mm3(p3 + 1, sanpseq);
                } else {
                    sanpseq = tn + join_ref(R, position + (int)extra.size() + 1 + (int)compm.size() + newdel, sanend);
                    r3 = find_mm3(position + 1, sanpseq);
                }
                MmResult r5 = find_mm5(position + (int)extra.size() + (int)compm.size() + newdel, wupseq);
                std::vector<Mism> mmm = r3.mm;
                mmm.insert(mmm.end(), r5.mm.begin(), r5.mm.end());
                HVar &vref = iget(position, vn);
                for (Mism &mi : mmm) {
                    string mb = mi.seq;
                    if (mb.size() > 1) mb = string(1, mb[0]) + "&" + mb.substr(1);
                    const int mp = mi.pos, me = mi.end;
                    if (!has_key(mp, mb)) continue;
                    HVar &var = N(mp).keys.at(mb);
                    if (var.cnt == 0) continue;
                    if (var.q / var.cnt < P.goodq) continue;
                    if (var.tp / var.cnt > (me == 3 ? r3.nm + 4 : r5.nm + 4)) continue;
                    if (var.cnt >= icnt + (int)insert1.size() || var.cnt / icnt >= 8) continue;
                    if (mp > position && me == 5) add_cov(position, var.cnt);
                    HVar *lref = nullptr;
                    if (mp > position && me == 3 && N(position).present && R.has(position)) {
                        char b = R.idx(position);
                        lref = nfind(position, string(1, b));
                    }
                    if (lref) add_sub(vref, var, lref);
                    else add_into(vref, var);
                    nerase_drop(mp, mb);
                }
                if (r3.misp != 0 && r3.mm.size() == 1 && has_key(r3.misp, r3.misnt) &&
                    N(r3.misp).keys.at(r3.misnt).cnt < icnt)
                    N(r3.misp).keys.erase(r3.misnt);
                if (r5.misp != 0 && r5.mm.size() == 1 && has_key(r5.misp, r5.misnt) &&
                    N(r5.misp).keys.at(r5.misnt).cnt < icnt)
                    N(r5.misp).keys.erase(r5.misnt);
                for (int sc5pp : r5.scp) {
                    Clip *k = clip(sc5, sc5pp);
                    if (!k || k->c.used) continue;
                    string seq = consensus(*k);
                    if (seq != " " && ismatch(seq, wupseq, -1)) {
                        if (sc5pp > position) add_cov(position, k->c.agg.cnt);
                        add_into(vref, k->c.agg);
                        k->c.used = true;
                    }
                }
                for (int sc3pp : r3.scp) {
                    Clip *k = clip(sc3, sc3pp);
                    if (!k || k->c.used) continue;
                    string seq = consensus(*k);
                    string mseq = !ins3.empty() ? sanpseq : vsub(sanpseq, sc3pp - position - 1);
                    if (seq != " " && ismatch(seq, mseq, 1)) {
                        const HVar &tv = k->c.agg;
                        if (sc3pp <= position || (int)insert1.size() > tv.tp / tv.cnt) add_cov(position, tv.cnt);
                        HVar *lref = nullptr;
                        if (sc3pp > position && N(position).present && R.has(position)) {
                            char b = R.idx(position);
                            lref = nfind(position, string(1, b));
                        }
                        if ((int)insert1.size() > tv.tp / tv.cnt) lref = nullptr;
                        add_sub(vref, tv, lref);
                        k->c.used = true;
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
                                HVar moved = iget(position, vn);
                                iget(position, tvn) = moved;
                                I(position).keys.erase(vn);
                            }
                        }
                    }
                }
                if (!r3.scp.empty() && !r5.scp.empty()) {
                    int first3 = r3.scp[0], first5 = r5.scp[0];
                    if (first3 > first5 + 3 && first3 - first5 < max_rl * 0.75) {
                        if (R.has(position) && N(position).present) {
                            char b = R.idx(position);
                            HVar *h = nfind(position, string(1, b));
                            if (h) adj_ref_factor(h, (first3 - first5 - 1) / (double)max_rl);
                        }
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
            PosMap &im = I(p);
            if (!im.present || !im.keys.count(vn)) continue;
            HVar &vref = im.keys.at(vn);
            string tn;
            if (keymatch::ins_amp_tail(vn, tn)) {  // (\+[ATGC]+)&[ATGC]+$
                auto t = im.keys.find(tn);
                if (t != im.keys.end() && vref.cnt < t->second.cnt) {
                    char b = R.idx(p);
                    add_sub(t->second, vref, maybe(p, b));
                    im.keys.erase(vn);
                }
            }
        }
    }

    // The batch's device find35match results for this region's listed clip
    // pairs (collect_lgins_pairs: per 5' clip its first pair and the 3'
    // clips of more than 10 characters in its position window, and every 3'
    // clip's consensus length)
    const int32_t *f35_res = nullptr;            // per pair: b5, b3, score
    std::vector<int64_t> f35_first;              // per t5 entry: its first pair, or -1
    std::vector<std::vector<int>> f35_near;      // per t5 entry: the 3' clips in its window, t3 order
    std::vector<int32_t> f35_len3;               // per t3 entry: consensus length (-1: not needed)

    // The 5'/3' clip lists realignlgins30 walks (by count), and the 3' clips
    // by position with their rank in t3.
    struct LgT { int pos; Clip *c; int cnt; };
    void lgins_lists(std::vector<LgT> &t5, std::vector<LgT> &t3, std::vector<std::pair<int, int>> &by_pos) {
        t5.clear();
        t3.clear();
        for (size_t k = 0; k < sc5.clips.size(); k++) {
            const int p = sc5.pos[k];
            if (!(p < Rg.start - 5000 || p > Rg.end + 5000)) t5.push_back({p, &sc5.clips[k], sc5.clips[k].c.agg.cnt});
        }
        for (size_t k = 0; k < sc3.clips.size(); k++) {
            const int p = sc3.pos[k];
            if (!(p < Rg.start - 5000 || p > Rg.end + 5000)) t3.push_back({p, &sc3.clips[k], sc3.clips[k].c.agg.cnt});
        }
        auto by_cnt = [](const LgT &a, const LgT &b) { return a.cnt != b.cnt ? a.cnt > b.cnt : a.pos < b.pos; };
        std::sort(t5.begin(), t5.end(), by_cnt);
        std::sort(t3.begin(), t3.end(), by_cnt);
        by_pos.resize(t3.size());
        for (size_t i = 0; i < t3.size(); i++) by_pos[i] = {t3[i].pos, (int)i};
        std::sort(by_pos.begin(), by_pos.end());
    }

    // Every clip pair realignlgins30 may hand to find35match: the pairs that
    // pass its position window, consensus lengths and count ratio (the clips'
    // `used` marks, which only skip pairs, are left out).  Appends each pair
    // as four int32 (offset and length of the 5' and of the 3' consensus in
    // `strs`) and records its index for find35.
    // the lists of the last lgins_lists call (collect_lgins_pairs builds them;
    // no clip count changes before realignlgins30 reads them)
    std::vector<LgT> lg_t5, lg_t3;
    std::vector<std::pair<int, int>> lg_by_pos;
    bool lg_ready = false;

    void collect_lgins_pairs(std::vector<int32_t> &pairs, string &strs) {
        lgins_lists(lg_t5, lg_t3, lg_by_pos);
        lg_ready = true;
        std::vector<LgT> &t5 = lg_t5, &t3 = lg_t3;
        const std::vector<std::pair<int, int>> &by_pos = lg_by_pos;
        // every 3' clip's consensus length; the "long" ones (more than 10
        // characters) by position with their rank in t3.  A 3' clip of 10 or
        // fewer characters does nothing in realignlgins30's loop: its
        // consensus is skipped right away, and consensus() marks a clip used
        // only for more than 12 characters
        std::vector<int32_t> off3(t3.size(), -1);
        f35_len3.assign(t3.size(), -1);
        std::vector<std::pair<int, int>> long_by_pos;
        for (const auto &pe : by_pos) {
            const int ib = pe.second;
            const string q = peek_consensus(*t3[ib].c);
            f35_len3[ib] = (int32_t)q.size();
            if (q.size() > 10) {
                off3[ib] = (int32_t)strs.size();
                strs += q;
                long_by_pos.push_back(pe);
            }
        }
        f35_first.assign(t5.size(), -1);
        f35_near.assign(t5.size(), std::vector<int>());
        int64_t k = 0;
        for (size_t ia = 0; ia < t5.size(); ia++) {
            const LgT &a = t5[ia];
            const string seq5 = peek_consensus(*a.c);
            if (seq5.size() <= 10) continue;
            const int p5 = a.pos;
            const int lo3 = (int)std::ceil(p5 - max_rl * 2.5) - 1, hi3 = p5 + max_rl - 10 + 1;
            std::vector<int> &near = f35_near[ia];
            for (auto it = std::lower_bound(long_by_pos.begin(), long_by_pos.end(), std::make_pair(lo3, INT32_MIN));
                 it != long_by_pos.end() && it->first <= hi3; ++it)
                near.push_back(it->second);
            std::sort(near.begin(), near.end());
            f35_first[ia] = k;
            int32_t off5 = -1;
            for (int ib : near) {
                const LgT &b = t3[ib];
                if (p5 - b.pos > max_rl * 2.5) continue;
                if (b.pos - p5 > max_rl - 10) continue;
                if (!(a.cnt / (double)b.cnt >= 0.08 && a.cnt / (double)b.cnt <= 12)) continue;
                if (off5 < 0) {
                    off5 = (int32_t)strs.size();
                    strs += seq5;
                }
                pairs.insert(pairs.end(), {off5, (int32_t)seq5.size(), off3[ib], f35_len3[ib]});
                k++;
            }
        }
    }

    // realignlgins30 (:1119-1350); its reference map is a copy (lookups that
    // insert stay local), the nested realignins/realigndel use the shared one
    void realignlgins30() {
        PRef RL = R;
        // the 3' clips by position (with their rank in t3): a 5' clip only
        // pairs with 3' clips in [p5 - 2.5 max_rl, p5 + max_rl - 10], and the
        // reference's loop over t3 does nothing else for the others, so the
        // pass visits just those, in t3 order
        if (!lg_ready) lgins_lists(lg_t5, lg_t3, lg_by_pos);
        lg_ready = false;
        std::vector<LgT> &t5 = lg_t5, &t3 = lg_t3;
        const std::vector<std::pair<int, int>> &by_pos = lg_by_pos;
        const bool dev = f35_res != nullptr;  // device results for the listed pairs
        std::vector<int> near_host;
        for (size_t ia = 0; ia < t5.size(); ia++) {
            LgT &a = t5[ia];
            const int p5 = a.pos;
            Clip &sc5v = *a.c;
            const int cnt5 = a.cnt;
            if (sc5v.c.used) continue;
            const string &seq5 = consensus(sc5v);
            if (seq5.size() <= 10) continue;
            const std::vector<int> *nearp = &near_host;
            if (dev) {
                nearp = &f35_near[ia];
            } else {
                const int lo3 = (int)std::ceil(p5 - max_rl * 2.5) - 1, hi3 = p5 + max_rl - 10 + 1;
                near_host.clear();
                for (auto it = std::lower_bound(by_pos.begin(), by_pos.end(), std::make_pair(lo3, INT32_MIN));
                     it != by_pos.end() && it->first <= hi3; ++it)
                    near_host.push_back(it->second);
                std::sort(near_host.begin(), near_host.end());
            }
            // the listed pairs of this 5' clip come in the order of its
            // window's 3' clips that pass the static tests
            int64_t kcur = dev ? f35_first[ia] : -1;
            for (int ni : *nearp) {
                LgT &b = t3[ni];
                int64_t kidx = -1;
                if (dev) {
                    const int pb = b.pos;
                    if (!(p5 - pb > max_rl * 2.5) && !(pb - p5 > max_rl - 10) &&
                        (cnt5 / (double)b.cnt >= 0.08 && cnt5 / (double)b.cnt <= 12) && f35_len3[ni] > 10)
                        kidx = kcur++;
                }
                try {
                    const int p3 = b.pos;
                    Clip &sc3v = *b.c;
                    const int cnt3 = b.cnt;
                    if (sc5v.c.used) break;
                    if (sc3v.c.used) continue;
                    if (p5 - p3 > max_rl * 2.5) continue;
                    if (p3 - p5 > max_rl - 10) continue;
                    const string &seq3 = consensus(sc3v);
                    if (seq3.size() <= 10) continue;
                    if (!(cnt5 / (double)cnt3 >= 0.08 && cnt5 / (double)cnt3 <= 12)) continue;
                    int bp5, bp3, score;
                    if (kidx >= 0) {
                        const int32_t *rr = f35_res + 3 * kidx;
                        bp5 = rr[0];
                        bp3 = rr[1];
                        score = rr[2];
                    } else {
                        keymatch::find35(seq5, seq3, bp5, bp3, score);
                    }
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
                    HVar *vref;
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
                            vref = &nget(p3, ins);
                        } else if (tmp.size() < ins.size()) {
                            ins = vsub(ins, 0, (int)ins.size() - (int)tmp.size()) + "&" + vsub(ins, p3 - p5);
                            ins = "+" + ins;
                            bi = p3 - 1;
                            vref = &iget(bi, ins);
                        } else {
                            ins = "-" + std::to_string(ins.size()) + "^" + ins;
                            bi = p3;
                            vref = &nget(p3, ins);
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
                        vref = &iget(bi, ins);
                    }
                    sc3v.c.used = true;
                    sc5v.c.used = true;
                    vref->pstd = true;
                    vref->qstd = true;
                    add_cov(bi, sc5v.c.agg.cnt);
                    if (ins[0] == '+') {
                        char rb = RL.idx(bi);
                        HVar *mvref = maybe(bi, rb);
                        add_sub(*vref, sc3v.c.agg, mvref);
                        add_into(*vref, sc5v.c.agg);
                        if (p3 - p5 >= 5 && p3 - p5 < max_rl - 10 && mvref && mvref->cnt != 0 &&
                            vref->cnt > 2 * mvref->cnt && no_passing_reads(p5, p3))
                            add_sub(*vref, *mvref, mvref);
                        std::map<int, std::map<string, int>> tins;
                        tins[bi][ins] = vref->cnt;
                        realignins(tins);
                    } else if (ins[0] == '-') {
                        char rb = RL.idx(bi);
                        add_sub(*vref, sc3v.c.agg, maybe(bi, rb));
                        add_into(*vref, sc5v.c.agg);
                        std::map<int, std::map<string, int>> tdel;
                        tdel[bi][ins] = vref->cnt;
                        realigndel(false, tdel);
                    } else {
                        add_into(*vref, sc3v.c.agg);
                        add_into(*vref, sc5v.c.agg);
                    }
                    break;
                } catch (const RefFail &) {
                } catch (const OutOfRange &) {
                }
            }
        }
    }

    // ------------------------------------------------------------------
    // diff of the mirror against its snapshots -> patches
    // ------------------------------------------------------------------
    void stats_into(Patch &q, const HVar &h) {
        q.fwd = h.fwd;
        q.rev = h.rev;
        q.hi = h.hi;
        q.lo = h.lo;
        q.extracnt = h.extracnt;
        q.cnt = h.cnt;
        q.tp = h.tp;
        q.q_sum = h.q;
        q.mq = h.mq;
        q.nm = h.nm;
        q.flags_or = (h.pstd ? (int)SF_PDIFF : 0) | (h.qstd ? (int)SF_QDIFF : 0);
    }
    void diff(std::vector<Patch> &out, string &keys) {
        auto blank = [] {
            Patch q;
            memset(&q, 0, sizeof q);
            return q;
        };
        auto create = [&](int p, int kind, const string &k, const HVar &h) {
            Patch q = blank();
            q.type = 5;
            q.region = region;
            q.pos = p;
            q.kind = kind;
            q.klen = (int)k.size();
            q.key_off = (int64_t)keys.size();
            keys += k;
            stats_into(q, h);
            out.push_back(q);
        };
        for (int pass = 0; pass < 2; pass++) {
            auto &cur = pass ? ins : nonins;
            auto &orig = pass ? ins0 : nonins0;
            const int kind = pass ? KIND_INS : KIND_NONINS;
            for (auto &pe : cur) {
                const int p = pe.first;
                if (!in_cells(p)) continue;
                const int64_t c = cell_of(p);
                const PosMap &F = pe.second, &O = orig.at(p);
                if (!pass && O.present && !F.present) {
                    // the entry left the map: its cell keys go and every slot
                    // of the position stops counting as an entry
                    Patch q = blank();
                    q.type = 6;
                    q.target = c;
                    out.push_back(q);
                    for (uint32_t i = mir.off[c]; i < mir.off[c + 1]; i++) {
                        if (mir.slots[i].kind != KIND_NONINS) continue;
                        Patch e = blank();
                        e.type = 1;
                        e.target = mir.sidx[i];
                        e.flags_or = (int)SF_NOMAP;
                        out.push_back(e);
                    }
                    continue;
                }
                for (auto &oe : O.keys) {
                    if (F.keys.count(oe.first)) continue;
                    Patch q = blank();
                    if (oe.second.slot >= 0) {
                        q.type = 1;
                        q.target = oe.second.slot;
                    } else {
                        q.type = 2;
                        q.target = oe.second.cell;
                        q.base = oe.second.base;
                    }
                    out.push_back(q);
                }
                for (auto &fe : F.keys) {
                    auto o = O.keys.find(fe.first);
                    if (o != O.keys.end() && same_stats(o->second, fe.second)) continue;
                    if (o != O.keys.end() && o->second.slot >= 0) {
                        Patch q = blank();
                        q.type = 4;
                        q.target = o->second.slot;
                        stats_into(q, fe.second);
                        out.push_back(q);
                        continue;
                    }
                    create(p, kind, fe.first, fe.second);
                    if (o != O.keys.end()) {  // a cell key moves to a slot
                        Patch q = blank();
                        q.type = 2;
                        q.target = o->second.cell;
                        q.base = o->second.base;
                        out.push_back(q);
                    }
                }
            }
        }
        for (auto &ce : cov_add) {
            if (!in_cells(ce.first) || ce.second == 0) continue;
            Patch q = blank();
            q.type = 3;
            q.target = cell_of(ce.first);
            q.cov_add = ce.second;
            out.push_back(q);
        }
    }

    // VariationRealigner::process (:135-161) in two parts: up to the indel
    // passes (collect_lgins_pairs then lists the clip pairs for the batch's
    // device find35 pass), and realignlgins30 plus the diff into patches
    void run_first(double *phase) {
        prof = phase;
        auto clk = [] { return std::chrono::steady_clock::now(); };
        auto t = clk();
        auto lap = [&](int k) {
            auto n = clk();
            phase[k] += std::chrono::duration<double, std::milli>(n - t).count();
            t = n;
        };
        std::map<int, std::map<string, int>> mnp, delcnt, inscnt;
        load_lists(mnp, delcnt, inscnt);
        lap(0);
        adjust_mnp(mnp);
        lap(1);
        realigndel(true, delcnt);
        lap(2);
        realignins(inscnt);
        lap(3);
    }
    void run_second(std::vector<Patch> &out, string &keys, double *phase) {
        prof = phase;
        auto clk = [] { return std::chrono::steady_clock::now(); };
        auto t = clk();
        auto lap = [&](int k) {
            auto n = clk();
            phase[k] += std::chrono::duration<double, std::milli>(n - t).count();
            t = n;
        };
        realignlgins30();
        lap(4);
        diff(out, keys);
        lap(5);
    }
};

}  // namespace

namespace {
struct MirrorLayout {
    size_t b_arr, b_cov, b_kf, b_off, cells;
    explicit MirrorLayout(int64_t nc) {
        auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
        b_arr = (size_t)nc * 16;
        b_cov = up16((size_t)nc * 4);
        b_kf = up16((size_t)nc);
        b_off = up16(((size_t)nc + 1) * 4);
        cells = 8 * b_arr + b_cov + b_kf + b_off;
    }
};
}  // namespace

// Queues the device side of the realigner's mirror on the context's stream
// without waiting: the flattened key lists (then `after_kernels` is recorded,
// if given), and the copies of the cells and the list offsets into pinned
// host memory.
rv_status mirror_launch(rv_ctx *ctx, cudaEvent_t after_kernels) {
    rv_status st;
    cudaStream_t s = ctx->stream;
    const int64_t nc = ctx->n_cells;
    const int64_t nb = (nc + 1023) / 1024;
    // list capacity: every listed key is a used slot
    if ((st = ensure(ctx, ctx->d_list_off, ctx->cap_list_off, (size_t)nc + 1)) ||
        (st = ensure(ctx, ctx->d_list_bsum, ctx->cap_list_bsum, (size_t)nb + 1)) ||
        (st = ensure(ctx, ctx->d_list_slots, ctx->cap_list_slots, (size_t)ctx->hash_cap)) ||
        (st = ensure(ctx, ctx->d_list_idx, ctx->cap_list_idx, (size_t)ctx->hash_cap)) ||
        (st = ensure(ctx, ctx->d_cons_meta, ctx->cap_cons_meta, (size_t)ctx->hash_cap)) ||
        (st = ensure(ctx, ctx->d_cons, ctx->cap_cons, (size_t)ctx->hash_cap)))
        return st;
    DevState ds = ctx->state();
    launch_list_offsets(ds, ctx->d_list_off, ctx->d_list_bsum, s);
    launch_list_fill(ds, ctx->d_list_off, ctx->d_list_slots, ctx->d_list_idx, s);
    launch_clip_consensus(ds, ctx->d_list_off, ctx->d_list_slots, ctx->d_cons_meta, ctx->d_cons, s);
    ctx->kernels += 6;
    if (after_kernels) HCUDA(cudaEventRecord(after_kernels, s));
    // pinned host copies: 8 cell arrays (16 B per cell each), cov, kflags, offsets
    const MirrorLayout L(nc);
    if (!ctx->h_mirror || ctx->cap_mirror < L.cells) {
        if (ctx->h_mirror) cudaFreeHost(ctx->h_mirror);
        ctx->h_mirror = nullptr;
        size_t cap = L.cells + L.cells / 4;
        HCUDA(cudaHostAlloc(&ctx->h_mirror, cap, cudaHostAllocDefault));
        ctx->cap_mirror = cap;
    }
    char *h = (char *)ctx->h_mirror;
    const Cells &C = ctx->cells;
    const void *dev_arr[8] = {C.fwd, C.rev, C.hi, C.tp, C.q, C.mq, C.nm, C.first};
    for (int k = 0; k < 8; k++, h += L.b_arr)
        if (nc) HCUDA(cudaMemcpyAsync(h, dev_arr[k], L.b_arr, cudaMemcpyDeviceToHost, s));
    if (nc) {
        // (coverage is not read by the realigner: its additions go back as deltas)
        HCUDA(cudaMemcpyAsync(h + L.b_cov, C.kflags, (size_t)nc, cudaMemcpyDeviceToHost, s));
        HCUDA(cudaMemcpyAsync(h + L.b_cov + L.b_kf, ctx->d_list_off, ((size_t)nc + 1) * 4, cudaMemcpyDeviceToHost, s));
    }
    ctx->mirror_pending = true;
    return RV_OK;
}

// find35match of n clip pairs on the context's device (k_find35): pairs as
// int32 quadruples into `strs`, results as (b5, b3, score) triples.
static rv_status device_find35(rv_ctx *ctx, const int32_t *pairs, int64_t n, const string &strs, int32_t *res) {
    const size_t b_pairs = (size_t)n * 16, b_strs = (strs.size() + 15) & ~(size_t)15, b_res = (size_t)n * 12;
    const size_t need = b_pairs + b_strs + b_res;
    if (ctx->cap_f35 < need || !ctx->d_f35) {
        if (ctx->d_f35) cudaFree(ctx->d_f35);
        ctx->d_f35 = nullptr;
        ctx->cap_f35 = 0;
        HCUDA(cudaMalloc(&ctx->d_f35, need + need / 4));
        ctx->cap_f35 = need + need / 4;
    }
    char *d = (char *)ctx->d_f35;
    cudaStream_t s = ctx->stream;
    HCUDA(cudaMemcpyAsync(d, pairs, b_pairs, cudaMemcpyHostToDevice, s));
    if (!strs.empty()) HCUDA(cudaMemcpyAsync(d + b_pairs, strs.data(), strs.size(), cudaMemcpyHostToDevice, s));
    launch_find35((const int32_t *)d, n, d + b_pairs, (int32_t *)(d + b_pairs + b_strs), s);
    HCUDA(cudaGetLastError());
    HCUDA(cudaMemcpyAsync(res, d + b_pairs + b_strs, b_res, cudaMemcpyDeviceToHost, s));
    HCUDA(cudaStreamSynchronize(s));
    ctx->kernels += 1;
    ctx->io_h2d += (int64_t)(b_pairs + strs.size());
    ctx->io_d2h += (int64_t)b_res;
    return RV_OK;
}

// VariationRealigner::process with -k 1 (src/VariationRealigner.cpp:135-161)
rv_status host_realign_full(rv_ctx *ctx) {
    const bool trace = getenv("RV_REALIGN_TRACE") != nullptr;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto t0 = now();
    auto ms = [&](std::chrono::steady_clock::time_point a) {
        return std::chrono::duration<double, std::milli>(now() - a).count();
    };
    Mirror mir;
    mir.ctx = ctx;
    rv_status st;
    cudaStream_t s = ctx->stream;
    const int64_t nc = ctx->n_cells;
    if (!ctx->mirror_pending && (st = mirror_launch(ctx, nullptr))) return st;
    ctx->mirror_pending = false;
    HCUDA(cudaStreamSynchronize(s));
    const MirrorLayout L(nc);
    char *h = (char *)ctx->h_mirror;
    char *host_arr[8];
    for (int k = 0; k < 8; k++) host_arr[k] = h + k * L.b_arr;
    char *h_cov = h + 8 * L.b_arr;
    char *h_kf = h_cov + L.b_cov;
    char *h_off = h_kf + L.b_kf;
    const uint32_t total = ((const uint32_t *)h_off)[nc];
    // the listed keys, their slot indices, the clip consensus records and characters
    const size_t b_sl = (size_t)total * sizeof(Slot), b_ix = ((size_t)total * 4 + 15) & ~(size_t)15;
    const size_t b_cm = b_ix, b_cc = ((size_t)total + 15) & ~(size_t)15;
    const size_t need_sl = b_sl + b_ix + b_cm + b_cc;
    if (!ctx->h_mirror_slots || ctx->cap_mirror_slots < need_sl) {
        if (ctx->h_mirror_slots) cudaFreeHost(ctx->h_mirror_slots);
        ctx->h_mirror_slots = nullptr;
        size_t cap = need_sl + need_sl / 4 + 4096;
        HCUDA(cudaHostAlloc(&ctx->h_mirror_slots, cap, cudaHostAllocDefault));
        ctx->cap_mirror_slots = cap;
    }
    char *h_sl = (char *)ctx->h_mirror_slots;
    char *h_ix = h_sl + b_sl;
    char *h_cm = h_ix + b_ix;
    char *h_cc = h_cm + b_cm;
    if (total) {
        HCUDA(cudaMemcpyAsync(h_sl, ctx->d_list_slots, b_sl, cudaMemcpyDeviceToHost, s));
        HCUDA(cudaMemcpyAsync(h_ix, ctx->d_list_idx, (size_t)total * 4, cudaMemcpyDeviceToHost, s));
        HCUDA(cudaMemcpyAsync(h_cm, ctx->d_cons_meta, (size_t)total * 4, cudaMemcpyDeviceToHost, s));
        HCUDA(cudaMemcpyAsync(h_cc, ctx->d_cons, (size_t)total, cudaMemcpyDeviceToHost, s));
    }
    mir.regions.resize(ctx->regions.size());
    if (!mir.regions.empty())
        HCUDA(cudaMemcpyAsync(mir.regions.data(), ctx->d_regions, mir.regions.size() * sizeof(Region),
                              cudaMemcpyDeviceToHost, s));
    HCUDA(cudaStreamSynchronize(s));
    if ((st = pull_arena(ctx))) return st;
    ctx->io_d2h += (int64_t)(L.cells - L.b_cov + (size_t)total * (sizeof(Slot) + 9) + ctx->h_arena.size());
    mir.fwd = (const uint32_t *)host_arr[0];
    mir.rev = (const uint32_t *)host_arr[1];
    mir.hi = (const uint32_t *)host_arr[2];
    mir.tp = (const uint32_t *)host_arr[3];
    mir.q = (const uint32_t *)host_arr[4];
    mir.mq = (const uint32_t *)host_arr[5];
    mir.nm = (const int32_t *)host_arr[6];
    mir.first = (const uint32_t *)host_arr[7];
    mir.kflags = (const uint8_t *)h_kf;
    mir.off = (const uint32_t *)h_off;
    mir.slots = (const Slot *)h_sl;
    mir.sidx = (const uint32_t *)h_ix;
    mir.cmeta = (const uint32_t *)h_cm;
    mir.cons = (const uint8_t *)h_cc;
    double t_fetch = ms(t0);
    // regions in parallel; patches concatenated in region order
    const int nreg = (int)ctx->regions.size();
    std::vector<std::vector<Patch>> patches((size_t)nreg);
    std::vector<string> keys((size_t)nreg);
    const int nt = pool_threads();
    std::mutex err_mu;
    string failure;
    std::vector<double> phase((size_t)nreg * 8, 0.0);
    std::vector<std::unique_ptr<RegionRealigner>> rrs((size_t)nreg);
    std::vector<std::vector<int32_t>> f35_pairs((size_t)nreg);
    std::vector<string> f35_strs((size_t)nreg);
    // the realigner up to the indel passes, and the clip pairs each region's
    // realignlgins30 may test (offsets local to the region)
    parallel_for(nreg, [&](int64_t r) {
        try {
            rrs[r].reset(new RegionRealigner(mir, ctx, (int)r));
            rrs[r]->run_first(phase.data() + 8 * r);
            auto tc = now();
            rrs[r]->collect_lgins_pairs(f35_pairs[r], f35_strs[r]);
            phase[8 * r + 6] += std::chrono::duration<double, std::milli>(now() - tc).count();
        } catch (const std::exception &e) {
            // the reference's own realigner terminates here (an exception it
            // does not catch); the batch reports it instead
            std::lock_guard<std::mutex> g(err_mu);
            if (failure.empty()) failure = "realigner, region " + std::to_string(r) + ": " + e.what();
        }
    });
    if (!failure.empty()) {
        ctx->err = failure;
        return RV_ERR_UNSUPPORTED;
    }
    const double t_first = ms(t0);
    // find35match of every listed pair of the batch, on the device
    auto tf = now();
    std::vector<int32_t> f35_res;
    std::vector<int64_t> pair_base((size_t)nreg + 1, 0), str_base((size_t)nreg + 1, 0);
    for (int r = 0; r < nreg; r++) {
        pair_base[r + 1] = pair_base[r] + (int64_t)f35_pairs[r].size() / 4;
        str_base[r + 1] = str_base[r] + (int64_t)f35_strs[r].size();
    }
    const int64_t np = pair_base[nreg];
    if (np > 0) {
        if (str_base[nreg] > INT32_MAX) {
            ctx->err = "realigner: clip consensus strings exceed 2 GB";
            return RV_ERR_CAPACITY;
        }
        std::vector<int32_t> all_pairs((size_t)np * 4);
        string all_strs((size_t)str_base[nreg], '\0');
        parallel_for(nreg, [&](int64_t r) {
            const std::vector<int32_t> &v = f35_pairs[r];
            int32_t *o = all_pairs.data() + 4 * pair_base[r];
            for (size_t i = 0; i < v.size(); i += 4) {
                o[i] = v[i] + (int32_t)str_base[r];
                o[i + 1] = v[i + 1];
                o[i + 2] = v[i + 2] + (int32_t)str_base[r];
                o[i + 3] = v[i + 3];
            }
            if (!f35_strs[r].empty()) memcpy(&all_strs[(size_t)str_base[r]], f35_strs[r].data(), f35_strs[r].size());
        });
        f35_res.resize((size_t)np * 3);
        if ((st = device_find35(ctx, all_pairs.data(), np, all_strs, f35_res.data()))) return st;
    }
    const double t_f35 = ms(tf);
    const double t_dev_done = ms(t0);
    parallel_for(nreg, [&](int64_t r) {
        try {
            RegionRealigner &rr = *rrs[r];
            if (np > 0) rr.f35_res = f35_res.data() + 3 * pair_base[r];
            rr.run_second(patches[r], keys[r], phase.data() + 8 * r);
            rrs[r].reset();
        } catch (const std::exception &e) {
            std::lock_guard<std::mutex> g(err_mu);
            if (failure.empty()) failure = "realigner, region " + std::to_string(r) + ": " + e.what();
        }
    });
    if (!failure.empty()) {
        ctx->err = failure;
        return RV_ERR_UNSUPPORTED;
    }
    std::vector<Patch> all;
    string all_keys;
    for (int r = 0; r < nreg; r++) {
        for (Patch q : patches[r]) {
            if (q.type == 5) q.key_off += (int64_t)all_keys.size();
            all.push_back(q);
        }
        all_keys += keys[r];
    }
    double t_run = ms(t0);
    st = apply_patches(ctx, all, all_keys);
    if (trace) {
        double sum[8] = {0};
        for (int r = 0; r < nreg; r++)
            for (int k = 0; k < 8; k++) sum[k] += phase[8 * r + k];
        fprintf(stderr, "realign -k 1: listed keys %u, patches %zu, threads %d, find35 pairs %lld; ms: fetch %.2f "
                "first-half %.2f device-find35 %.2f (done at %.2f) run %.2f total %.2f; thread-ms: setup %.2f mnp %.2f "
                "del %.2f ins %.2f lgins %.2f diff %.2f collect %.2f\n",
                total, all.size(), nt, (long long)np, t_fetch, t_first, t_f35, t_dev_done, t_run, ms(t0), sum[0],
                sum[1], sum[2], sum[3], sum[4], sum[5], sum[6]);
    }
    return st;
}

}  // namespace rv
