// Scoring kernels: per-site statistics of ToVarsBuilder::process
// (src/ToVarsBuilder.cpp:97-205, createVariant :466-536, createInsertion
// :358-452, calcHicov :570-587, CMP_VARI :20-26, collectVarsAtPosition
// :327-346, the numeric part of collectReferenceVariants :730-1098), the
// numeric pre-screen of Variant::isGoodVar (include/Variant.h:197-248) and
// the two-sided Fisher exact test of the --fisher output
// (src/modes/simpleMode.cpp:96-108) in FP64.
#include <cuda_runtime.h>

#include <algorithm>

#include "rv_walk.cuh"

namespace rv {

constexpr int kMaxVars = 32;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t FCS_PDIFF = 1u << 30, FCS_QDIFF = 1u << 31;

__device__ __forceinline__ int64_t cell_index(const Region &R, int p) { return R.cell_base + (p - R.clo); }

// Link every string-keyed allele into the list of its position.
__global__ void k_link_slots(DevState st) {
    unsigned long long n = used_count(st.hash);
    for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < n;
         u += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = st.hash.used[u];
        Slot &s = st.hash.slots[i];
        if (s.fp == 0ULL || s.kind == KIND_SPLICE) continue;
        const Region &R = st.regions[s.region];
        if (s.pos < R.clo || s.pos > R.chi) continue;
        int64_t c = cell_index(R, s.pos);
        bool clip = s.kind != KIND_NONINS && s.kind != KIND_INS;
        s.next = atomicExch(clip ? &st.head_sc[c] : &st.head[c], (uint32_t)i);
    }
}

__global__ void k_check_collisions(DevState st) {
    // every inserter XORs h2 of its key into the slot: for an odd number of
    // inserters of one key the result is h2, for an even number it is 0
    unsigned long long n = used_count(st.hash);
    for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < n;
         u += (unsigned long long)gridDim.x * blockDim.x) {
        const Slot &s = st.hash.slots[st.hash.used[u]];
        if (s.fp == 0ULL) continue;
        unsigned long long h1, h2;
        unsigned long long a = fmix64(((unsigned long long)(uint32_t)s.region << 32) ^ (uint32_t)s.pos ^
                                      ((unsigned long long)s.kind << 58) ^ ((unsigned long long)s.klen << 44));
        unsigned long long b = fmix64(a ^ 0x9e3779b97f4a7c15ULL);
        const uint8_t *k = st.hash.arena + s.koff;
        int n_ = s.klen;
        for (int ii = 0; ii < n_;) {
            unsigned long long w = 0;
            int m = n_ - ii < 8 ? n_ - ii : 8;
            for (int j = 0; j < m; j++) w |= (unsigned long long)k[ii + j] << (8 * j);
            a = fmix64(a ^ w) + 0x632be59bd9b4e019ULL;
            b = fmix64(b + w * 0x94d049bb133111ebULL);
            ii += m;
        }
        h1 = a ? a : 1;
        h2 = b;
        int inserters = s.fwd + s.rev;  // every observation re-inserts the key
        (void)inserters;
        if (h1 != s.fp || (s.h2x != 0ULL && s.h2x != h2)) atomicOr(st.err, ERR_COLLISION);
    }
}

struct V {
    int kind;       // 0 single (key_off = base), 1 hash slot (key_off = slot index)
    int key;        // base 0..3 or slot index
    int cnt, fwd, rev, hi, lo, extracnt;
    double tp, q, mq, nm;
    bool pstd, qstd;
    // derived Variant fields
    int ttcov, hicov;
    double freq, pmean, qual, mqv, qratio, hifreq, extrafreq, nmv;
    int bias;
};

__device__ int strand_bias(int f, int r, const DevParams &P) {  // include/VariationUtils.h:511-521
    if (f + r <= 12) return f * r > 0 ? 2 : 0;
    return (f / (double)(f + r) >= P.bias && r / (double)(f + r) >= P.bias && f >= P.min_bias_reads &&
            r >= P.min_bias_reads) ? 2 : 1;
}

__device__ void finish_var(V &v, int ttcov, int hicov, const DevParams &P) {
    v.ttcov = ttcov;
    v.hicov = hicov;
    v.bias = strand_bias(v.fwd, v.rev, P);
    v.freq = v.cnt / (double)ttcov;
    v.pmean = v.tp / (double)v.cnt;
    v.qual = v.q / v.cnt;
    v.mqv = v.mq / (double)v.cnt;
    v.qratio = v.hi / (v.lo != 0 ? (double)v.lo : 0.5);
    v.hifreq = hicov > 0 ? v.hi / (double)hicov : 0;
    v.extrafreq = v.extracnt != 0 ? v.extracnt / (double)ttcov : 0;
    v.nmv = v.nm / (double)v.cnt;
}

// lexicographic compare of two keys (std::string::compare order)
__device__ int key_cmp(const DevState &st, const V &a, const V &b) {
    const char bases[4] = {'A', 'C', 'G', 'T'};
    char ca[1], cb[1];
    const char *pa, *pb;
    int na, nb;
    if (a.kind == 0) { ca[0] = bases[a.key]; pa = ca; na = 1; }
    else { const Slot &s = st.hash.slots[a.key]; pa = (const char *)st.hash.arena + s.koff; na = s.klen; }
    if (b.kind == 0) { cb[0] = bases[b.key]; pb = cb; nb = 1; }
    else { const Slot &s = st.hash.slots[b.key]; pb = (const char *)st.hash.arena + s.koff; nb = s.klen; }
    int m = na < nb ? na : nb;
    for (int i = 0; i < m; i++) {
        unsigned char x = (unsigned char)pa[i], y = (unsigned char)pb[i];
        if (x != y) return x < y ? -1 : 1;
    }
    return na == nb ? 0 : (na < nb ? -1 : 1);
}

__device__ bool cmp_vari(const DevState &st, const V &a, const V &b) {  // CMP_VARI
    double r = a.qual * a.cnt - b.qual * b.cnt;
    if (r < 0.00001 && r > -0.00001) return key_cmp(st, a, b) < 0;
    return r > 0;
}

__device__ __forceinline__ int slot_cnt(const Slot &s) {
    return (s.flags & SF_OVR) ? s.first_tp : s.fwd + s.rev;
}

__device__ void load_slot(const Slot &s, int idx, V &v) {
    v.kind = 1;
    v.key = idx;
    v.cnt = slot_cnt(s);
    v.fwd = s.fwd;
    v.rev = s.rev;
    v.hi = s.hi;
    v.lo = s.lo;
    v.extracnt = s.extracnt;
    v.q = s.q_sum;
    if (s.flags & SF_OVR) {
        v.tp = __longlong_as_double(s.tp_sum);
        v.mq = __longlong_as_double(s.mq_sum);
        v.nm = __longlong_as_double(s.nm_sum);
        v.pstd = (s.flags & SF_PDIFF) != 0;
        v.qstd = (s.flags & SF_QDIFF) != 0;
    } else {
        v.tp = (double)s.tp_sum;
        v.mq = (double)s.mq_sum;
        v.nm = (double)s.nm_sum;
        v.pstd = (s.flags & (SF_PDIFF | SF_FORCE_STD)) != 0;
        v.qstd = (s.flags & (SF_QDIFF | SF_FORCE_STD)) != 0;
    }
}

// A single-base key the -k 1 realigner rewrote lives in a slot (its cell key
// is erased): returns the base 0..3 of such a slot, else -1.
__device__ __forceinline__ int promoted_base(const DevState &st, const Slot &s) {
    if (s.kind != KIND_NONINS || s.klen != 1) return -1;
    return base_index((char)st.hash.arena[s.koff]);
}

struct PosKeys {
    uint32_t *ins;       // insertion slots (storage of the caller, ins_cap entries)
    int ins_cap;
    int n_ins;           // insertion keys at the position (may exceed ins_cap: then only counted)
    int n_nonins;        // keys present in the position's nonInsertionVariants map
    bool in_map;         // the position has an entry in nonInsertionVariants
    int single_mask;     // present A/C/G/T keys
    __device__ bool overflow() const { return n_ins > ins_cap; }
};

// Queues a position for the wide pass (its alleles exceed the caller's arrays).
__device__ void push_wide(WidePos *list, unsigned int *n, unsigned int cap, unsigned int *err, int region, int pos,
                          int need, bool forced) {
    const unsigned int k = atomicAdd(n, 1u);
    if (k >= cap) { atomicOr(err, ERR_WIDE_FULL); return; }
    WidePos w;
    w.region = region;
    w.pos = pos;
    w.need = need;
    w.forced = forced ? 1 : 0;
    list[k] = w;
}

__device__ void gather_keys(const DevState &st, const Region &R, int p, PosKeys &k) {
    int64_t c = cell_index(R, p);
    uint8_t kf = st.cells.kflags[c];
    int exist = kf & 15, erased = (kf >> 4) & 15;
    k.single_mask = exist & ~erased;
    k.n_nonins = __popc(k.single_mask);
    k.in_map = exist != 0;
    k.n_ins = 0;
    for (uint32_t s = st.head[c]; s != kNone; s = st.hash.slots[s].next) {
        const Slot &sl = st.hash.slots[s];
        if (sl.kind == KIND_NONINS) {
            if (!(sl.flags & SF_NOMAP)) k.in_map = true;
            if (!(sl.flags & SF_ERASED)) {
                k.n_nonins++;
                int b = promoted_base(st, sl);
                if (b >= 0) k.single_mask |= 1 << b;
            }
        } else if (sl.kind == KIND_INS && !(sl.flags & SF_ERASED)) {
            if (k.n_ins < k.ins_cap) k.ins[k.n_ins] = s;
            k.n_ins++;
        }
    }
}

// sort the insertion keys of a position by key string (createInsertion sorts them)
__device__ void sort_ins(const DevState &st, PosKeys &k) {
    for (int i = 1; i < k.n_ins; i++) {
        uint32_t x = k.ins[i];
        V vx; vx.kind = 1; vx.key = (int)x;
        int j = i - 1;
        while (j >= 0) {
            V vy; vy.kind = 1; vy.key = (int)k.ins[j];
            if (key_cmp(st, vy, vx) <= 0) break;
            k.ins[j + 1] = k.ins[j];
            j--;
        }
        k.ins[j + 1] = x;
    }
}

__device__ char ref_at(const DevState &st, const Region &R, int p) {
    return (p >= R.ws && p <= R.we) ? st.ref[p - 1] : (char)0;
}

// The reference-base key of position p (base b): its cell (returns 0, `g` =
// cell word index), a promoted slot (returns 1, `slot`), or none (-1).
__device__ int ref_key_at(const DevState &st, const Region &R, int p, int b, int64_t &g, uint32_t &slot) {
    if (b < 0 || p < R.clo || p > R.chi) return -1;
    int64_t c = cell_index(R, p);
    uint8_t kf = st.cells.kflags[c];
    if (((kf >> b) & 1) && !((kf >> (4 + b)) & 1)) { g = 4 * c + b; return 0; }
    for (uint32_t s = st.head[c]; s != kNone; s = st.hash.slots[s].next) {
        const Slot &sl = st.hash.slots[s];
        if (!(sl.flags & SF_ERASED) && promoted_base(st, sl) == b) { slot = s; return 1; }
    }
    return -1;
}

// createInsertion's coverage bookkeeping for position p; when `apply` the
// reference counts at p+1 are adjusted (src/ToVarsBuilder.cpp:403-417).
// Returns the updated total coverage.
__device__ int insertion_pass(const DevState &st, const Region &R, int p, int tpc, const PosKeys &k, bool apply) {
    for (int i = 0; i < k.n_ins; i++) {
        const Slot &s = st.hash.slots[k.ins[i]];
        int cnt = slot_cnt(s);
        int ttcov = tpc;
        if (cnt > tpc && s.extracnt != 0 && cnt - tpc < s.extracnt) ttcov = cnt;
        if (ttcov < cnt) {
            ttcov = cnt;
            int p1 = p + 1;
            if (p1 <= R.chi) {
                int64_t c1 = cell_index(R, p1);
                uint32_t cov1 = st.cells.cov[c1];
                bool has1 = (p1 >= R.ws && p1 <= R.we);
                if (cov1 != 0 && has1 && ttcov < (int)cov1 - cnt) {
                    ttcov = (int)cov1;
                    if (apply) {
                        int64_t g = 0;
                        uint32_t rs = kNone;
                        int w = ref_key_at(st, R, p1, base_index(ref_at(st, R, p1)), g, rs);
                        if (w == 0) {
                            atomicSub(&st.cells.fwd[g], (uint32_t)s.fwd);
                            atomicSub(&st.cells.rev[g], (uint32_t)s.rev);
                        } else if (w == 1) {
                            atomicSub(&st.hash.slots[rs].fwd, s.fwd);
                            atomicSub(&st.hash.slots[rs].rev, s.rev);
                        }
                    }
                }
            }
            tpc = ttcov;
        }
    }
    return tpc;
}

// ToVarsBuilder visits a position when it has a nonInsertionVariants entry
// with at least one key or an insertion, and nonzero coverage.
__device__ bool visited(const DevState &st, const Region &R, int p, PosKeys &k) {
    gather_keys(st, R, p, k);
    if (!k.in_map) return false;
    if (k.n_nonins == 0 && k.n_ins == 0) return false;
    return st.cells.cov[cell_index(R, p)] != 0;
}

// Apply the insertion adjustments of every visited position (in ascending
// position order semantics: a position's adjustment of p+1 is visible when
// p+1 is scored).  Positions with more than kMaxVars insertion keys are left
// to k_ins_adjust_wide.
__global__ void k_ins_adjust(DevState st) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < st.cells.n_cells;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (st.head[t] == kNone) continue;
        // region of cell t
        int lo = 0, hi = st.n_regions - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (st.regions[mid].cell_base <= t) lo = mid; else hi = mid - 1;
        }
        const Region &R = st.regions[lo];
        int p = R.clo + (int)(t - R.cell_base);
        uint32_t ins[kMaxVars];
        PosKeys k;
        k.ins = ins;
        k.ins_cap = kMaxVars;
        if (!visited(st, R, p, k) || k.n_ins == 0) continue;
        if (k.overflow()) {
            push_wide(st.wide_ins, st.n_wide_ins, st.wide_cap, st.err, lo, p, k.n_ins, false);
            continue;
        }
        sort_ins(st, k);
        insertion_pass(st, R, p, (int)st.cells.cov[t], k, true);
    }
}

// Scratch offsets of a wide list: off[i] = the sum over j < i of
// max(1, need_j) + 8 (entry j's alleles and insertion keys), off[n] the
// total.  One block; the wide kernels queued behind it read them, so the
// wide passes need no host round trip.
__global__ void k_wide_offsets(const WidePos *list, const unsigned int *n_ptr, unsigned int cap, int64_t *off) {
    __shared__ int64_t warp_sum[32];
    __shared__ int64_t carry;
    unsigned int n = *n_ptr;
    if (n > cap) n = cap;
    if (threadIdx.x == 0) {
        carry = 0;
        off[0] = 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (unsigned int base = 0; base < n; base += blockDim.x) {
        const unsigned int i = base + threadIdx.x;
        int64_t v = i < n ? (int64_t)max(1, list[i].need) + 8 : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v += t;
        }
        if (lane == 31) warp_sum[wid] = v;
        __syncthreads();
        if (wid == 0) {
            int64_t w = lane < nw ? warp_sum[lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                const int64_t t = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += t;
            }
            if (lane < nw) warp_sum[lane] = w;
        }
        __syncthreads();
        const int64_t incl = carry + (wid ? warp_sum[wid - 1] : 0) + v;
        if (i < n) off[i + 1] = incl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = incl;
        __syncthreads();
    }
}

// The same for the queued wide positions, one thread each, with their
// insertion keys in global scratch (off[i]: first scratch entry of entry i,
// from k_wide_offsets).  Scratch of fewer than off[n] entries: nothing is
// done and the error word says so (the host grows it and runs this again).
__global__ void k_ins_adjust_wide(DevState st, const int64_t *off, uint32_t *ins_scratch, int64_t scratch_cap) {
    unsigned int n = *st.n_wide_ins;
    if (n > st.wide_cap) n = st.wide_cap;
    if (n == 0) return;
    if (off[n] > scratch_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(st.err, ERR_WIDE_INS_SCRATCH);
        return;
    }
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const WidePos w = st.wide_ins[i];
        const Region &R = st.regions[w.region];
        PosKeys k;
        k.ins = ins_scratch + off[i];
        k.ins_cap = (int)(off[i + 1] - off[i]);
        if (!visited(st, R, w.pos, k) || k.n_ins == 0 || k.overflow()) continue;
        sort_ins(st, k);
        insertion_pass(st, R, w.pos, (int)st.cells.cov[cell_index(R, w.pos)], k, true);
    }
}

__device__ double log_choose(int n, int k) {
    return lgamma((double)n + 1.0) - lgamma((double)k + 1.0) - lgamma((double)(n - k) + 1.0);
}

// log(k!) from the context's table (the same lgamma values, computed once)
__device__ __forceinline__ double log_choose_t(const double *lf, int n, int k) { return lf[n] - lf[k] - lf[n - k]; }

__global__ void k_fill_logfact(double *lf, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        lf[k] = lgamma((double)k + 1.0);
}

// Two-sided Fisher exact test on (n11 n12; n21 n22) from the hypergeometric
// definition: sum of table probabilities not above the observed one
// (relative slack 1e-7 for ties).
__device__ double fisher_two_sided(int n11, int n12, int n21, int n22, const double *lf = nullptr) {
    int r1 = n11 + n12, c1 = n11 + n21, n = n11 + n12 + n21 + n22;
    int lo = r1 + c1 - n > 0 ? r1 + c1 - n : 0;
    int hi = r1 < c1 ? r1 : c1;
    if (n11 < 0 || n12 < 0 || n21 < 0 || n22 < 0 || lo >= hi) return 1.0;
    if (lf && n < kLogFact) {
        double base = log_choose_t(lf, n, c1);
        double p_obs = exp(log_choose_t(lf, r1, n11) + log_choose_t(lf, n - r1, c1 - n11) - base);
        double thr = p_obs * (1.0 + 1e-7);
        double st = 0.0;
        for (int x = lo; x <= hi; ++x) {
            double p = exp(log_choose_t(lf, r1, x) + log_choose_t(lf, n - r1, c1 - x) - base);
            if (p <= thr) st += p;
        }
        return st > 1.0 ? 1.0 : st;
    }
    double base = log_choose(n, c1);
    double p_obs = exp(log_choose(r1, n11) + log_choose(n - r1, c1 - n11) - base);
    double thr = p_obs * (1.0 + 1e-7);
    double st = 0.0;
    for (int x = lo; x <= hi; ++x) {
        double p = exp(log_choose(r1, x) + log_choose(n - r1, c1 - x) - base);
        if (p <= thr) st += p;
    }
    return st > 1.0 ? 1.0 : st;
}

// Scores position p of region `lo`: ToVarsBuilder::process for one position
// (src/ToVarsBuilder.cpp:97-205).  Positions that pass the screens (or every
// position with variants when `forced`) write all their alleles as CandVars.
// `vs` / `insbuf` hold up to vcap alleles / insertion keys (per-thread
// arrays, or global scratch in the wide pass); a position with more is
// queued for the wide pass (when `wide` is false) and not scored here.
__device__ void score_position(const DevState &st, const DevParams &P, int lo, int p, bool forced, V *vs, int vcap,
                               uint32_t *insbuf, bool wide) {
    const Region &R = st.regions[lo];
    if (p < R.clo || p > R.chi) return;
    int64_t c = cell_index(R, p);
    char rb = ref_at(st, R, p);
    int rbi = base_index(rb);
    bool hasp = p >= R.ws && p <= R.we;
    // quick screen for positions holding only A/C/G/T keys: skip when only
    // the reference base was seen, or when no other base could pass the
    // -f gate and the numeric part of isGoodVar
    if (!forced && st.head[c] == kNone && !P.do_pileup) {
        uint8_t kf0 = st.cells.kflags[c];
        int ex = kf0 & 15 & ~(kf0 >> 4);
        if (ex == 0) return;
        uint32_t cov0 = st.cells.cov[c];
        if (cov0 == 0) return;
        if (hasp && rbi >= 0 && ex == (1 << rbi)) return;
        const uint4 f4 = *reinterpret_cast<const uint4 *>(st.cells.fwd + 4 * c);
        const uint4 r4 = *reinterpret_cast<const uint4 *>(st.cells.rev + 4 * c);
        const uint4 h4 = *reinterpret_cast<const uint4 *>(st.cells.hi + 4 * c);
        const uint32_t fa[4] = {f4.x, f4.y, f4.z, f4.w}, ra[4] = {r4.x, r4.y, r4.z, r4.w};
        const uint32_t ha[4] = {h4.x, h4.y, h4.z, h4.w};
        // the -f gate needs some non-reference allele with freq > -f; an
        // emitted record needs one with freq >= -f and hicnt >= -r (they
        // may be different alleles, e.g. at freq exactly -f)
        bool gate = false, pass = false;
        for (int b = 0; b < 4; b++) {
            if (!((ex >> b) & 1) || (hasp && b == rbi)) continue;
            int cnt = (int)(fa[b] + ra[b]);
            if (cnt <= 0) continue;
            double fr = cnt / (double)cov0;
            if (fr > P.freq) gate = true;
            if (fr >= P.freq && (int)ha[b] >= P.minr) pass = true;
            if (P.dataset_min > 0 && cnt >= P.dataset_min) pass = gate = true;
        }
        // somatic mode keeps every covered position (no -f gate), so only
        // the emission condition screens
        if (!pass || !(gate || P.somatic)) return;
    }
    PosKeys k;
    k.ins = insbuf;
    k.ins_cap = vcap;
    if (!visited(st, R, p, k)) return;
    {
        // alleles at the position: present A/C/G/T cells, live string keys
        int need = k.n_ins + __popc(k.single_mask & 15);
        for (uint32_t s = st.head[cell_index(R, p)]; s != kNone; s = st.hash.slots[s].next) {
            const Slot &sl = st.hash.slots[s];
            if (sl.kind == KIND_NONINS && !(sl.flags & SF_ERASED)) need++;
        }
        if (need > vcap || k.overflow()) {
            if (!wide) push_wide(st.wide_score, st.n_wide_score, st.wide_cap, st.err, lo, p, need, forced);
            else atomicOr(st.err, ERR_WIDE_FULL);
            return;
        }
    }
    // isTheSameVariationOnRef (src/ToVarsBuilder.cpp:213-233)
    if (!forced && !P.do_pileup && !P.somatic && k.n_nonins == 1 && k.n_ins == 0 && hasp && rbi >= 0 &&
        k.single_mask == (1 << rbi))
        return;
    int tpc = (int)st.cells.cov[c];
    // calcHicov
    int hicov = 0;
    int nv = 0;
    const uint8_t kfc = st.cells.kflags[c];
    const int cell_mask = kfc & 15 & ~(kfc >> 4);
    for (int b = 0; b < 4; b++) {
        if (!((cell_mask >> b) & 1)) continue;
        int64_t g = 4 * c + b;
        hicov += (int)st.cells.hi[g];
    }
    for (uint32_t s = st.head[c]; s != kNone; s = st.hash.slots[s].next) {
        const Slot &sl = st.hash.slots[s];
        if (!(sl.flags & SF_ERASED) && (sl.kind == KIND_NONINS || sl.kind == KIND_INS)) hicov += sl.hi;
    }
    // createVariant (non-insertion keys with a count)
    for (int b = 0; b < 4; b++) {
        if (!((cell_mask >> b) & 1)) continue;
        int64_t g = 4 * c + b;
        V v;
        v.kind = 0;
        v.key = b;
        v.fwd = (int)st.cells.fwd[g];
        v.rev = (int)st.cells.rev[g];
        v.cnt = v.fwd + v.rev;
        if (v.cnt == 0) continue;
        v.hi = (int)st.cells.hi[g];
        v.lo = v.cnt - v.hi;
        v.extracnt = 0;
        v.tp = (double)(int)st.cells.tp[g];
        v.q = (double)(int)st.cells.q[g];
        v.mq = (double)(int)st.cells.mq[g];
        v.nm = (double)st.cells.nm[g];
        uint32_t f = st.cells.first[g];
        v.pstd = (f & FCS_PDIFF) != 0;
        v.qstd = (f & FCS_QDIFF) != 0;
        finish_var(v, tpc, hicov, P);
        if (nv < vcap) vs[nv++] = v;
    }
    for (uint32_t s = st.head[c]; s != kNone; s = st.hash.slots[s].next) {
        const Slot &sl = st.hash.slots[s];
        if (sl.kind != KIND_NONINS || (sl.flags & SF_ERASED)) continue;
        V v;
        load_slot(sl, (int)s, v);
        if (v.cnt == 0) continue;
        const int pb = promoted_base(st, sl);
        if (pb >= 0) { v.kind = 0; v.key = pb; }
        int ttcov = tpc;
        if (v.cnt > tpc && v.extracnt > 0 && v.cnt - tpc < v.extracnt) ttcov = v.cnt;
        finish_var(v, ttcov, hicov, P);
        if (nv < vcap) vs[nv++] = v; else atomicOr(st.err, ERR_UNSUPPORTED);
    }
    // createInsertion
    if (k.n_ins > 0) {
        sort_ins(st, k);
        int hic = hicov;
        for (int i = 0; i < k.n_ins; i++) {
            const Slot &sl = st.hash.slots[k.ins[i]];
            V v;
            load_slot(sl, (int)k.ins[i], v);
            int ttcov = tpc;
            if (v.cnt > tpc && v.extracnt != 0 && v.cnt - tpc < v.extracnt) ttcov = v.cnt;
            if (ttcov < v.cnt) {
                ttcov = v.cnt;
                int p1 = p + 1;
                if (p1 <= R.chi) {
                    uint32_t cov1 = st.cells.cov[cell_index(R, p1)];
                    if (cov1 != 0 && p1 >= R.ws && p1 <= R.we && ttcov < (int)cov1 - v.cnt) ttcov = (int)cov1;
                }
                tpc = ttcov;
            }
            if (hic < v.hi) hic = v.hi;
            finish_var(v, ttcov, hic, P);
            if (nv < vcap) vs[nv++] = v; else atomicOr(st.err, ERR_UNSUPPORTED);
        }
    }
    // sort by CMP_VARI (insertion sort; few alleles per position)
    for (int i = 1; i < nv; i++) {
        V x = vs[i];
        int j = i - 1;
        while (j >= 0 && cmp_vari(st, x, vs[j])) { vs[j + 1] = vs[j]; j--; }
        vs[j + 1] = x;
    }
    // collectVarsAtPosition: the reference allele is the single key equal to the reference base
    int ref_i = -1;
    double maxfreq = 0;
    int n_var = 0;
    for (int i = 0; i < nv; i++) {
        if (hasp && vs[i].kind == 0 && vs[i].key == rbi) ref_i = i;
        else { n_var++; if (vs[i].freq > maxfreq) maxfreq = vs[i].freq; }
    }
    // only zero-count keys: the reference dereferences a null reference
    // variant there (src/ToVarsBuilder.cpp:737-743); nothing is emitted
    if (nv == 0) return;
    if (!forced) {
        if (!P.do_pileup && !P.somatic && !P.dataset_min && maxfreq <= P.freq) return;
        // pileup mode (-p) prints the reference allele of a position without
        // variants (src/modes/simpleMode.cpp:163-174)
        if (n_var == 0 && !(P.do_pileup && ref_i >= 0)) return;
    }
    // numeric pre-screen of isGoodVar: a necessary condition for emission
    bool any = false;
    for (int i = 0; i < nv; i++) {
        if (i == ref_i) continue;
        const V &v = vs[i];
        if (v.freq >= P.freq && v.hi >= P.minr && v.pmean >= P.read_pos_filter && v.qual >= P.goodq &&
            v.qratio >= P.qratio)
            any = true;
        if (P.dataset_min > 0 && v.cnt >= P.dataset_min) any = true;
    }
    if (!any && !P.do_pileup && !forced) return;
    // reference strand counts (collectReferenceVariants :730-760)
    int rfc = 0, rrc = 0;
    if (ref_i >= 0) { rfc = vs[ref_i].fwd; rrc = vs[ref_i].rev; }
    if (tpc > (int)st.cells.cov[c] && p + 1 <= R.chi) {
        int p1 = p + 1;
        int64_t g = 0;
        uint32_t rs = kNone;
        int w = (p1 >= R.ws && p1 <= R.we) ? ref_key_at(st, R, p1, base_index(ref_at(st, R, p1)), g, rs) : -1;
        if (w == 0) {
            rfc = (int)st.cells.fwd[g];
            rrc = (int)st.cells.rev[g];
        } else if (w == 1) {
            rfc = st.hash.slots[rs].fwd;
            rrc = st.hash.slots[rs].rev;
        }
    }
    unsigned int base = atomicAdd(st.n_cand, (unsigned int)nv);
    if (base + nv > st.cand_cap) { atomicOr(st.err, ERR_CAND_FULL); return; }
    int rank = 0;
    for (int i = 0; i < nv; i++) {
        const V &v = vs[i];
        CandVar &o = st.cand[base + i];
        o.region = lo;
        o.pos = p;
        o.kind = (i == ref_i) ? 0 : 1;
        o.rank = (i == ref_i) ? -1 : rank++;
        if (v.kind == 0) { o.key_off = v.key; o.key_len = -1; }
        else { const Slot &sl = st.hash.slots[v.key]; o.key_off = (int)sl.koff; o.key_len = sl.klen; }
        // raw counts (the record writers clamp negatives where the reference does)
        int fwd = v.fwd < 0 ? 0 : v.fwd, rev = v.rev < 0 ? 0 : v.rev;
        int rf = rfc < 0 ? 0 : rfc, rr = rrc < 0 ? 0 : rrc;
        o.pc = v.cnt;
        o.fwd = v.fwd;
        o.rev = v.rev;
        o.hicnt = v.hi;
        o.hicov = v.hicov;
        o.tpc = tpc;
        o.rfc = rfc;
        o.rrc = rrc;
        o.bias = v.bias;
        o.ref_bias = ref_i >= 0 ? vs[ref_i].bias : -1;
        o.pstd = v.pstd;
        o.qstd = v.qstd;
        o.pass = (v.freq >= P.freq && v.hi >= P.minr && v.pmean >= P.read_pos_filter && v.qual >= P.goodq &&
                  v.qratio >= P.qratio) ? 1 : 0;
        o.nvars = nv;
        o.freq = v.freq;
        o.pmean = v.pmean;
        o.qual = v.qual;
        o.mq = v.mqv;
        o.qratio = v.qratio;
        o.hifreq = v.hifreq;
        o.extrafreq = v.extrafreq;
        o.nm = v.nmv;
        // the records' Fisher test (src/modes/simpleMode.cpp:96-108): every
        // printed allele; pileup mode also prints alleles failing isGoodVar
        // and, at a position without variants, the reference allele with no
        // variant reads
        if (P.fisher && !P.somatic && !P.dataset_min && o.kind == 1 && (o.pass || P.do_pileup)) {
            o.fisher_p = fisher_two_sided(rf, rr, fwd, rev, st.logfact);
            double ad = (double)(rf * rev), bc = (double)(rr * fwd);
            o.fisher_ratio = (bc != 0 && ad != 0) ? (ad > bc ? ad / bc : bc / ad) : 0.0;
        } else if (P.fisher && !P.somatic && !P.dataset_min && o.kind == 0 && P.do_pileup && n_var == 0) {
            o.fisher_p = fisher_two_sided(rf, rr, 0, 0, st.logfact);
            o.fisher_ratio = 0.0;
        } else {
            o.fisher_p = 0;
            o.fisher_ratio = 0;
        }
    }
}

// Each block scores a contiguous chunk of positions; the region of the
// chunk start is found once and threads advance from it.
constexpr int kScoreChunk = 2048;

__global__ void k_score(DevState st, DevParams P) {
    __shared__ int s_lo;
    for (int64_t c0 = (int64_t)blockIdx.x * kScoreChunk; c0 < st.n_score; c0 += (int64_t)gridDim.x * kScoreChunk) {
        __syncthreads();
        if (threadIdx.x == 0) {
            int a = 0, b = st.n_regions - 1;
            while (a < b) {
                int mid = (a + b + 1) >> 1;
                if (st.score_base[mid] <= c0) a = mid; else b = mid - 1;
            }
            s_lo = a;
        }
        __syncthreads();
        const int lo0 = s_lo;
        for (int64_t t = c0 + threadIdx.x; t < c0 + kScoreChunk && t < st.n_score; t += blockDim.x) {
            int lo = lo0;
            while (lo + 1 < st.n_regions && st.score_base[lo + 1] <= t) lo++;
            V vs[kMaxVars];
            uint32_t ins[kMaxVars];
            score_position(st, P, lo, st.regions[lo].start + (int)(t - st.score_base[lo]), false, vs, kMaxVars, ins,
                           false);
        }
    }
}

// Listed (region, position) pairs, scored without screens: in somatic mode
// the positions where the other sample has a candidate.
__global__ void k_score_list(DevState st, DevParams P, const int2 *list, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int2 e = list[i];
        if (e.x < 0 || e.x >= st.n_regions) continue;
        const Region &R = st.regions[e.x];
        if (e.y < R.start || e.y > R.end) continue;
        V vs[kMaxVars];
        uint32_t ins[kMaxVars];
        score_position(st, P, e.x, e.y, true, vs, kMaxVars, ins, false);
    }
}

// The queued wide positions, one thread each, with their alleles and
// insertion keys in global scratch (off[i]: first scratch entry of entry i,
// from k_wide_offsets; the alleles in the first scratch_cap entries, the
// insertion keys after them).  Too little scratch: as k_ins_adjust_wide.
__global__ void k_score_wide(DevState st, DevParams P, const int64_t *off, V *v_scratch, uint32_t *ins_scratch,
                             int64_t scratch_cap) {
    unsigned int n = *st.n_wide_score;
    if (n > st.wide_cap) n = st.wide_cap;
    if (n == 0) return;
    if (off[n] > scratch_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(st.err, ERR_WIDE_SCORE_SCRATCH);
        return;
    }
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const WidePos w = st.wide_score[i];
        const int cap = (int)(off[i + 1] - off[i]);
        score_position(st, P, w.region, w.pos, w.forced != 0, v_scratch + off[i], cap, ins_scratch + off[i], true);
    }
}

size_t wide_entry_bytes() { return sizeof(V) + sizeof(uint32_t); }

void launch_wide_offsets(const DevState &st, int list, int64_t *off, cudaStream_t s) {
    k_wide_offsets<<<1, 1024, 0, s>>>(list == 0 ? st.wide_ins : st.wide_score,
                                      list == 0 ? st.n_wide_ins : st.n_wide_score, st.wide_cap, off);
}

// scratch: `entries` wide entries (wide_entry_bytes each)
void launch_ins_adjust_wide(const DevState &st, const int64_t *off, void *scratch, int64_t entries, cudaStream_t s) {
    k_ins_adjust_wide<<<64, 64, 0, s>>>(st, off, (uint32_t *)scratch, scratch ? entries : 0);
}

void launch_score_wide(const DevState &st, const DevParams &P, const int64_t *off, void *scratch, int64_t entries,
                       cudaStream_t s) {
    V *vs = (V *)scratch;
    uint32_t *ins = scratch ? (uint32_t *)(vs + entries) : nullptr;
    k_score_wide<<<64, 64, 0, s>>>(st, P, off, vs, ins, scratch ? entries : 0);
}

// Features of the learned filter: 40 floats per candidate allele, from its
// site statistics, its key and the reference around it.
__device__ int run_len(const DevState &st, const Region &R, int p, int dir) {
    char b = ref_at(st, R, p);
    if (!b) return 0;
    int n = 0;
    for (int q = p + dir; n < 20 && q >= R.ws && q <= R.we && st.ref[q - 1] == b; q += dir) n++;
    return n;
}

__global__ void k_features(DevState st, DevParams P, const CandVar *cand, int64_t n, float *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const CandVar c = cand[i];
        float *f = out + i * 40;
        const Region &R = st.regions[c.region];
        const int fwd = max(c.fwd, 0), rev = max(c.rev, 0), rf = max(c.rfc, 0), rr = max(c.rrc, 0);
        const float pc = (float)max(c.pc, 0), tpc = (float)max(c.tpc, 1);
        f[0] = log1pf((float)c.tpc) / 8.f;
        f[1] = log1pf(pc) / 8.f;
        f[2] = (float)c.freq;
        f[3] = log1pf((float)c.hicnt) / 8.f;
        f[4] = log1pf((float)c.hicov) / 8.f;
        f[5] = (float)c.hifreq;
        f[6] = pc > 0 ? fwd / pc : 0.5f;
        f[7] = rf + rr > 0 ? rf / (float)(rf + rr) : 0.5f;
        f[8] = c.bias * 0.5f;
        f[9] = c.ref_bias * 0.5f;
        f[10] = (float)c.pstd;
        f[11] = (float)c.qstd;
        f[12] = (float)c.pmean / 75.f;
        f[13] = (float)c.qual / 40.f;
        f[14] = (float)c.mq / 60.f;
        f[15] = log1pf((float)c.qratio) / 4.f;
        f[16] = (float)c.extrafreq;
        f[17] = (float)c.nm / 10.f;
        const double fp = fisher_two_sided(rf, rr, fwd, rev, st.logfact);
        f[18] = fminf(-log10f(fmaxf((float)fp, 1e-30f)), 30.f) / 10.f;
        const double ad = (double)rf * rev, bc = (double)rr * fwd;
        const double ratio = (bc != 0 && ad != 0) ? (ad > bc ? ad / bc : bc / ad) : 0.0;
        f[19] = log1pf((float)ratio) / 4.f;
        int kind = 0;  // 0 SNV, 1 MNV, 2 insertion, 3 deletion, 4 other
        int klen = 1;
        if (c.key_len >= 0) {
            const uint8_t *k = st.hash.arena + c.key_off;
            klen = c.key_len;
            if (k[0] == '+') kind = 2;
            else if (k[0] == '-') kind = 3;
            else if (klen > 2 && k[1] == '&') kind = 1;
            else kind = 4;
        }
        for (int j = 0; j < 5; j++) f[20 + j] = kind == j ? 1.f : 0.f;
        f[25] = klen / 20.f;
        f[26] = c.nvars / 8.f;
        f[27] = c.rank / 8.f;
        f[28] = c.rank == 0 ? 1.f : 0.f;
        f[29] = run_len(st, R, c.pos, -1) / 20.f;
        f[30] = run_len(st, R, c.pos, 1) / 20.f;
        int gc = 0, tot = 0, rep = 0;
        for (int q = c.pos - 20; q <= c.pos + 20; q++) {
            char b = ref_at(st, R, q);
            if (!b) continue;
            tot++;
            if (b == 'G' || b == 'C') gc++;
            if (q + 2 <= c.pos + 20 && b == ref_at(st, R, q + 2)) rep++;
        }
        f[31] = tot ? gc / (float)tot : 0.f;
        f[32] = rep / 40.f;
        f[33] = c.hicov / tpc;
        f[34] = pc > 0 ? c.hicnt / pc : 0.f;
        f[35] = (rf + rr) / tpc;
        f[36] = c.pc >= P.minr ? 1.f : 0.f;
        f[37] = c.freq >= P.freq ? 1.f : 0.f;
        f[38] = (float)c.pass;
        f[39] = log1pf((float)abs(fwd - rev)) / 8.f;
    }
}

void launch_features(const DevState &st, const DevParams &P, const CandVar *cand, int64_t n, float *out,
                     cudaStream_t s) {
    if (n > 0) k_features<<<(int)std::min<int64_t>((n + 127) / 128, 4096), 128, 0, s>>>(st, P, cand, n, out);
}

// Batched Fisher tests (rv_fisher_batch): one warp per table.  The lanes
// split the hypergeometric terms x = lo, lo + 1, ..., hi (a deep table has
// thousands, each an FP64 exp) and the partial sums are added by shuffles;
// the same terms and tie slack as fisher_two_sided, summed in another order.
__global__ void k_fisher(const int32_t *tab, int64_t n, double *p2, double *ratio, const double *lf) {
    const int lane = (int)(threadIdx.x & 31u);
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const int a = tab[4 * i], b = tab[4 * i + 1], c = tab[4 * i + 2], d = tab[4 * i + 3];
        const int r1 = a + b, c1 = a + c, nn = a + b + c + d;
        const int lo = r1 + c1 - nn > 0 ? r1 + c1 - nn : 0;
        const int hi = r1 < c1 ? r1 : c1;
        double two;
        if (a < 0 || b < 0 || c < 0 || d < 0 || lo >= hi) {
            two = 1.0;
        } else if (!lf || nn >= kLogFact) {
            two = fisher_two_sided(a, b, c, d, lf);  // (no table: one lane, lgamma terms)
        } else {
            const double base = log_choose_t(lf, nn, c1);
            const double p_obs = exp(log_choose_t(lf, r1, a) + log_choose_t(lf, nn - r1, c1 - a) - base);
            const double thr = p_obs * (1.0 + 1e-7);
            double part = 0.0;
            for (int x = lo + lane; x <= hi; x += 32) {
                const double p = exp(log_choose_t(lf, r1, x) + log_choose_t(lf, nn - r1, c1 - x) - base);
                if (p <= thr) part += p;
            }
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
            two = part > 1.0 ? 1.0 : part;
        }
        if (lane == 0) {
            p2[i] = two;
            const double ad = (double)a * d, bc = (double)b * c;
            ratio[i] = (bc != 0 && ad != 0) ? (ad > bc ? ad / bc : bc / ad) : 0.0;
        }
    }
}

__global__ void k_clear_err_bits(unsigned int *err, unsigned int keep) { atomicAnd(err, keep); }

void launch_clear_err_bits(const DevState &st, unsigned int keep, cudaStream_t s) {
    k_clear_err_bits<<<1, 1, 0, s>>>(st.err, keep);
}

void launch_link(const DevState &st, cudaStream_t s) { k_link_slots<<<592, 256, 0, s>>>(st); }
void launch_collisions(const DevState &st, cudaStream_t s) { k_check_collisions<<<592, 256, 0, s>>>(st); }
void launch_ins_adjust(const DevState &st, cudaStream_t s) {
    if (st.cells.n_cells > 0) k_ins_adjust<<<1216, 256, 0, s>>>(st);
}
void launch_score(const DevState &st, const DevParams &P, cudaStream_t s) {
    if (st.n_score > 0) {
        int64_t chunks = (st.n_score + kScoreChunk - 1) / kScoreChunk;
        k_score<<<(int)std::min<int64_t>(chunks, 4864), 256, 0, s>>>(st, P);
    }
}
void launch_score_list(const DevState &st, const DevParams &P, const int2 *list, int n, cudaStream_t s) {
    if (n > 0) k_score_list<<<(n + 127) / 128 < 1216 ? (n + 127) / 128 : 1216, 128, 0, s>>>(st, P, list, n);
}
void launch_fisher(const int32_t *tab, int64_t n, double *p2, double *ratio, cudaStream_t s, const double *lf) {
    if (n > 0)  // four tables (warps) per block
        k_fisher<<<(int)((n + 3) / 4 < 8192 ? (n + 3) / 4 : 8192), 128, 0, s>>>(tab, n, p2, ratio, lf);
}
void launch_fill_logfact(double *lf, cudaStream_t s) { k_fill_logfact<<<256, 256, 0, s>>>(lf, kLogFact); }

}  // namespace rv
