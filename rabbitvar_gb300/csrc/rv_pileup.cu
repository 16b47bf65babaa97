// Pileup kernels: the record filter, the per-read CIGAR walk and the
// allele-count maps (CigarParser::process, src/parseCigar.cpp:410-974).
//
//  * k_pileup_tiles: blocks pull tiles (a region's consecutive reads) from a
//    device work queue, a few each; each thread walks one read; A/C/G/T
//    observations go into a shared-memory histogram covering the tile's
//    window (kTileW positions), flushed to the per-position global cells once
//    per tile; string-keyed alleles (MNV, indels, soft clips) go to a global
//    open-addressing hash table.
//  * k_pileup_serial: regions whose reads reach outside the reference window
//    are walked in file order by one thread, reproducing the reference map's
//    insert-on-lookup behaviour exactly.
//  * k_resolve_deferred: decides, for every reference-base subtraction after
//    an insertion, whether that key existed when the insertion was seen (the
//    getVariationMaybe lookup of src/parseCigar.cpp:1475) by re-walking the
//    same and earlier reads, then applies it.
#include <cuda_runtime.h>

#include <algorithm>

#include "rv_walk.cuh"

namespace rv {

__device__ __forceinline__ void set_err(unsigned int *err, unsigned int bits) { atomicOr(err, bits); }

// ---------------------------------------------------------------------------
// device hash table of string-keyed alleles
// ---------------------------------------------------------------------------
__device__ Slot *hash_get(const Hash &H, unsigned int *err, int region, int kind, int pos, const char *k, int n) {
    unsigned long long h1, h2;
    key_hashes(region, kind, pos, k, n, h1, h2);
    unsigned long long i = h1 & H.mask;
    for (int step = 0; step <= 4096; step++) {
        Slot *s = &H.slots[i];
        unsigned long long old = atomicCAS(&s->fp, 0ULL, h1);
        if (old == 0ULL) {
            s->region = region;
            s->pos = pos;
            s->kind = (uint16_t)kind;
            s->klen = (uint16_t)n;
            unsigned long long off = n ? atomicAdd(H.arena_used, (unsigned long long)n) : 0ULL;
            if (off + n > H.arena_cap) {
                set_err(err, ERR_ARENA_FULL);
                s->koff = 0;
                s->klen = 0;
            } else {
                s->koff = (uint32_t)off;
                for (int j = 0; j < n; j++) H.arena[off + j] = (uint8_t)k[j];
            }
            note_used(H, i);
            atomicXor(&s->h2x, h2);
            return s;
        }
        if (old == h1) {
            atomicXor(&s->h2x, h2);
            return s;
        }
        i = (i + 1) & H.mask;
    }
    set_err(err, ERR_HASH_FULL);
    return nullptr;
}

// Queues a map entry for the in-order replay of its pstd/qstd (k_fix_order).
__device__ void push_order_fix(const DevState &st, int region, int pos, int base, int64_t index) {
    unsigned int k = atomicAdd(st.n_ofix, 1u);
    if (k >= st.ofix_cap) { set_err(st.err, ERR_FIX_FULL); return; }
    OrderFix f;
    f.region = region;
    f.pos = pos;
    f.base = base;
    f.pad = 0;
    f.index = index;
    st.ofix[k] = f;
}

__device__ void slot_obs(const DevState &st, Slot *s, const Obs &o, double goodq, uint32_t stamp) {
    if (o.dir) atomicAdd(&s->rev, 1); else atomicAdd(&s->fwd, 1);
    if (o.q >= goodq) atomicAdd(&s->hi, 1); else atomicAdd(&s->lo, 1);
    atomicAdd((unsigned long long *)&s->tp_sum, (unsigned long long)(long long)o.tp);
    atomicAdd(&s->q_sum, o.q);
    atomicAdd((unsigned long long *)&s->mq_sum, (unsigned long long)(long long)o.mapq);
    atomicAdd((unsigned long long *)&s->nm_sum, (unsigned long long)(long long)o.nm);
    if (o.creates) atomicAdd(&s->obs, 1);
    atomicMin(&s->min_stamp, stamp);
    if (o.std_rel) {
        // pstd/qstd (src/parseCigar.cpp:902-914): "not all values equal", tested
        // against whichever observation claimed the first slot
        int old_tp = atomicCAS(&s->first_tp, INT32_MIN, o.tp);
        if (old_tp != INT32_MIN && old_tp != o.tp) atomicOr(&s->flags, SF_PDIFF);
        unsigned long long qb = (unsigned long long)__double_as_longlong(o.q);
        unsigned long long old_q = atomicCAS(&s->first_q, 0xFFF8DEADBEEF0001ULL, qb);
        if (old_q != 0xFFF8DEADBEEF0001ULL && old_q != qb) atomicOr(&s->flags, SF_QDIFF);
        if (o.tp == 0 || o.q == 0.0) {
            if (!(atomicOr(&s->flags, SF_ZERO) & SF_ZERO))
                push_order_fix(st, s->region, s->pos, -1, (int64_t)(s - st.hash.slots));
        }
    }
}

__device__ __forceinline__ void clear_slot(Slot &s) {
    s.fp = 0;
    s.h2x = 0;
    s.region = 0;
    s.pos = 0;
    s.kind = 0;
    s.klen = 0;
    s.koff = 0;
    s.fwd = s.rev = s.hi = s.lo = s.obs = s.extracnt = 0;
    s.tp_sum = s.mq_sum = s.nm_sum = 0;
    s.q_sum = 0.0;
    s.first_q = 0xFFF8DEADBEEF0001ULL;
    s.first_tp = INT32_MIN;
    s.flags = 0;
    s.min_stamp = 0xFFFFFFFFu;
    s.next = 0xFFFFFFFFu;
}

// Whole table (a table just allocated).
__global__ void k_init_slots(Slot *slots, unsigned long long n) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        clear_slot(slots[i]);
}

// Only the slots the previous run claimed (its used-slot list); the count is
// read before the counters are reset.
__global__ void k_clear_used(Slot *slots, const uint32_t *used, const unsigned int *n_used,
                             unsigned long long cap) {
    unsigned long long n = *n_used;
    if (n > cap) n = cap;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        clear_slot(slots[used[i]]);
}

// ---------------------------------------------------------------------------
// per-position cells
// ---------------------------------------------------------------------------
// packed first (tp, q) of pstd-relevant observations: tp in bits 0-11,
// q in bits 12-21, bit 29 zero-seen, bit 30 pdiff, bit 31 qdiff
constexpr uint32_t FC_ZERO = 1u << 29, FC_PDIFF = 1u << 30, FC_QDIFF = 1u << 31;
constexpr uint32_t FC_VAL = (1u << 22) - 1;

__device__ __forceinline__ void first_merge(uint32_t *w, uint32_t v, uint32_t flags) {
    // v: packed value (nonzero); merge into word *w.  Flag bits may change
    // concurrently, so retry the claim while the value field is still empty
    // (bounded: each retry means another thread changed the word).
    uint32_t cur = *((volatile uint32_t *)w);
    for (int it = 0; it < 64 && (cur & FC_VAL) == 0; it++) {
        uint32_t old = atomicCAS(w, cur, cur | v);
        if (old == cur) { cur |= v; break; }
        cur = old;
    }
    uint32_t f = flags;
    uint32_t cv = cur & FC_VAL;
    if (cv != 0 && cv != v) {
        if ((cv & 0xFFFu) != (v & 0xFFFu)) f |= FC_PDIFF;
        if ((cv >> 12) != (v >> 12)) f |= FC_QDIFF;
    }
    if (f & ~cur) atomicOr(w, f);
}

__device__ __forceinline__ int64_t cell_of(const Region &R, int p) { return R.cell_base + (p - R.clo); }

// Direct global update of one A/C/G/T observation (outside a tile window, or
// the in-order walker).
__device__ void cell_obs_global(const DevState &st, int region, const Region &R, int p, int b, const Obs &o,
                                double goodq) {
    const Cells &C = st.cells;
    unsigned int *err = st.err;
    if (p < R.clo || p > R.chi) { set_err(err, ERR_CELL_RANGE); return; }
    int64_t c = cell_of(R, p);
    int64_t g = 4 * c + b;
    int qi = (int)o.q;
    if (o.dir) atomicAdd(&C.rev[g], 1u); else atomicAdd(&C.fwd[g], 1u);
    if (o.q >= goodq) atomicAdd(&C.hi[g], 1u);
    atomicAdd(&C.tp[g], (uint32_t)o.tp);
    atomicAdd(&C.q[g], (uint32_t)qi);
    atomicAdd(&C.mq[g], (uint32_t)o.mapq);
    atomicAdd(&C.nm[g], o.nm);
    atomicAdd(&C.cov[c], 1u);
    atomicOr((unsigned int *)&C.kflags[c & ~3LL], 1u << (b + 8 * (c & 3)));
    if (o.std_rel) {
        if (o.tp <= 0 || o.tp > 4095 || qi <= 0 || qi > 1023) {
            // outside the packed value range (a zero among them): replayed in
            // read order after the pileup
            if (!(atomicOr(&C.first[g], FC_ZERO) & FC_ZERO)) push_order_fix(st, region, p, b, g);
        } else {
            first_merge(&C.first[g], (uint32_t)o.tp | ((uint32_t)qi << 12), 0u);
        }
    }
}

// ---------------------------------------------------------------------------
// sinks
// ---------------------------------------------------------------------------
struct SinkBase {
    const DevState *st;
    const DevParams *P;
    const Region *R;
    int region_idx;
    __device__ bool done() const { return false; }  // the walk may stop early (no: every observation counts)
    __device__ void error(unsigned int bits) { set_err(st->err, bits); }
    __device__ void cov(int p, int n) {
        if (p < R->clo || p > R->chi) { error(ERR_CELL_RANGE); return; }
        atomicAdd(&st->cells.cov[cell_of(*R, p)], (uint32_t)n);
    }
    __device__ void event(int kind, int pos, const char *k, int n, const Obs &o, int64_t read) {
        Slot *s = hash_get(st->hash, st->err, region_idx, kind, pos, k, n);
        if (s) slot_obs(*st, s, o, P->goodq, (uint32_t)read);
    }
    // maxReadLength: every read of a region would hit the same word, so the
    // atomic is taken only when the read is longer than the value seen
    __device__ void max_len(int tlen) {
        if (tlen > *(const volatile int *)&R->max_read_len) atomicMax((int *)&R->max_read_len, tlen);
    }
};

// Tile-histogram packing of one (position, base) cell in shared memory,
// three 32-bit words (32-bit shared atomics are native; 64-bit ones are not):
//   w0: fwd (bits 0-9) | rev (10-19) | hi (20-29)
//   w1: tp (bits 0-16) | q (17-31)
//   w2: mapq (bits 0-15) | nm + 128 (16-31)
// valid for tiles of at most kTileReads (256) reads, one observation per read
// and position, tp in 1..511, q in 1..127, mapq <= 255, nm in -128..127;
// anything else goes straight to the global cells.  The word arrays are
// addressed in the shared state space (the generic forms cannot be proven not
// to alias the walker's local-memory object).
__device__ __forceinline__ void shared_add_u32(uint32_t addr, uint32_t v) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(v));
}
__device__ __forceinline__ uint32_t shared_ld_u32(uint32_t addr) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}
__device__ __forceinline__ void shared_or_u32(uint32_t addr, uint32_t v) {
    asm volatile("red.shared.or.b32 [%0], %1;" ::"r"(addr), "r"(v));
}
__device__ __forceinline__ uint32_t shared_cas_u32(uint32_t addr, uint32_t cmp, uint32_t v) {
    uint32_t old;
    asm volatile("atom.shared.cas.b32 %0, [%1], %2, %3;" : "=r"(old) : "r"(addr), "r"(cmp), "r"(v));
    return old;
}

__device__ __forceinline__ uint32_t shared_ld_u8(uint32_t addr) {
    uint32_t v;
    asm volatile("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}

// AGG: lanes of a warp that emit into the same (position, base) cell at
// the same time (reads starting at the same position, as in deep pileups)
// are found with __match_any_sync; their three packed words are summed with
// warp reductions and one lane does the shared atomics and the first-value
// check for the group.
template <bool AGG>
struct TileFast {
    uint32_t w_s;       // shared-space address of the word arrays (w0 | w1 | w2 | first, 4*kTileW words each)
    uint32_t ref_s;     // shared-space address of the reference bases wlo .. wlo + kTileW - 1
    uint32_t code_s;    // and of their codes (ref_code_of)
    int wlo;
    int goodq;          // integer quality threshold (DevParams::goodq_i)
    // reference base at p (inside the region's window): from the tile's shared copy
    __device__ __forceinline__ char ref(const char *refp, int p) const {
        unsigned d = (unsigned)(p - wlo);
        return d < (unsigned)kTileW ? (char)shared_ld_u8(ref_s + d) : __ldg(refp + p - 1);
    }
    // its code (ref_code_of), from the tile's shared copy of the codes
    __device__ __forceinline__ int ref_code(const char *refp, int p) const {
        unsigned d = (unsigned)(p - wlo);
        return d < (unsigned)kTileW ? (int)shared_ld_u8(code_s + d) : ref_code_of(__ldg(refp + p - 1));
    }
    __device__ __forceinline__ bool emit(int p, int b, int dir, int tp, int q, int mapq, int nm) const {
        if (AGG) return emit_warp(p, b, dir, tp, q, mapq, nm);
        return emit_any(p, b, dir, tp, q, mapq, nm, true);
    }
    // The observation of each active lane, aggregated over the lanes that hit
    // the same cell; lanes whose observation does not fit the packing return
    // false (the caller's global path).
    __device__ __forceinline__ bool emit_warp(int p, int b, int dir, int tp, int q, int mapq, int nm) const {
        const unsigned d = (unsigned)(p - wlo);
        const bool ok = d < (unsigned)kTileW && (unsigned)(tp - 1) <= 510u && (unsigned)(q - 1) <= 126u &&
                        (unsigned)mapq <= 255u && (unsigned)(nm + 128) <= 255u;
        const unsigned act = __activemask();
        const unsigned okm = __ballot_sync(act, ok);
        if (!ok) return false;
        const uint32_t ix = 4u * d + (uint32_t)b;
        const unsigned peers = __match_any_sync(okm, ix);
        const uint32_t v0 = (dir ? (1u << 10) : 1u) + (q >= goodq ? (1u << 20) : 0u);
        const uint32_t v1 = (uint32_t)tp | ((uint32_t)q << 17);
        const uint32_t v2 = (uint32_t)mapq | ((uint32_t)(nm + 128) << 16);
        const uint32_t s0 = __reduce_add_sync(peers, v0);
        const uint32_t s1 = __reduce_add_sync(peers, v1);
        const uint32_t s2 = __reduce_add_sync(peers, v2);
        int same_tp = 0, same_q = 0;
        __match_all_sync(peers, tp, &same_tp);
        __match_all_sync(peers, q, &same_q);
        const int lane = (int)(threadIdx.x & 31u);
        if (lane != __ffs(peers) - 1) return true;
        const uint32_t a0 = w_s + 4u * ix;
        constexpr uint32_t kArr = 4u * 4u * kTileW;  // bytes per word array
        shared_add_u32(a0, s0);
        shared_add_u32(a0 + kArr, s1);
        shared_add_u32(a0 + 2u * kArr, s2);
        const uint32_t v = (uint32_t)tp | ((uint32_t)q << 12);
        const uint32_t fa = a0 + 3u * kArr;
        uint32_t need = (same_tp ? 0u : FC_PDIFF) | (same_q ? 0u : FC_QDIFF);
        uint32_t f = shared_ld_u32(fa);
        bool claimed = false;
        for (int it = 0; it < 64 && (f & FC_VAL) == 0u; it++) {
            uint32_t old = shared_cas_u32(fa, f, f | v);
            if (old == f) { claimed = true; f |= v; break; }
            f = old;
        }
        if (!claimed) {
            const uint32_t fv = f & FC_VAL;
            if ((fv & 0xFFFu) != (v & 0xFFFu)) need |= FC_PDIFF;
            if ((fv >> 12) != (v >> 12)) need |= FC_QDIFF;
        }
        if (need & ~f) shared_or_u32(fa, need);
        return true;
    }
    // std_rel: the observation takes part in pstd/qstd (M-op bases do, the
    // soft-clip re-alignment counts do not)
    __device__ __forceinline__ bool emit_any(int p, int b, int dir, int tp, int q, int mapq, int nm, bool std_rel) const {
        unsigned d = (unsigned)(p - wlo);
        if (d >= (unsigned)kTileW || (unsigned)(tp - 1) > 510u || (unsigned)(q - 1) > 126u || (unsigned)mapq > 255u ||
            (unsigned)(nm + 128) > 255u)
            return false;
        const uint32_t ix = 4u * d + (uint32_t)b;
        const uint32_t a0 = w_s + 4u * ix;
        constexpr uint32_t kArr = 4u * 4u * kTileW;  // bytes per word array
        shared_add_u32(a0, (dir ? (1u << 10) : 1u) + (q >= goodq ? (1u << 20) : 0u));
        shared_add_u32(a0 + kArr, (uint32_t)tp | ((uint32_t)q << 17));
        shared_add_u32(a0 + 2u * kArr, (uint32_t)mapq | ((uint32_t)(nm + 128) << 16));
        if (!std_rel) return true;
        const uint32_t v = (uint32_t)tp | ((uint32_t)q << 12);
        const uint32_t fa = a0 + 3u * kArr;
        uint32_t f = shared_ld_u32(fa);
        // claim the value slot if empty (bounded retries: flag bits may change)
        for (int it = 0; it < 64 && (f & FC_VAL) == 0u; it++) {
            uint32_t old = shared_cas_u32(fa, f, f | v);
            if (old == f) return true;
            f = old;
        }
        const uint32_t fv = f & FC_VAL;
        uint32_t need = 0u;
        if (!(f & FC_PDIFF) && (fv & 0xFFFu) != (v & 0xFFFu)) need |= FC_PDIFF;
        if (!(f & FC_QDIFF) && (fv >> 12) != (v >> 12)) need |= FC_QDIFF;
        if (need) shared_or_u32(fa, need);
        return true;
    }
};

// Tile sink: A/C/G/T observations inside [wlo, wlo + kTileW) accumulate in
// shared memory; subtractions are deferred.
template <bool AGG>
struct TileSink : SinkBase {
    TileFast<AGG> f;
    using Fast = TileFast<AGG>;
    __device__ Fast fast() const { return f; }
    __device__ bool phantom(int) const { return false; }
    // Positions below 1 never get queried by the walk; above the window only
    // edge reads of regions marked for the in-order walk can reach.
    __device__ void touch_phantom(int p) {
        if (p >= 1) error(ERR_UNSUPPORTED);
    }
    __device__ void single(int p, int b, const Obs &o, int64_t) {
        if (f.emit_any(p, b, o.dir, o.tp, (int)o.q, o.mapq, o.nm, o.std_rel)) return;
        cell_obs_global(*st, region_idx, *R, p, b, o, P->goodq);
    }
    __device__ void subtract(int p, int b, int dir, int tp, int q, int mapq, int nm, int64_t read, int ci) {
        unsigned int k = atomicAdd(st->n_deferred, 1u);
        if (k >= st->deferred_cap) { error(ERR_DEFER_FULL); return; }
        Deferred &d = st->deferred[k];
        d.region = region_idx; d.pos = p; d.read = read; d.ci = ci; d.base = b;
        d.dir = dir; d.tp = tp; d.q = q; d.mapq = mapq; d.nm = nm; d.pad = 0;
    }
};

__device__ void apply_subtract(const Cells &C, const Region &R, unsigned int *err, int p, int b, int dir, int tp,
                               int q, int mapq, int nm, double goodq) {
    if (p < R.clo || p > R.chi) { set_err(err, ERR_CELL_RANGE); return; }
    int64_t g = 4 * cell_of(R, p) + b;
    if (dir) atomicSub(&C.rev[g], 1u); else atomicSub(&C.fwd[g], 1u);
    if (q >= goodq) atomicSub(&C.hi[g], 1u);
    atomicSub(&C.tp[g], (uint32_t)tp);
    atomicSub(&C.q[g], (uint32_t)q);
    atomicSub(&C.mq[g], (uint32_t)mapq);
    atomicSub(&C.nm[g], nm);
}

// In-order sink for the exact serial walker.
struct SerialSink : SinkBase {
    using Fast = NoFast;
    __device__ Fast fast() const { return Fast(); }
    uint32_t *ph_hi;   // bitmap of inserted positions above the window
    uint32_t *ph_lo;   // bitmap of inserted positions below the window
    static constexpr int kPh = 4096;
    __device__ bool phantom(int p) const {
        if (p > R->we) { int d = p - R->we - 1; return d < kPh && ((ph_hi[d >> 5] >> (d & 31)) & 1u); }
        if (p < R->ws) { int d = R->ws - 1 - p; return d < kPh && ((ph_lo[d >> 5] >> (d & 31)) & 1u); }
        return false;
    }
    __device__ void touch_phantom(int p) {
        if (p > R->we) {
            int d = p - R->we - 1;
            if (d < kPh) ph_hi[d >> 5] |= 1u << (d & 31); else error(ERR_UNSUPPORTED);
        } else if (p < R->ws) {
            int d = R->ws - 1 - p;
            if (d < kPh) ph_lo[d >> 5] |= 1u << (d & 31); else error(ERR_UNSUPPORTED);
        }
    }
    __device__ void single(int p, int b, const Obs &o, int64_t) {
        cell_obs_global(*st, region_idx, *R, p, b, o, P->goodq);
    }
    // existence of the key is decided in read order by k_resolve_deferred
    __device__ void subtract(int p, int b, int dir, int tp, int q, int mapq, int nm, int64_t read, int ci) {
        unsigned int k = atomicAdd(st->n_deferred, 1u);
        if (k >= st->deferred_cap) { error(ERR_DEFER_FULL); return; }
        Deferred &d = st->deferred[k];
        d.region = region_idx; d.pos = p; d.read = read; d.ci = ci; d.base = b;
        d.dir = dir; d.tp = tp; d.q = q; d.mapq = mapq; d.nm = nm; d.pad = 0;
    }
};

// A read is an edge read when its walk may look up reference positions past
// the loaded window (the reference's map then inserts 0 entries that later
// lookups see); edge reads of a region are walked in file order by one thread.
__device__ __forceinline__ bool is_edge(const Region &R, int span_hi) { return span_hi + kEdgeMargin > R.we; }

// Probe sink: reports whether the walked read creates key (pos, base) before
// it reaches the insertion (read, ci) that asked.
struct ProbeSink {
    using Fast = NoFast;
    __device__ Fast fast() const { return Fast(); }
    const Region *R;
    int pos, base;
    int64_t stop_read;
    int stop_ci;
    bool stopped, found;
    // the answer is known once the key was seen or the asking insertion reached
    __device__ bool done() const { return found || stopped; }
    __device__ bool phantom(int) const { return false; }
    __device__ void touch_phantom(int) {}
    __device__ void error(unsigned int) {}
    __device__ void cov(int, int) {}
    __device__ void event(int, int, const char *, int, const Obs &, int64_t) {}
    __device__ void max_len(int) {}
    __device__ void single(int p, int b, const Obs &, int64_t) {
        if (!stopped && p == pos && b == base) found = true;
    }
    __device__ void subtract(int, int, int, int, int, int, int, int64_t read, int ci) {
        if (read == stop_read && ci == stop_ci) stopped = true;
    }
};

// Detection sink for edge reads: records whether the walk would insert a
// 0 entry past the reference window (the only way the in-order semantics can
// differ from a parallel walk); produces nothing else.
struct DetectSink {
    using Fast = NoFast;
    __device__ Fast fast() const { return Fast(); }
    const Region *R;
    int *hit;
    __device__ bool done() const { return false; }
    __device__ bool phantom(int) const { return false; }
    __device__ void touch_phantom(int p) {
        if (p > R->we) atomicExch(hit, 1);
    }
    __device__ void error(unsigned int) {}
    __device__ void cov(int, int) {}
    __device__ void event(int, int, const char *, int, const Obs &, int64_t) {}
    __device__ void max_len(int) {}
    __device__ void single(int, int, const Obs &, int64_t) {}
    __device__ void subtract(int, int, int, int, int, int, int, int64_t, int) {}
};

// Replay sink of k_fix_order: follows one map entry's observations in read
// order and applies the reference's pstd/qstd rule to them ("set when the
// value differs from the previous one and the previous one is nonzero",
// src/parseCigar.cpp:902-914 for M-op keys, 1446-1451 for insertions, and
// the same rule for deletions).  On the edge reads of a region the in-order
// walker handles, the reference map's insert-on-lookup past the window is
// emulated as k_pileup_serial does.
struct OrderSink {
    using Fast = NoFast;
    __device__ Fast fast() const { return Fast(); }
    const Region *R;
    int region_idx;
    int pos, base, kind;        // base >= 0: A/C/G/T cell key; base < 0: slot of `kind` with fingerprint fp
    unsigned long long fp;
    bool track;                 // emulate insert-on-lookup (an edge read of an in-order region)
    uint32_t *ph_hi, *ph_lo;    // SerialSink::kPh bits each
    int pp;
    double pq;
    bool pstd, qstd;
    __device__ bool done() const { return false; }
    __device__ bool phantom(int p) const {
        if (!track) return false;
        if (p > R->we) { int d = p - R->we - 1; return d < SerialSink::kPh && ((ph_hi[d >> 5] >> (d & 31)) & 1u); }
        if (p < R->ws) { int d = R->ws - 1 - p; return d < SerialSink::kPh && ((ph_lo[d >> 5] >> (d & 31)) & 1u); }
        return false;
    }
    __device__ void touch_phantom(int p) {
        if (!track) return;
        if (p > R->we) {
            int d = p - R->we - 1;
            if (d < SerialSink::kPh) ph_hi[d >> 5] |= 1u << (d & 31);
        } else if (p < R->ws) {
            int d = R->ws - 1 - p;
            if (d < SerialSink::kPh) ph_lo[d >> 5] |= 1u << (d & 31);
        }
    }
    __device__ void take(const Obs &o) {
        if (!pstd && pp != 0 && o.tp != pp) pstd = true;
        if (!qstd && pq != 0.0 && o.q != pq) qstd = true;
        pp = o.tp;
        pq = o.q;
    }
    __device__ void error(unsigned int) {}
    __device__ void cov(int, int) {}
    __device__ void max_len(int) {}
    __device__ void subtract(int, int, int, int, int, int, int, int64_t, int) {}
    __device__ void single(int p, int b, const Obs &o, int64_t) {
        if (base >= 0 && p == pos && b == base && o.std_rel) take(o);
    }
    __device__ void event(int k, int p, const char *key, int n, const Obs &o, int64_t) {
        if (base >= 0 || p != pos || k != kind || !o.std_rel) return;
        unsigned long long h1, h2;
        key_hashes(region_idx, k, p, key, n, h1, h2);
        if (h1 == fp) take(o);
    }
};

// Record filters of next_record (src/recordPreprocessor.cpp:101-180) plus the
// region-overlap test of sam_itr_querys.
__device__ bool read_passes(const Batch &B, const DevParams &P, const Region &R, int64_t r) {
    int pos = B.pos[r];
    if (pos >= R.end) return false;
    const uint32_t *c = B.cigar + B.cig_off[r];
    int n = B.n_cigar[r], span = 0;
    for (int k = 0; k < n; k++) {
        int o = cig_op(__ldg(c + k));
        if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) span += cig_len(__ldg(c + k));
    }
    int flag = B.flag[r];
    int endpos = ((flag & 4) || span == 0) ? pos + 1 : pos + span;
    if (endpos <= R.start - 1) return false;
    if (flag & P.samfilter) return false;
    if ((int)B.mapq[r] < P.min_mapq) return false;
    if (B.l_qseq[r] == 1) return false;
    if (B.skip && B.skip[r]) return false;
    return true;
}

// read span incl. soft clips, used for tile windows
// With -k 1 (`widen`) the CIGAR rewrite can turn insertions into soft clips
// that reach further out: the span grows by the read's inserted bases.
__device__ void read_span(const Batch &B, int64_t r, int &lo, int &hi, bool widen = false) {
    const uint32_t *c = B.cigar + B.cig_off[r];
    int n = B.n_cigar[r], span = 0, ins = 0;
    int clip5 = 0, clip3 = 0;
    for (int k = 0; k < n; k++) {
        uint32_t w = __ldg(c + k);
        int o = cig_op(w);
        if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) span += cig_len(w);
        if (o == 1) ins += cig_len(w);
    }
    if (!widen) ins = 0;
    if (n > 0) {
        uint32_t w0 = __ldg(c), w1 = __ldg(c + n - 1);
        if (cig_op(w0) == 4 || cig_op(w0) == 1) clip5 = cig_len(w0);
        if (cig_op(w1) == 4 || cig_op(w1) == 1) clip3 = cig_len(w1);
    }
    int pos1 = B.pos[r] + 1;
    lo = pos1 - clip5 - 1 - ins;
    hi = pos1 + span + clip3 + ins;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// The region fields the batch preparation computed from the read spans
// (span_lo/hi, serial) stay; only the per-launch edge flag is reset.
__global__ void k_region_reset(DevState st) {
    int reg = blockIdx.x * blockDim.x + threadIdx.x;
    if (reg < st.n_regions) st.regions[reg].edge_hit = 0;
}

template <int TW, int MINB, bool AGG>
__global__ void __launch_bounds__(kPileupThreads, MINB) k_pileup_tiles(DevState st, DevParams P, int quota) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *w0 = (uint32_t *)smem;
    uint32_t *w1 = w0 + 4 * TW;
    uint32_t *w2 = w1 + 4 * TW;
    uint32_t *first = w2 + 4 * TW;
    __shared__ int s_tile;
    __shared__ char s_ref[TW];
    __shared__ uint8_t s_code[TW];
    for (int done = 0; done < quota; done++) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(st.tile_counter, 1u);
        __syncthreads();
        int t = s_tile;
        if (t >= st.n_tiles) return;
        const Tile tile = st.tiles[t];
        const Region &R = st.regions[tile.region];
        // window start: the lowest span start of the tile's non-edge reads
        // (computed by the batch preparation from the same CIGAR arithmetic as read_span)
        const int wlo = tile.wlo;
        for (int i = threadIdx.x; i < 4 * 4 * TW; i += blockDim.x) w0[i] = 0u;
        for (int i = threadIdx.x; i < TW; i += blockDim.x) {
            const int64_t p = (int64_t)wlo + i;  // 1-based; the walk reads it only inside [ws, we]
            const char c = (p >= 1 && p <= st.ref_len) ? st.ref[p - 1] : (char)0;
            s_ref[i] = c;
            s_code[i] = (uint8_t)ref_code_of(c);
        }
        __syncthreads();
        TileSink<AGG> sink;
        sink.st = &st;
        sink.P = &P;
        sink.R = &R;
        sink.region_idx = tile.region;
        sink.f.w_s = (uint32_t)__cvta_generic_to_shared(w0);
        sink.f.wlo = wlo;
        sink.f.ref_s = (uint32_t)__cvta_generic_to_shared(s_ref);
        sink.f.code_s = (uint32_t)__cvta_generic_to_shared(s_code);
        sink.f.goodq = P.goodq_i;
        {
            Walker<TileSink<AGG>> w(P, sink, R, st.ref, st.ref_len);
            // lane-strided read order: warp w, lane l walks the tile's read
            // 8 l + w, so a warp's lanes hold reads spread over the whole tile
            // (consecutive reads of a deep pileup start at the same position
            // and would hit the same histogram words together)
            static_assert(kTileReads == 256 && kPileupThreads == 256, "tile read permutation");
            const int64_t k = (int64_t)((threadIdx.x & 31u) * 8u + (threadIdx.x >> 5));
            for (int64_t e = tile.r0 + k; e < tile.r1; e += blockDim.x) {
                const int64_t r = st.tile_reads[e];
                if (!read_passes(st.batch, P, R, r)) continue;
                if (R.serial && R.edge_hit) {
                    int a, b;
                    read_span(st.batch, r, a, b, P.local_realign != 0);
                    if (is_edge(R, b)) continue;
                }
                w.walk(st.batch, r);
            }
        }
        __syncthreads();
        // flush the tile histogram into the global cells
        const Cells &C = st.cells;
        for (int i = threadIdx.x; i < 4 * TW; i += blockDim.x) {
            uint32_t c = w0[i];
            if (c == 0u) continue;
            int p = wlo + (i >> 2);
            int b = i & 3;
            if (p > R.chi) { set_err(st.err, ERR_CELL_RANGE); continue; }
            int64_t cell = cell_of(R, p);
            int64_t g = 4 * cell + b;
            uint32_t f = c & 0x3FFu, rv_ = (c >> 10) & 0x3FFu, h = (c >> 20) & 0x3FFu;
            uint32_t s1 = w1[i], s2 = w2[i];
            int nmsum = (int)(s2 >> 16) - 128 * (int)(f + rv_);
            if (f) atomicAdd(&C.fwd[g], f);
            if (rv_) atomicAdd(&C.rev[g], rv_);
            if (h) atomicAdd(&C.hi[g], h);
            atomicAdd(&C.tp[g], s1 & 0x1FFFFu);
            atomicAdd(&C.q[g], s1 >> 17);
            atomicAdd(&C.mq[g], s2 & 0xFFFFu);
            if (nmsum) atomicAdd(&C.nm[g], nmsum);
            atomicAdd(&C.cov[cell], f + rv_);
            atomicOr((unsigned int *)&C.kflags[cell & ~3LL], 1u << (b + 8 * (cell & 3)));
            uint32_t fw = first[i];
            if (fw) first_merge(&C.first[g], fw & FC_VAL, fw & ~FC_VAL);
        }
        __syncthreads();
    }
}

// For regions with edge reads: walk the edge reads in parallel with the
// detection sink; if none would touch a position past the window, the
// parallel walk is exact and the region leaves the in-order path.
// kEdgeBlocks blocks per region, each over a slice of the reads near the
// window end.
constexpr int kEdgeBlocks = 16;
__global__ void k_edge_detect(DevState st, DevParams P) {
    int reg = blockIdx.x / kEdgeBlocks, part = blockIdx.x % kEdgeBlocks;
    if (reg >= st.n_regions) return;
    Region &R = st.regions[reg];
    if (!R.serial) return;
    __shared__ int hit;
    if (threadIdx.x == 0) hit = 0;
    __syncthreads();
    // the first read that can reach within kEdgeMargin of the window end
    // (R.reach: the farthest any read of the region reaches past its start)
    int64_t lo = R.r0, hi = R.r1;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (st.batch.pos[mid] + 1 + R.reach + kEdgeMargin <= R.we) lo = mid + 1; else hi = mid;
    }
    DetectSink sink;
    sink.R = &R;
    sink.hit = &hit;
    Walker<DetectSink> w(P, sink, R, st.ref, st.ref_len);
    for (int64_t r = lo + part * (int64_t)blockDim.x + threadIdx.x; r < R.r1; r += (int64_t)kEdgeBlocks * blockDim.x) {
        if (!read_passes(st.batch, P, R, r)) continue;
        int a, b;
        read_span(st.batch, r, a, b, P.local_realign != 0);
        if (!is_edge(R, b)) continue;
        w.walk(st.batch, r);
    }
    __syncthreads();
    if (threadIdx.x == 0 && hit != 0) atomicOr(&R.edge_hit, 1);
}

// One block per region with edge reads; thread 0 walks them in file order.
__global__ void k_pileup_serial(DevState st, DevParams P) {
    int reg = blockIdx.x;
    if (reg >= st.n_regions) return;
    const Region &R = st.regions[reg];
    if (!R.serial || !R.edge_hit) return;
    __shared__ uint32_t ph_hi[SerialSink::kPh / 32], ph_lo[SerialSink::kPh / 32];
    for (int i = threadIdx.x; i < SerialSink::kPh / 32; i += blockDim.x) { ph_hi[i] = 0; ph_lo[i] = 0; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    SerialSink sink;
    sink.st = &st;
    sink.P = &P;
    sink.R = &R;
    sink.region_idx = reg;
    sink.ph_hi = ph_hi;
    sink.ph_lo = ph_lo;
    Walker<SerialSink> w(P, sink, R, st.ref, st.ref_len);
    // edge reads are the ones that can reach within kEdgeMargin of the window
    // end (reads are coordinate sorted; R.reach is the farthest any read of
    // the region reaches past its start): the first by binary search
    int64_t lo = R.r0, hi = R.r1;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (st.batch.pos[mid] + 1 + R.reach + kEdgeMargin <= R.we) lo = mid + 1; else hi = mid;
    }
    for (int64_t r = lo; r < R.r1; r++) {
        if (!read_passes(st.batch, P, R, r)) continue;
        int a, b;
        read_span(st.batch, r, a, b, P.local_realign != 0);
        if (!is_edge(R, b)) continue;
        w.walk(st.batch, r);
    }
}

// One thread per deferred subtraction.
__global__ void k_resolve_deferred(DevState st, DevParams P, int max_probe_reads) {
    unsigned int n = *st.n_deferred;
    if (n > st.deferred_cap) n = st.deferred_cap;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const Deferred d = st.deferred[k];
        const Region &R = st.regions[d.region];
        ProbeSink ps;
        ps.R = &R;
        ps.pos = d.pos;
        ps.base = d.base;
        ps.stop_read = d.read;
        ps.stop_ci = d.ci;
        ps.stopped = false;
        ps.found = false;
        Walker<ProbeSink> w(P, ps, R, st.ref, st.ref_len);
        w.walk(st.batch, d.read);
        int probes = 0;
        for (int64_t r = d.read - 1; !ps.found && r >= R.r0; r--) {
            int a, b;
            read_span(st.batch, r, a, b, P.local_realign != 0);
            // reads are coordinate-sorted: stop once no earlier read can reach
            // pos (R.reach: the farthest any read of the region reaches past its start)
            if (st.batch.pos[r] + 1 + R.reach < d.pos) break;
            if (a > d.pos || b < d.pos) continue;
            if (!read_passes(st.batch, P, R, r)) continue;
            if (++probes > max_probe_reads) { set_err(st.err, ERR_PROBE_LIMIT); break; }
            ps.stopped = false;
            ps.stop_read = -1;
            w.walk(st.batch, r);
        }
        if (ps.found) apply_subtract(st.cells, R, st.err, d.pos, d.base, d.dir, d.tp, d.q, d.mapq, d.nm, P.goodq);
    }
}

// One thread per queued entry (OrderFix): replays the reads that can observe
// the entry's position, in file order, and sets its pstd/qstd flags to the
// reference's order-dependent result.  Entries are rare (zero qualities or
// read positions), so the replay walks whole reads with the general walker.
__global__ void k_fix_order(DevState st, DevParams P) {
    unsigned int n = *st.n_ofix;
    if (n > st.ofix_cap) n = st.ofix_cap;
    uint32_t ph_hi[SerialSink::kPh / 32], ph_lo[SerialSink::kPh / 32];
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const OrderFix f = st.ofix[k];
        const Region &R = st.regions[f.region];
        OrderSink os;
        os.R = &R;
        os.region_idx = f.region;
        os.pos = f.pos;
        os.base = f.base;
        os.kind = 0;
        os.fp = 0;
        if (f.base < 0) {
            const Slot &sl = st.hash.slots[f.index];
            os.kind = sl.kind;
            os.fp = sl.fp;
        }
        os.track = false;
        os.ph_hi = ph_hi;
        os.ph_lo = ph_lo;
        os.pp = 0;
        os.pq = 0.0;
        os.pstd = os.qstd = false;
        const bool in_order = R.serial && R.edge_hit;
        if (in_order)
            for (int i = 0; i < SerialSink::kPh / 32; i++) { ph_hi[i] = 0; ph_lo[i] = 0; }
        // first read that can reach the position (R.reach: the farthest any
        // read of the region reaches past its start); in an in-order region,
        // the first edge read if that comes earlier (its inserts past the
        // window are seen by later edge reads)
        int64_t lo = R.r0, hi = R.r1;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (st.batch.pos[mid] + 1 + R.reach < f.pos) lo = mid + 1; else hi = mid;
        }
        if (in_order) {
            int64_t a = R.r0, b = R.r1;
            while (a < b) {
                int64_t mid = (a + b) / 2;
                if (st.batch.pos[mid] + 1 + R.reach + kEdgeMargin <= R.we) a = mid + 1; else b = mid;
            }
            if (a < lo) lo = a;
        }
        Walker<OrderSink> w(P, os, R, st.ref, st.ref_len);
        for (int64_t r = lo; r < R.r1; r++) {
            // a read starts at most its length before its position
            if (st.batch.pos[r] - st.batch.max_lq > f.pos) break;
            if (!read_passes(st.batch, P, R, r)) continue;
            int a, b;
            read_span(st.batch, r, a, b, P.local_realign != 0);
            const bool edge = in_order && is_edge(R, b);
            if (!edge && (a > f.pos || b < f.pos)) continue;
            os.track = edge;
            w.walk(st.batch, r);
        }
        if (f.base >= 0) {
            uint32_t v = st.cells.first[f.index] & ~(FC_PDIFF | FC_QDIFF);
            st.cells.first[f.index] = v | (os.pstd ? FC_PDIFF : 0u) | (os.qstd ? FC_QDIFF : 0u);
        } else {
            Slot &sl = st.hash.slots[f.index];
            sl.flags = (sl.flags & ~(SF_PDIFF | SF_QDIFF)) | (os.pstd ? SF_PDIFF : 0u) | (os.qstd ? SF_QDIFF : 0u);
        }
    }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
void launch_init_slots(Slot *slots, unsigned long long n, cudaStream_t s) {
    k_init_slots<<<592, 256, 0, s>>>(slots, n);
}

void launch_clear_used(Slot *slots, const uint32_t *used, const unsigned int *n_used, unsigned long long cap,
                       cudaStream_t s) {
    k_clear_used<<<592, 256, 0, s>>>(slots, used, n_used, cap);
}

void launch_region_reset(const DevState &st, cudaStream_t s) {
    if (st.n_regions > 0) k_region_reset<<<(st.n_regions + 255) / 256, 256, 0, s>>>(st);
}

size_t pileup_smem_bytes() { return (size_t)kTileW * 4 * 4 * 4; }

// Instantiations differing in the minimum resident blocks per SM (and so in
// the register budget per thread) and in warp aggregation of the shared
// histogram updates; the autotuner times them and keeps the fastest
// (RV_PILEUP_VARIANT pins one, 0..5: 0-2 direct updates with 2/3/4 blocks
// per SM, 3-5 the same with warp aggregation).
using PileupKernel = void (*)(DevState, DevParams, int);
static PileupKernel pileup_variant(int v) {
    switch (v) {
    case 0: return k_pileup_tiles<kTileW, 2, false>;
    case 1: return k_pileup_tiles<kTileW, 3, false>;
    case 2: return k_pileup_tiles<kTileW, 4, false>;
    case 3: return k_pileup_tiles<kTileW, 2, true>;
    case 4: return k_pileup_tiles<kTileW, 3, true>;
    default: return k_pileup_tiles<kTileW, 4, true>;
    }
}
int pileup_variants() { return 6; }

// Blocks of the tile kernel are not persistent: each pulls at most `quota`
// tiles from the shared counter and exits, so the grid is ceil(tiles /
// quota) blocks and block slots free up continuously.  The launch carries
// stream priority `priority` (the device's lowest): the blocks of a
// higher-priority kernel queued meanwhile (another batch's realigner pass,
// its scoring kernels, each dependent on the one before) take the next free
// slots instead of waiting for the whole pileup.  Tiles are independent
// (every histogram update is an atomic or an order-free merge), so neither
// the quota nor the interleaving changes a result.
int tile_quota(int64_t n_tiles, int resident_blocks) {
    // at most 16 tiles per block (a few milliseconds on a deep batch; a
    // block's exit writes its threads' local-memory state back), and at
    // least 8 waves of resident blocks' worth
    const int64_t per = (int64_t)std::max(1, resident_blocks) * 8;
    return (int)std::max<int64_t>(1, std::min<int64_t>(16, n_tiles / per));
}

cudaError_t launch_pileup(const DevState &st, const DevParams &P, int resident_blocks, cudaStream_t s, int variant,
                          int priority) {
    size_t smem = pileup_smem_bytes();
    PileupKernel k = pileup_variant(variant);
    // (a larger shared-memory carveout was measured slower: the walker's
    // local-memory state lives in L1)
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (st.n_tiles <= 0) return cudaSuccess;
    const int quota = tile_quota(st.n_tiles, resident_blocks);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = priority;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(((int64_t)st.n_tiles + quota - 1) / quota));
    cfg.blockDim = dim3(kPileupThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k, st, P, quota);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

int pileup_blocks_per_sm(int variant) {
    int n = 0;
    cudaFuncSetAttribute(pileup_variant(variant), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pileup_smem_bytes());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pileup_variant(variant), kPileupThreads, pileup_smem_bytes());
    return n;
}

void launch_edge_detect(const DevState &st, const DevParams &P, cudaStream_t s) {
    if (st.n_regions > 0) k_edge_detect<<<st.n_regions * kEdgeBlocks, 128, 0, s>>>(st, P);
}

void launch_serial(const DevState &st, const DevParams &P, cudaStream_t s) {
    if (st.n_regions > 0) k_pileup_serial<<<st.n_regions, 128, 0, s>>>(st, P);
}

void launch_resolve(const DevState &st, const DevParams &P, cudaStream_t s) {
    k_resolve_deferred<<<152, 128, 0, s>>>(st, P, 1 << 16);
}

void launch_fix_order(const DevState &st, const DevParams &P, cudaStream_t s) {
    k_fix_order<<<16, 64, 0, s>>>(st, P);
}


}  // namespace rv
