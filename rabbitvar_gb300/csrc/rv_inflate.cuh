// rv_inflate.cuh -- DEFLATE (RFC 1951) decoding of one BGZF member by one
// warp, and the BAM record checks the device record finder uses.
//
// BGZF (SAM/BAM specification section 4.1) cuts a BAM stream into gzip
// members of at most 64 KiB of output each, every member a complete raw
// DEFLATE stream: members decode independently, so one device warp inflates
// one member.  The warp's lanes run the bit-level decoder in lockstep (the
// same loads and table lookups: no divergence) and split the parallel parts:
// filling the first-level Huffman tables, and match copies (lane k writes
// bytes k, k+32, ... of a match, each read from the already written window,
// out[o+k] = out[o-d + k mod d], so overlapping matches need no ordering
// within the copy).  The warp's tables live in shared memory (`Tables`,
// about 2.5 KB); input is read through aligned 32-bit loads of the read-only
// compressed buffer; output goes straight to the member's slot of the
// decompressed stream.  Every load is bounded by the buffer and by the
// member's compressed length, every store by the member's declared output
// length; malformed input ends the member with an error code.
//
// The functions are __host__ __device__ (one lane on the host) so the same
// code can be checked on the CPU; the product path runs them only in
// k_inflate (rv_bgzf.cu).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define RVZ_HD __host__ __device__ __forceinline__
#else
#define RVZ_HD inline
#endif

namespace rvz {

enum : int {
    kLitFast = 9,   // first-level table bits, literal/length code
    kDistFast = 8,  // first-level table bits, distance code (and the code-length code)
};

enum : int {
    ERR_NONE = 0,
    ERR_BLOCK_TYPE = 1,   // reserved block type 3
    ERR_STORED_LEN = 2,   // LEN / NLEN mismatch
    ERR_CODE = 3,         // over-subscribed Huffman code, or a code that is not in the table
    ERR_LENGTHS = 4,      // code-length repeat past the end, or a repeat of nothing
    ERR_SYMBOL = 5,       // length symbol 286/287 or distance symbol 30/31
    ERR_DISTANCE = 6,     // distance before the start of the member's output
    ERR_OUTPUT = 7,       // more output than the member's ISIZE
    ERR_INPUT = 8,        // read past the member's compressed bytes
    ERR_SHORT = 9,        // less output than ISIZE
};

// One member's decode tables (shared memory of the warp on the device).
struct Tables {
    uint32_t lit_fast[1 << kLitFast];   // decoded entries (entry_of), 0: longer code or unused
    uint32_t dist_fast[1 << kDistFast];
    uint16_t lit_count[16], dist_count[16];
    uint16_t lit_sym[288], dist_sym[32];
    uint8_t lens[320];
    uint32_t pad;  // odd word count: the warps' tables start in different banks
};

RVZ_HD uint32_t rev_bits(uint32_t code, int len) {
#ifdef __CUDA_ARCH__
    return __brev(code) >> (32 - len);
#else
    uint32_t r = 0;
    for (int b = 0; b < len; b++) r |= ((code >> b) & 1u) << (len - 1 - b);
    return r;
#endif
}

// LSB-first bit reader over [p, p + n) of a buffer that ends at `buf_end`.
// Loads are aligned 32-bit words, never outside [buf_begin, buf_end) rounded
// to words (the caller pads the buffer to a whole number of words).
struct BitIn {
    const uint32_t *w;       // next word to load
    const uint32_t *wlim;    // one past the last word of the buffer
    uint64_t acc;
    int have;
    int64_t left_bits;       // bits of the member not yet loaded into acc (may go negative: over-read)

    RVZ_HD void init(const uint8_t *p, uint32_t n, const uint8_t *buf_end) {
        const uintptr_t a = (uintptr_t)p;
        w = (const uint32_t *)(a & ~(uintptr_t)3);
        wlim = (const uint32_t *)(((uintptr_t)buf_end + 3) & ~(uintptr_t)3);
        const int skip = (int)(a & 3) * 8;
        acc = 0;
        have = 0;
        left_bits = (int64_t)n * 8 + skip;
        load();
        acc >>= skip;
        have -= skip;
    }
    RVZ_HD void load() {
        uint32_t x = 0;
        if (w < wlim) {
#ifdef __CUDA_ARCH__
            x = __ldg(w);
#else
            x = *w;
#endif
        }
        w++;
        acc |= (uint64_t)x << have;
        have += 32;
        left_bits -= 32;
    }
    // at least 32 valid bits in acc afterwards
    RVZ_HD void refill() {
        if (have < 32) load();
    }
    RVZ_HD uint32_t peek(int k) const { return (uint32_t)(acc & ((1ull << k) - 1)); }
    RVZ_HD void drop(int k) {
        acc >>= k;
        have -= k;
    }
    RVZ_HD uint32_t get(int k) {  // k <= 32
        refill();
        const uint32_t v = k ? peek(k) : 0u;
        drop(k);
        return v;
    }
    // bits consumed past the member's end (> 0: the stream ran over)
    RVZ_HD int64_t overrun() const { return -(left_bits + have); }
};

// The lanes cooperating on one member: lane index within the group, group
// size (a warp or part of one on the device, 1 on the host), the group's
// lane mask, and the barrier that orders the group's shared- and
// global-memory writes.
struct Lanes {
    int lane, n;
    unsigned mask;
    RVZ_HD void sync() const {
#ifdef __CUDA_ARCH__
        __syncwarp(mask);
#elif defined(RVZ_HOST_SYNC)
        RVZ_HOST_SYNC(n);  // a host build may emulate a warp with threads and a barrier
#endif
    }
};

RVZ_HD int len_base(int s);
RVZ_HD int len_extra(int s);
RVZ_HD int dist_base(int s);
RVZ_HD int dist_extra(int s);

// A decoded symbol as one word, so the decode loop needs no per-symbol
// arithmetic: bits 0-3 code length (0: no code), bits 4-5 kind, bits 8+
// the payload.  Literal/length alphabet: a literal (byte at 8-15), the end
// of the block, or a length (base at 8-16, extra bits at 20-23).  Distance
// alphabet: base at 8-22, extra bits at 24-27.  Code-length alphabet: the
// symbol at 8-15.
enum : int { MAP_LIT = 0, MAP_DIST = 1, MAP_RAW = 2 };
enum : uint32_t { K_LIT = 0, K_EOB = 1, K_LEN = 2, K_BAD = 3 };

RVZ_HD uint32_t entry_of(int sym, int l, int map) {
    const uint32_t L = (uint32_t)l;
    if (map == MAP_LIT) {
        if (sym < 256) return L | (K_LIT << 4) | ((uint32_t)sym << 8);
        if (sym == 256) return L | (K_EOB << 4);
        if (sym < 286)
            return L | (K_LEN << 4) | ((uint32_t)len_base(sym - 257) << 8) | ((uint32_t)len_extra(sym - 257) << 20);
        return L | (K_BAD << 4);
    }
    if (map == MAP_DIST) {
        if (sym < 30) return L | ((uint32_t)dist_base(sym) << 8) | ((uint32_t)dist_extra(sym) << 24);
        return L | (K_BAD << 4);
    }
    return L | ((uint32_t)sym << 8);
}

// Canonical Huffman code (RFC 1951 3.2.2) from code lengths: a first-level
// table of `fbits` bits plus count/symbol arrays for the bit-serial slow path.
// Every lane computes the counts and offsets; the symbol list and the table
// entries are written by the lanes in parallel.
RVZ_HD bool build(const uint8_t *len, int n, uint32_t *fast, int fbits, uint16_t *count, uint16_t *sym, int map,
                  const Lanes &w) {
    uint16_t cnt[16];
    for (int l = 0; l < 16; l++) cnt[l] = 0;
    for (int i = 0; i < n; i++) cnt[len[i]]++;
    cnt[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; l++) {
        left <<= 1;
        left -= cnt[l];
        if (left < 0) return false;
    }
    // offs[l]: index of the first length-l symbol in `sym`; first[l]: its code
    uint16_t offs[16];
    uint32_t first[16];
    offs[0] = offs[1] = 0;
    first[0] = first[1] = 0;
    for (int l = 1; l < 15; l++) {
        offs[l + 1] = (uint16_t)(offs[l] + cnt[l]);
        first[l + 1] = (first[l] + cnt[l]) << 1;
    }
    w.sync();  // earlier readers of the tables are done
    for (int l = w.lane; l < 16; l += w.n) count[l] = cnt[l];
    // symbols in canonical order: symbol i goes after the earlier symbols of its length
    for (int i = w.lane; i < n; i += w.n) {
        const int l = len[i];
        if (!l) continue;
        int r = 0;
        for (int j = 0; j < i; j++) r += len[j] == l;
        sym[offs[l] + r] = (uint16_t)i;
    }
    const int size = 1 << fbits;
    for (int i = w.lane; i < size; i += w.n) fast[i] = 0;
    w.sync();
    // codes no longer than fbits fill every table entry they prefix
    const int nfast = offs[fbits < 15 ? fbits + 1 : 15] + (fbits < 15 ? 0 : cnt[15]);
    for (int idx = w.lane; idx < nfast; idx += w.n) {
        int l = 1;
        while (l < 15 && idx >= offs[l + 1]) l++;
        const uint32_t code = first[l] + (uint32_t)(idx - offs[l]);
        const uint32_t e = entry_of(sym[idx], l, map);
        for (uint32_t f = rev_bits(code, l); f < (uint32_t)size; f += 1u << l) fast[f] = e;
    }
    w.sync();
    return true;
}

// One symbol's entry (entry_of); 0 for a code that is not in the table.
RVZ_HD uint32_t decode(BitIn &b, const uint32_t *fast, int fbits, const uint16_t *count, const uint16_t *sym, int map) {
    b.refill();
    const uint32_t e = fast[b.peek(fbits)];
    if (e & 15) {
        b.drop((int)(e & 15));
        return e;
    }
    int code = 0, first = 0, index = 0;
    uint64_t a = b.acc;
    for (int l = 1; l < 16; l++) {
        code |= (int)(a & 1);
        a >>= 1;
        const int c = count[l];
        if (code - c < first) {
            b.drop(l);
            return entry_of(sym[index + (code - first)], l, map);
        }
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
    }
    return 0;
}

RVZ_HD int len_base(int s) {  // s in [0, 28]
    return s < 8 ? 3 + s : (s == 28 ? 258 : ((4 + ((s - 8) & 3)) << (((s - 8) >> 2) + 1)) + 3);
}
RVZ_HD int len_extra(int s) { return (s < 8 || s == 28) ? 0 : ((s - 8) >> 2) + 1; }
RVZ_HD int dist_base(int s) {  // s in [0, 29]
    return s < 4 ? 1 + s : ((2 + (s & 1)) << ((s >> 1) - 1)) + 1;
}
RVZ_HD int dist_extra(int s) { return s < 4 ? 0 : (s >> 1) - 1; }

// A member's output slot and the bytes produced so far.
struct Out {
    uint8_t *g;
    uint32_t cap;  // ISIZE
    uint32_t o;

    RVZ_HD void put(uint8_t v, const Lanes &w) {
        if (w.lane == 0) g[o] = v;
        o++;
    }
    // out[o + k] = out[o - d + k mod d]: reads only bytes written before this
    // match, so the lanes copy in any order
    RVZ_HD void copy(uint32_t d, uint32_t len, const Lanes &w) {
        w.sync();
        const uint8_t *src = g + (o - d);
        uint8_t *dst = g + o;
        if (d >= len)
            for (uint32_t k = (uint32_t)w.lane; k < len; k += (uint32_t)w.n) dst[k] = src[k];
        else
            for (uint32_t k = (uint32_t)w.lane; k < len; k += (uint32_t)w.n) dst[k] = src[k % d];
        o += len;
    }
};

// The symbols of one block up to its end-of-block code.  Every symbol other
// than end-of-block adds at least one byte, so a block ends within ISIZE + 1
// symbols; reads past the member's end are checked once per block.
RVZ_HD int codes(BitIn &b, Tables &t, Out &out, const Lanes &w) {
    for (;;) {
        const uint32_t e = decode(b, t.lit_fast, kLitFast, t.lit_count, t.lit_sym, MAP_LIT);
        if (!e) return ERR_CODE;
        const uint32_t kind = (e >> 4) & 3;
        if (kind == K_LIT) {
            if (out.o >= out.cap) return ERR_OUTPUT;
            out.put((uint8_t)(e >> 8), w);
            continue;
        }
        if (kind == K_EOB) return ERR_NONE;
        if (kind == K_BAD) return ERR_SYMBOL;
        const uint32_t len = ((e >> 8) & 0x1FF) + b.get((int)((e >> 20) & 15));
        const uint32_t f = decode(b, t.dist_fast, kDistFast, t.dist_count, t.dist_sym, MAP_DIST);
        if (!f) return ERR_CODE;
        if (f & 0x30) return ERR_SYMBOL;
        const uint32_t d = ((f >> 8) & 0x7FFF) + b.get((int)((f >> 24) & 15));
        if (d > out.o) return ERR_DISTANCE;
        if (len > out.cap - out.o) return ERR_OUTPUT;
        out.copy(d, len, w);
    }
}

// Inflates the raw DEFLATE stream [in, in + n) into out[0, cap); returns an
// ERR_* code (ERR_NONE when exactly `cap` bytes came out).
RVZ_HD int inflate(const uint8_t *in, uint32_t n, const uint8_t *buf_end, uint8_t *dst, uint32_t cap, Tables &t,
                   const Lanes &w) {
    BitIn b;
    b.init(in, n, buf_end);
    Out out{dst, cap, 0u};
    int last = 0;
    do {
        last = (int)b.get(1);
        const int type = (int)b.get(2);
        if (type == 0) {
            b.drop(b.have & 7);
            const uint32_t len = b.get(16), nlen = b.get(16);
            if ((len ^ 0xFFFFu) != nlen) return ERR_STORED_LEN;
            if (len > cap - out.o) return ERR_OUTPUT;
            for (uint32_t k = 0; k < len; k++) out.put((uint8_t)b.get(8), w);
        } else if (type == 1) {
            w.sync();
            for (int i = w.lane; i < 288; i += w.n) t.lens[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
            w.sync();
            build(t.lens, 288, t.lit_fast, kLitFast, t.lit_count, t.lit_sym, MAP_LIT, w);
            for (int i = w.lane; i < 30; i += w.n) t.lens[i] = 5;
            w.sync();
            build(t.lens, 30, t.dist_fast, kDistFast, t.dist_count, t.dist_sym, MAP_DIST, w);
            const int e = codes(b, t, out, w);
            if (e) return e;
        } else if (type == 2) {
            const int hlit = (int)b.get(5) + 257, hdist = (int)b.get(5) + 1, hclen = (int)b.get(4) + 4;
            if (hlit > 286 || hdist > 30) return ERR_SYMBOL;
            const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19];
            for (int i = 0; i < 19; i++) cl[i] = 0;
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)b.get(3);
            w.sync();
            for (int i = w.lane; i < 19; i += w.n) t.lens[i] = cl[i];
            w.sync();
            // the code-length code borrows the distance tables
            if (!build(t.lens, 19, t.dist_fast, kDistFast, t.dist_count, t.dist_sym, MAP_RAW, w)) return ERR_CODE;
            int k = 0;
            uint8_t prev = 0;
            while (k < hlit + hdist) {
                const uint32_t ce = decode(b, t.dist_fast, kDistFast, t.dist_count, t.dist_sym, MAP_RAW);
                if (!ce) return ERR_CODE;
                const int s = (int)(ce >> 8);
                if (b.overrun() > 0) return ERR_INPUT;
                if (s < 16) {
                    if (w.lane == 0) t.lens[k] = (uint8_t)s;
                    prev = (uint8_t)s;
                    k++;
                    continue;
                }
                int rep;
                uint8_t val = 0;
                if (s == 16) {
                    if (k == 0) return ERR_LENGTHS;
                    val = prev;
                    rep = 3 + (int)b.get(2);
                } else if (s == 17) {
                    rep = 3 + (int)b.get(3);
                } else {
                    rep = 11 + (int)b.get(7);
                }
                if (k + rep > hlit + hdist) return ERR_LENGTHS;
                for (int j = w.lane; j < rep; j += w.n) t.lens[k + j] = val;
                prev = val;
                k += rep;
            }
            w.sync();
            if (t.lens[256] == 0) return ERR_CODE;  // no end-of-block code
            if (!build(t.lens, hlit, t.lit_fast, kLitFast, t.lit_count, t.lit_sym, MAP_LIT, w)) return ERR_CODE;
            if (!build(t.lens + hlit, hdist, t.dist_fast, kDistFast, t.dist_count, t.dist_sym, MAP_DIST, w)) return ERR_CODE;
            const int e = codes(b, t, out, w);
            if (e) return e;
        } else {
            return ERR_BLOCK_TYPE;
        }
        if (b.overrun() > 0) return ERR_INPUT;
    } while (!last);
    return out.o == cap ? ERR_NONE : ERR_SHORT;
}

// ---------------------------------------------------------------------------
// BAM records (SAM/BAM specification section 4.2)
// ---------------------------------------------------------------------------
RVZ_HD uint32_t rd16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
RVZ_HD uint32_t rd32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// Whether a plausible alignment record starts at offset o of the stream
// d[0, total): block_size covers the fixed fields, the name, the CIGAR and
// the sequence; reference ids lie in [-1, n_ref); the read name is printable
// and NUL-terminated; every CIGAR operation is one of MIDNSHP=X.  Used only to
// pick a candidate start; the chain of starts is verified separately.
RVZ_HD bool record_plausible(const uint8_t *d, uint64_t total, uint64_t o, int32_t n_ref, uint32_t *size) {
    if (o + 36 > total) return false;
    const uint32_t bs = rd32(d + o);
    if (bs < 32 || bs > total - o - 4) return false;
    const uint8_t *r = d + o + 4;
    const int32_t tid = (int32_t)rd32(r), pos = (int32_t)rd32(r + 4);
    const int32_t ntid = (int32_t)rd32(r + 20), npos = (int32_t)rd32(r + 24);
    if (tid < -1 || tid >= n_ref || ntid < -1 || ntid >= n_ref || pos < -1 || npos < -1) return false;
    const uint32_t lrn = r[8], nc = rd16(r + 12);
    const int32_t lq = (int32_t)rd32(r + 16);
    if (lrn < 1 || lq < 0) return false;
    const uint64_t need = 32ull + lrn + 4ull * nc + ((uint64_t)lq + 1) / 2 + (uint64_t)lq;
    if (need > bs) return false;
    if (r[32 + lrn - 1] != 0) return false;
    for (uint32_t k = 0; k + 1 < lrn; k++)
        if (r[32 + k] < 33 || r[32 + k] > 126) return false;
    for (uint32_t k = 0; k < nc; k++)
        if ((r[32 + lrn + 4 * k] & 15) > 8) return false;
    *size = bs;
    return true;
}

}  // namespace rvz
