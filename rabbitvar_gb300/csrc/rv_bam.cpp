// Host BAM/BGZF decoder producing the structure-of-arrays read batches the
// GPU path consumes (the record side of RecordPreprocessor,
// src/recordPreprocessor.cpp:10-32,101-180, which the reference obtains from
// htslib).  Written from the SAM/BAM v1 specification (BGZF section 4.1,
// records 4.2) and RFC 1951 (DEFLATE); BGZF members inflate independently,
// so they are decoded on several host threads.  Batch arrays live in pinned
// host memory so the upload to the GPU is a plain DMA.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "rv_bam_internal.h"
#include "rvgpu_io.h"

namespace {

// ---------------------------------------------------------------------------
// DEFLATE (RFC 1951) decoder: stored, fixed-Huffman and dynamic-Huffman blocks
// ---------------------------------------------------------------------------
struct Bits {
    const uint8_t *p;
    size_t n, pos = 0;
    uint64_t acc = 0;
    int have = 0;
    bool bad = false;
    Bits(const uint8_t *d, size_t len) : p(d), n(len) {}
    void fill() {
        while (have <= 56) {
            uint64_t b = pos < n ? p[pos] : 0;
            if (pos >= n) { if (have == 0) bad = true; }
            pos++;
            acc |= b << have;
            have += 8;
        }
    }
    uint32_t get(int k) {
        if (k == 0) return 0;
        if (have < k) fill();
        uint32_t v = (uint32_t)(acc & ((1ULL << k) - 1));
        acc >>= k;
        have -= k;
        return v;
    }
    void align() { int r = have & 7; acc >>= r; have -= r; }
};

// Canonical Huffman code, decoded through a first-level table of 9 bits and
// a bit-serial slow path for longer codes.
struct Huff {
    uint16_t count[16];
    uint16_t sym[320];
    int16_t fast[512];   // (symbol << 4 | length), -1 when the code is longer than 9 bits
    bool build(const uint8_t *len, int n) {
        memset(count, 0, sizeof count);
        for (int i = 0; i < n; i++) count[len[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; l++) {
            left <<= 1;
            left -= count[l];
            if (left < 0) return false;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = offs[l] + count[l];
        for (int i = 0; i < n; i++)
            if (len[i]) sym[offs[len[i]]++] = (uint16_t)i;
        // fast table: walk codes in canonical order
        for (int i = 0; i < 512; i++) fast[i] = -1;
        int code = 0, idx = 0;
        for (int l = 1; l <= 9; l++) {
            for (int k = 0; k < count[l]; k++) {
                // canonical codes are stored MSB-first; the stream delivers LSB-first
                int rev = 0;
                for (int b = 0; b < l; b++) rev |= ((code >> b) & 1) << (l - 1 - b);
                for (int fill = rev; fill < 512; fill += (1 << l)) fast[fill] = (int16_t)((sym[idx] << 4) | l);
                code++;
                idx++;
            }
            code <<= 1;
        }
        return true;
    }
    int decode(Bits &bs) const {
        if (bs.have < 16) bs.fill();
        int f = fast[bs.acc & 511];
        if (f >= 0) {
            int l = f & 15;
            bs.acc >>= l;
            bs.have -= l;
            return f >> 4;
        }
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; l++) {
            code |= (int)bs.get(1);
            int c = count[l];
            if (code - c < first) return sym[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits &bs, const Huff &lit, const Huff &dist, uint8_t *out, size_t cap, size_t &o) {
    for (;;) {
        int s = lit.decode(bs);
        if (s < 0 || bs.bad) return false;
        if (s < 256) {
            if (o >= cap) return false;
            out[o++] = (uint8_t)s;
        } else if (s == 256) {
            return true;
        } else {
            s -= 257;
            if (s >= 29) return false;
            int len = kLenBase[s] + (int)bs.get(kLenExtra[s]);
            int ds = dist.decode(bs);
            if (ds < 0 || ds >= 30) return false;
            size_t d = kDistBase[ds] + bs.get(kDistExtra[ds]);
            if (d > o || o + len > cap) return false;
            for (int k = 0; k < len; k++, o++) out[o] = out[o - d];
        }
    }
}

bool inflate_raw(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t &produced) {
    Bits bs(in, n);
    size_t o = 0;
    static Huff fixed_lit, fixed_dist;
    static std::atomic<int> fixed_ready{0};
    if (fixed_ready.load() == 0) {
        uint8_t l[288];
        for (int i = 0; i < 144; i++) l[i] = 8;
        for (int i = 144; i < 256; i++) l[i] = 9;
        for (int i = 256; i < 280; i++) l[i] = 7;
        for (int i = 280; i < 288; i++) l[i] = 8;
        Huff a, b;
        a.build(l, 288);
        uint8_t d[30];
        for (int i = 0; i < 30; i++) d[i] = 5;
        b.build(d, 30);
        static std::atomic<int> once{0};
        if (once.exchange(1) == 0) {
            fixed_lit = a;
            fixed_dist = b;
            fixed_ready.store(1);
        }
        while (fixed_ready.load() == 0) std::this_thread::yield();
    }
    int last;
    do {
        last = (int)bs.get(1);
        int type = (int)bs.get(2);
        if (type == 0) {
            bs.align();
            uint32_t len = bs.get(16), nlen = bs.get(16);
            if ((len ^ 0xFFFF) != nlen || o + len > cap) return false;
            for (uint32_t k = 0; k < len; k++) out[o++] = (uint8_t)bs.get(8);
        } else if (type == 1) {
            if (!inflate_codes(bs, fixed_lit, fixed_dist, out, cap, o)) return false;
        } else if (type == 2) {
            int hlit = (int)bs.get(5) + 257, hdist = (int)bs.get(5) + 1, hclen = (int)bs.get(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)bs.get(3);
            Huff clh;
            if (!clh.build(cl, 19)) return false;
            uint8_t lens[320];
            int k = 0;
            while (k < hlit + hdist) {
                int s = clh.decode(bs);
                if (s < 0) return false;
                if (s < 16) lens[k++] = (uint8_t)s;
                else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (s == 16) { if (k == 0) return false; val = lens[k - 1]; rep = 3 + (int)bs.get(2); }
                    else if (s == 17) rep = 3 + (int)bs.get(3);
                    else rep = 11 + (int)bs.get(7);
                    if (k + rep > hlit + hdist) return false;
                    while (rep--) lens[k++] = val;
                }
            }
            Huff lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) return false;
            if (!inflate_codes(bs, lit, dist, out, cap, o)) return false;
        } else {
            return false;
        }
        if (bs.bad) return false;
    } while (!last);
    produced = o;
    return true;
}

uint32_t rd32(const uint8_t *p) { uint32_t v; memcpy(&v, p, 4); return v; }
uint16_t rd16(const uint8_t *p) { uint16_t v; memcpy(&v, p, 2); return v; }

template <class T>
T *pinned(size_t n, std::vector<void *> &owned) {
    void *p = nullptr;
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        p = malloc(bytes);
        if (!p) return nullptr;
        owned.push_back((void *)((uintptr_t)p | 1));  // tag: malloc'd
    } else {
        owned.push_back(p);
    }
    return (T *)p;
}

}  // namespace

bool bgzf_members(const uint8_t *raw, size_t n, std::vector<BgzfMember> &out, uint64_t &total) {
    out.clear();
    size_t p = 0;
    total = 0;
    while (p + 18 <= n) {
        const uint8_t *h = raw + p;
        if (h[0] != 31 || h[1] != 139 || h[2] != 8 || !(h[3] & 4)) return false;
        uint16_t xlen = rd16(h + 10);
        int bsize = -1;
        for (size_t q = 12; q + 4 <= 12u + xlen && p + q + 4 <= n;) {
            uint16_t slen = rd16(h + q + 2);
            if (h[q] == 'B' && h[q + 1] == 'C' && slen == 2 && p + q + 6 <= n) bsize = rd16(h + q + 4);
            q += 4 + slen;
        }
        if (bsize < 0) return false;
        size_t blen = (size_t)bsize + 1;
        if (p + blen > n || blen < 12u + xlen + 8) return false;
        BgzfMember m;
        m.in_off = p + 12 + xlen;
        m.in_len = (uint32_t)(blen - 12 - xlen - 8);
        m.out_len = rd32(h + blen - 4);
        if (m.out_len > 65536) return false;
        m.out_off = total;
        total += m.out_len;
        out.push_back(m);
        p += blen;
    }
    return p == n;
}

int64_t bam_parse_header(const uint8_t *d, uint64_t n, uint64_t total, rv_bam *bam) {
    bam->names.clear();
    bam->lens.clear();
    auto need = [&](uint64_t k) { return k <= n ? 1 : (k <= total ? 0 : -1); };
    int r;
    if ((r = need(8)) <= 0) return r;
    if (memcmp(d, "BAM\1", 4) != 0) return -1;
    uint64_t q = 8 + (uint64_t)rd32(d + 4);
    if ((r = need(q + 4)) <= 0) return r;
    uint32_t n_ref = rd32(d + q);
    q += 4;
    for (uint32_t i = 0; i < n_ref; i++) {
        if ((r = need(q + 4)) <= 0) return r;
        uint32_t ln = rd32(d + q);
        q += 4;
        if ((r = need(q + ln + 4)) <= 0) return r;
        bam->names.emplace_back((const char *)d + q, strnlen((const char *)d + q, ln));
        q += ln;
        bam->lens.push_back((int32_t)rd32(d + q));
        q += 4;
    }
    bam->name_ptrs.clear();
    for (auto &s : bam->names) bam->name_ptrs.push_back(s.c_str());
    return (int64_t)q;
}

extern "C" {

rv_status rv_bam_read(const char *path, int threads, rv_bam **out) {
    if (!path || !out) return RV_ERR_ARG;
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return RV_ERR_ARG;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<uint8_t> raw((size_t)std::max(sz, 0L));
    size_t got = sz > 0 ? fread(raw.data(), 1, raw.size(), f) : 0;
    fclose(f);
    if (got != raw.size()) return RV_ERR_FORMAT;
    return rv_bam_read_mem(raw.data(), raw.size(), threads, out);
}

rv_status rv_bam_read_mem(const uint8_t *bgzf, size_t n, int threads, rv_bam **out) {
    if (!bgzf || !out) return RV_ERR_ARG;
    *out = nullptr;
    struct {
        const uint8_t *p;
        size_t n;
        const uint8_t *data() const { return p; }
        size_t size() const { return n; }
    } raw{bgzf, n};
    std::vector<BgzfMember> blks;
    uint64_t total = 0;
    if (!bgzf_members(raw.data(), raw.size(), blks, total)) return RV_ERR_FORMAT;
    rv_bam *bam = new rv_bam();
    bam->data.resize(total + 8);
    std::atomic<size_t> next{0};
    std::atomic<int> bad{0};
    int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = std::min<int>(nt, (int)std::max<size_t>(1, blks.size()));
    auto work = [&]() {
        for (;;) {
            size_t i = next.fetch_add(1);
            if (i >= blks.size()) break;
            const BgzfMember &b = blks[i];
            size_t produced = 0;
            if (b.out_len && (!inflate_raw(raw.data() + b.in_off, b.in_len, bam->data.data() + b.out_off, b.out_len,
                                           produced) ||
                              produced != b.out_len))
                bad.store(1);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    if (bad.load()) { delete bam; return RV_ERR_FORMAT; }
    const std::vector<uint8_t> &d = bam->data;
    const int64_t hdr = bam_parse_header(d.data(), total, total, bam);
    if (hdr <= 0) { delete bam; return RV_ERR_FORMAT; }
    size_t q = (size_t)hdr;
    while (q + 4 <= total) {
        uint32_t bs = rd32(&d[q]);
        if (bs < 32 || q + 4 + bs > total) { delete bam; return RV_ERR_FORMAT; }
        bam->rec_off.push_back(q);
        bam->rec_tid.push_back((int32_t)rd32(&d[q + 4]));
        q += 4 + bs;
    }
    *out = bam;
    return RV_OK;
}

rv_status rv_bam_contigs(const rv_bam *bam, int *n, const char *const **names, const int32_t **lens) {
    if (!bam || !n) return RV_ERR_ARG;
    *n = (int)bam->names.size();
    if (names) *names = bam->name_ptrs.data();
    if (lens) *lens = bam->lens.data();
    return RV_OK;
}

rv_status rv_bam_batch(rv_bam *bam, int tid, rv_read_batch *out) {
    if (!bam || !out) return RV_ERR_ARG;
    if (bam->gpu) return bam_gpu_batch(bam, tid, out, false);
    const std::vector<uint8_t> &d = bam->data;
    std::vector<size_t> sel;
    int64_t ncig = 0, nb = 0;
    for (size_t i = 0; i < bam->rec_off.size(); i++) {
        if (bam->rec_tid[i] != tid) continue;
        const uint8_t *r = &d[bam->rec_off[i] + 4];
        ncig += rd16(r + 12);
        int32_t lq = (int32_t)rd32(r + 16);
        nb += ((int64_t)lq + 31) / 32 * 32;
        sel.push_back(i);
    }
    int64_t n = (int64_t)sel.size();
    auto &own = bam->owned;
    int32_t *pos = pinned<int32_t>(n, own), *mpos = pinned<int32_t>(n, own), *nm = pinned<int32_t>(n, own),
            *lq = pinned<int32_t>(n, own);
    uint16_t *flag = pinned<uint16_t>(n, own), *nc = pinned<uint16_t>(n, own);
    uint8_t *mapq = pinned<uint8_t>(n, own);
    uint32_t *coff = pinned<uint32_t>(n, own), *cig = pinned<uint32_t>(ncig, own);
    uint64_t *boff = pinned<uint64_t>(n, own);
    uint8_t *seq = pinned<uint8_t>(nb / 2 + 16, own), *qual = pinned<uint8_t>(nb + 32, own);
    if (!pos || !mpos || !nm || !lq || !flag || !nc || !mapq || !coff || !cig || !boff || !seq || !qual)
        return RV_ERR_CAPACITY;
    int64_t ci = 0, bi = 0;
    for (int64_t k = 0; k < n; k++) {
        const uint8_t *r = &d[bam->rec_off[sel[k]] + 4];
        uint32_t bs = rd32(&d[bam->rec_off[sel[k]]]);
        pos[k] = (int32_t)rd32(r + 4);
        uint8_t l_name = r[8];
        mapq[k] = r[9];
        nc[k] = rd16(r + 12);
        flag[k] = rd16(r + 14);
        lq[k] = (int32_t)rd32(r + 16);
        mpos[k] = (int32_t)rd32(r + 24);
        const uint8_t *v = r + 32 + l_name;
        coff[k] = (uint32_t)ci;
        memcpy(cig + ci, v, (size_t)nc[k] * 4);
        ci += nc[k];
        v += (size_t)nc[k] * 4;
        boff[k] = (uint64_t)bi;
        int L = lq[k];
        memcpy(seq + bi / 2, v, (size_t)(L + 1) / 2);
        v += (L + 1) / 2;
        memcpy(qual + bi, v, (size_t)L);
        v += L;
        bi += ((int64_t)L + 31) / 32 * 32;
        // NM tag among the optional fields
        nm[k] = INT32_MIN;
        const uint8_t *end = r + bs;
        while (v + 3 <= end) {
            uint8_t t = v[2];
            const uint8_t *val = v + 3;
            int sz = (t == 'A' || t == 'c' || t == 'C') ? 1 : (t == 's' || t == 'S') ? 2 : (t == 'i' || t == 'I' || t == 'f') ? 4 : -1;
            if (v[0] == 'N' && v[1] == 'M' && sz > 0) {
                int64_t x = 0;
                switch (t) {
                case 'c': x = (int8_t)val[0]; break;
                case 'C': x = val[0]; break;
                case 's': { int16_t y; memcpy(&y, val, 2); x = y; break; }
                case 'S': x = rd16(val); break;
                case 'i': { int32_t y; memcpy(&y, val, 4); x = y; break; }
                case 'I': x = rd32(val); break;
                default: break;
                }
                nm[k] = (int32_t)x;
                break;
            }
            if (sz > 0) v = val + sz;
            else if (t == 'Z' || t == 'H') { while (val < end && *val) val++; v = val + 1; }
            else if (t == 'B') {
                uint8_t sub = val[0];
                uint32_t cnt = rd32(val + 1);
                int es = (sub == 'c' || sub == 'C') ? 1 : (sub == 's' || sub == 'S') ? 2 : 4;
                v = val + 5 + (size_t)cnt * es;
            } else break;
        }
    }
    out->n_reads = n;
    out->pos = pos;
    out->flag = flag;
    out->mapq = mapq;
    out->mpos = mpos;
    out->nm = nm;
    out->n_cigar = nc;
    out->cig_off = coff;
    out->cigar = cig;
    out->n_cigar_words = ncig;
    out->l_qseq = lq;
    out->base_off = boff;
    out->seq = seq;
    out->qual = qual;
    out->n_bases = bi;
    return RV_OK;
}

rv_status rv_bam_batch_host(rv_bam *bam, int tid, rv_read_batch *out) {
    if (!bam || !out) return RV_ERR_ARG;
    if (bam->gpu) return bam_gpu_batch(bam, tid, out, true);
    return rv_bam_batch(bam, tid, out);
}

void rv_bam_free(rv_bam *bam) {
    if (!bam) return;
    if (bam->gpu) bam_gpu_free(bam->gpu);
    for (void *p : bam->owned) {
        if ((uintptr_t)p & 1) free((void *)((uintptr_t)p & ~(uintptr_t)1));
        else cudaFreeHost(p);
    }
    delete bam;
}

rv_status rv_fasta_read(const char *path, const char *name, char **seq, int64_t *len) {
    if (!path || !seq || !len) return RV_ERR_ARG;
    *seq = nullptr;
    *len = 0;
    FILE *f = fopen(path, "rb");
    if (!f) return RV_ERR_ARG;
    std::string cur, s;
    bool want = false, found = false;
    char line[1 << 16];
    while (fgets(line, sizeof line, f)) {
        size_t n = strlen(line);
        while (n && (line[n - 1] == '\n' || line[n - 1] == '\r')) line[--n] = 0;
        if (line[0] == '>') {
            if (want) break;
            cur.assign(line + 1);
            size_t sp = cur.find_first_of(" \t");
            if (sp != std::string::npos) cur.resize(sp);
            want = !name || cur == name;
            found |= want;
            continue;
        }
        if (want) s.append(line, n);
    }
    fclose(f);
    if (!found) return RV_ERR_ARG;
    *seq = (char *)malloc(s.size() + 1);
    memcpy(*seq, s.data(), s.size());
    (*seq)[s.size()] = 0;
    *len = (int64_t)s.size();
    return RV_OK;
}

void rv_free(void *p) { free(p); }

void *rv_alloc_pinned(size_t bytes) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
}

void rv_free_pinned(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
