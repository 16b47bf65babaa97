// Oracle test infrastructure: project-written implementation of the subset
// of the htslib API that RabbitVar calls (see htslib/*.h in this folder).
// htslib itself is not installed here.  Everything below is written from the
// public format specifications:
//   * BGZF (SAM/BAM spec section 4.1): concatenated gzip members, each with a
//     "BC" extra subfield giving the member size; payload is raw DEFLATE.
//   * BAM records (section 4.2), FASTA index .fai (five tab-separated columns).
// Files are inflated once per process and shared read-only between threads;
// region queries return the records overlapping [beg, end) in file order,
// which is what htslib's sam_itr_querys/sam_itr_next yield.
#include "htslib/hts.h"
#include "htslib/sam.h"
#include "htslib/faidx.h"
#include "htslib/kfunc.h"
#include "../fisher_oracle.h"

#include <zlib.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

const char seq_nt16_str[] = "=ACMGRSVTWYHKDBN";

namespace {

struct RecEntry {
    int32_t tid;
    int64_t pos;
    int64_t endpos;
    size_t offset;  // offset of the record's block_size field in the BAM stream
};

struct BamImage {
    std::vector<uint8_t> bytes;  // whole decompressed BAM stream
    std::vector<std::string> names;
    std::vector<uint32_t> lens;
    std::vector<RecEntry> recs;
    std::vector<int64_t> max_span;  // per tid
};

std::mutex g_cache_mu;
std::map<std::string, std::shared_ptr<BamImage>> g_cache;

uint32_t rd32(const uint8_t *p) { uint32_t v; memcpy(&v, p, 4); return v; }
int32_t rdi32(const uint8_t *p) { int32_t v; memcpy(&v, p, 4); return v; }
uint16_t rd16(const uint8_t *p) { uint16_t v; memcpy(&v, p, 2); return v; }

bool bgzf_inflate_file(const char *fn, std::vector<uint8_t> &out) {
    FILE *f = fopen(fn, "rb");
    if (!f) return false;
    std::vector<uint8_t> raw;
    {
        fseek(f, 0, SEEK_END);
        long n = ftell(f);
        fseek(f, 0, SEEK_SET);
        raw.resize((size_t)n);
        if (n > 0 && fread(raw.data(), 1, (size_t)n, f) != (size_t)n) { fclose(f); return false; }
        fclose(f);
    }
    size_t p = 0;
    while (p + 18 <= raw.size()) {
        const uint8_t *h = raw.data() + p;
        if (h[0] != 31 || h[1] != 139 || h[2] != 8 || !(h[3] & 4)) return false;
        uint16_t xlen = rd16(h + 10);
        int bsize = -1;
        for (size_t q = 12; q + 4 <= 12u + xlen;) {
            uint16_t slen = rd16(h + q + 2);
            if (h[q] == 'B' && h[q + 1] == 'C' && slen == 2) bsize = rd16(h + q + 4);
            q += 4 + slen;
        }
        if (bsize < 0) return false;
        size_t blen = (size_t)bsize + 1;
        if (p + blen > raw.size()) return false;
        uint32_t isize = rd32(h + blen - 4);
        size_t cdata = 12 + xlen, clen = blen - cdata - 8;
        size_t old = out.size();
        out.resize(old + isize);
        if (isize > 0) {
            z_stream zs;
            memset(&zs, 0, sizeof zs);
            if (inflateInit2(&zs, -15) != Z_OK) return false;
            zs.next_in = const_cast<uint8_t *>(h + cdata);
            zs.avail_in = (uInt)clen;
            zs.next_out = out.data() + old;
            zs.avail_out = isize;
            int rc = inflate(&zs, Z_FINISH);
            inflateEnd(&zs);
            if (rc != Z_STREAM_END) return false;
        }
        p += blen;
    }
    return true;
}

int64_t ref_len_of(const uint8_t *cig, uint32_t n) {
    int64_t len = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t c = rd32(cig + 4 * i);
        if (bam_cigar_type(bam_cigar_op(c)) & 2) len += bam_cigar_oplen(c);
    }
    return len;
}

std::shared_ptr<BamImage> load_bam(const char *fn) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_cache.find(fn);
    if (it != g_cache.end()) return it->second;
    auto img = std::make_shared<BamImage>();
    if (!bgzf_inflate_file(fn, img->bytes)) return nullptr;
    const std::vector<uint8_t> &b = img->bytes;
    if (b.size() < 12 || memcmp(b.data(), "BAM\1", 4) != 0) return nullptr;
    size_t p = 4;
    uint32_t l_text = rd32(&b[p]); p += 4 + l_text;
    uint32_t n_ref = rd32(&b[p]); p += 4;
    for (uint32_t i = 0; i < n_ref; ++i) {
        uint32_t l_name = rd32(&b[p]); p += 4;
        img->names.emplace_back((const char *)&b[p]);
        p += l_name;
        img->lens.push_back(rd32(&b[p])); p += 4;
    }
    img->max_span.assign(n_ref, 1);
    while (p + 4 <= b.size()) {
        uint32_t bs = rd32(&b[p]);
        const uint8_t *r = &b[p + 4];
        RecEntry e;
        e.tid = rdi32(r);
        e.pos = rdi32(r + 4);
        uint8_t l_read_name = r[8];
        uint16_t n_cigar = rd16(r + 12);
        uint16_t flag = rd16(r + 14);
        int64_t rl = ref_len_of(r + 32 + l_read_name, n_cigar);
        e.endpos = ((flag & BAM_FUNMAP) || rl == 0) ? e.pos + 1 : e.pos + rl;
        e.offset = p;
        if (e.tid >= 0 && e.tid < (int32_t)n_ref)
            img->max_span[e.tid] = std::max(img->max_span[e.tid], e.endpos - e.pos);
        img->recs.push_back(e);
        p += 4 + bs;
    }
    g_cache[fn] = img;
    return img;
}

}  // namespace

struct rvshim_file {
    std::shared_ptr<BamImage> img;
};
struct rvshim_index {
    std::shared_ptr<BamImage> img;
};
struct rvshim_iter {
    std::shared_ptr<BamImage> img;
    size_t cur, stop;
    int32_t tid;
    int64_t beg, end;
};
struct rvshim_fai {
    struct Entry { int64_t len, off; int lb, lw; };
    std::map<std::string, Entry> ents;
    std::string path;
};

samFile *sam_open(const char *fn, const char *mode) {
    (void)mode;
    auto img = load_bam(fn);
    if (!img) return nullptr;
    samFile *f = new rvshim_file;
    f->img = img;
    return f;
}

int sam_close(samFile *fp) { delete fp; return 0; }

bam_hdr_t *sam_hdr_read(samFile *fp) {
    bam_hdr_t *h = (bam_hdr_t *)calloc(1, sizeof(bam_hdr_t));
    int n = (int)fp->img->names.size();
    h->n_targets = n;
    h->target_len = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    h->target_name = (char **)malloc(sizeof(char *) * (n ? n : 1));
    for (int i = 0; i < n; ++i) {
        h->target_len[i] = fp->img->lens[i];
        h->target_name[i] = strdup(fp->img->names[i].c_str());
    }
    return h;
}

void bam_hdr_destroy(bam_hdr_t *h) {
    if (!h) return;
    for (int i = 0; i < h->n_targets; ++i) free(h->target_name[i]);
    free(h->target_name);
    free(h->target_len);
    free(h);
}

hts_idx_t *sam_index_load(samFile *fp, const char *fn) {
    (void)fn;
    hts_idx_t *x = new rvshim_index;
    x->img = fp->img;
    return x;
}

void hts_idx_destroy(hts_idx_t *idx) { delete idx; }
void hts_itr_destroy(hts_itr_t *iter) { delete iter; }

static bool parse_region(const char *reg, std::string &name, int64_t &beg, int64_t &end) {
    std::string s(reg);
    size_t colon = s.rfind(':');
    beg = 0;
    end = INT64_MAX;
    if (colon == std::string::npos) { name = s; return true; }
    name = s.substr(0, colon);
    std::string rest;
    for (char c : s.substr(colon + 1)) if (c != ',') rest.push_back(c);
    size_t dash = rest.find('-');
    long long b = atoll(rest.substr(0, dash).c_str());
    beg = b > 0 ? b - 1 : 0;
    if (dash != std::string::npos && dash + 1 < rest.size()) end = atoll(rest.substr(dash + 1).c_str());
    else if (dash == std::string::npos) end = beg + 1;
    return true;
}

hts_itr_t *sam_itr_querys(const hts_idx_t *idx, bam_hdr_t *hdr, const char *region) {
    std::string name;
    int64_t beg, end;
    parse_region(region, name, beg, end);
    int32_t tid = -1;
    for (int i = 0; i < hdr->n_targets; ++i)
        if (name == hdr->target_name[i]) { tid = i; break; }
    hts_itr_t *it = new rvshim_iter;
    it->img = idx->img;
    it->tid = tid;
    it->beg = beg;
    it->end = end;
    const auto &recs = it->img->recs;
    if (tid < 0) { it->cur = it->stop = 0; return it; }
    int64_t lo_pos = beg - it->img->max_span[tid];
    auto lo = std::lower_bound(recs.begin(), recs.end(), std::make_pair(tid, lo_pos),
                               [](const RecEntry &e, const std::pair<int32_t, int64_t> &k) {
                                   return e.tid < k.first || (e.tid == k.first && e.pos < k.second);
                               });
    it->cur = (size_t)(lo - recs.begin());
    it->stop = recs.size();
    return it;
}

static void fill_record(const BamImage &img, const RecEntry &e, bam1_t *b) {
    const uint8_t *base = img.bytes.data() + e.offset;
    uint32_t bs = rd32(base);
    const uint8_t *r = base + 4;
    uint8_t l_read_name = r[8];
    uint32_t n_cigar = rd16(r + 12);
    int32_t l_seq = rdi32(r + 16);
    // pad the read name with NULs so the CIGAR is 4-byte aligned, as htslib does
    uint8_t extranul = (uint8_t)((4 - (l_read_name & 3)) & 3);
    size_t var_len = bs - 32;
    size_t l_data = var_len + extranul;
    size_t need = l_data + 4096;  // slack: RabbitVar may write a longer CIGAR back in place
    if (b->m_data < need) {
        b->data = (uint8_t *)realloc(b->data, need);
        b->m_data = (uint32_t)need;
    }
    memset(b->data, 0, need);
    b->core.tid = rdi32(r);
    b->core.pos = rdi32(r + 4);
    b->core.bin = rd16(r + 10);
    b->core.qual = r[9];
    b->core.l_extranul = extranul;
    b->core.flag = rd16(r + 14);
    b->core.l_qname = (uint16_t)(l_read_name + extranul);
    b->core.n_cigar = n_cigar;
    b->core.l_qseq = l_seq;
    b->core.mtid = rdi32(r + 20);
    b->core.mpos = rdi32(r + 24);
    b->core.isize = rdi32(r + 28);
    const uint8_t *v = r + 32;
    memcpy(b->data, v, l_read_name);
    memcpy(b->data + l_read_name + extranul, v + l_read_name, var_len - l_read_name);
    b->l_data = (int)l_data;
}

int sam_itr_next(samFile *fp, hts_itr_t *it, bam1_t *b) {
    (void)fp;
    const auto &recs = it->img->recs;
    while (it->cur < it->stop) {
        const RecEntry &e = recs[it->cur];
        if (e.tid != it->tid || e.pos >= it->end) { it->cur = it->stop; break; }
        ++it->cur;
        if (e.endpos > it->beg) {
            fill_record(*it->img, e, b);
            return b->l_data;
        }
    }
    return -1;
}

bam1_t *bam_init1(void) { return (bam1_t *)calloc(1, sizeof(bam1_t)); }
void bam_destroy1(bam1_t *b) {
    if (!b) return;
    free(b->data);
    free(b);
}

hts_pos_t bam_endpos(const bam1_t *b) {
    if ((b->core.flag & BAM_FUNMAP) || b->core.n_cigar == 0) return b->core.pos + 1;
    int64_t rl = ref_len_of((const uint8_t *)bam_get_cigar(b), b->core.n_cigar);
    return rl ? b->core.pos + rl : b->core.pos + 1;
}

static int aux_type_size(uint8_t t) {
    switch (t) {
    case 'A': case 'c': case 'C': return 1;
    case 's': case 'S': return 2;
    case 'i': case 'I': case 'f': return 4;
    default: return -1;
    }
}

uint8_t *bam_aux_get(const bam1_t *b, const char tag[2]) {
    uint8_t *p = bam_get_aux(b), *end = b->data + b->l_data;
    while (p + 3 <= end) {
        uint8_t t = p[2];
        if (p[0] == (uint8_t)tag[0] && p[1] == (uint8_t)tag[1]) return p + 2;
        uint8_t *q = p + 3;
        int sz = aux_type_size(t);
        if (sz > 0) q += sz;
        else if (t == 'Z' || t == 'H') { while (q < end && *q) ++q; ++q; }
        else if (t == 'B') {
            uint8_t sub = q[0];
            uint32_t cnt = rd32(q + 1);
            q += 5 + (size_t)cnt * aux_type_size(sub);
        } else return nullptr;
        p = q;
    }
    return nullptr;
}

int64_t bam_aux2i(const uint8_t *s) {
    switch (s[0]) {
    case 'c': return (int8_t)s[1];
    case 'C': return s[1];
    case 's': { int16_t v; memcpy(&v, s + 1, 2); return v; }
    case 'S': return rd16(s + 1);
    case 'i': return rdi32(s + 1);
    case 'I': return rd32(s + 1);
    default: return 0;
    }
}

char *bam_aux2Z(const uint8_t *s) {
    if (!s || (s[0] != 'Z' && s[0] != 'H')) return nullptr;
    return (char *)(s + 1);
}

faidx_t *fai_load(const char *fn) {
    std::string idxp = std::string(fn) + ".fai";
    FILE *f = fopen(idxp.c_str(), "r");
    if (!f) return nullptr;
    faidx_t *fai = new rvshim_fai;
    fai->path = fn;
    char name[4096];
    long long len, off;
    int lb, lw;
    while (fscanf(f, "%4095s %lld %lld %d %d", name, &len, &off, &lb, &lw) == 5)
        fai->ents[name] = {len, off, lb, lw};
    fclose(f);
    return fai;
}

void fai_destroy(faidx_t *fai) { delete fai; }

char *fai_fetch(const faidx_t *fai, const char *reg, int *len) {
    std::string name;
    int64_t beg, end;
    parse_region(reg, name, beg, end);
    auto it = fai->ents.find(name);
    if (it == fai->ents.end()) { *len = -2; return nullptr; }
    const auto &e = it->second;
    if (end > e.len) end = e.len;
    if (beg > end) beg = end;
    int64_t n = end - beg;
    char *out = (char *)malloc((size_t)n + 1);
    FILE *f = fopen(fai->path.c_str(), "rb");
    int64_t k = 0;
    if (f) {
        for (int64_t i = beg; i < end; ++i) {
            int64_t fo = e.off + (i / e.lb) * e.lw + (i % e.lb);
            if (i == beg || (i % e.lb) == 0) fseek(f, fo, SEEK_SET);
            int c = fgetc(f);
            if (c == EOF) break;
            out[k++] = (char)c;
        }
        fclose(f);
    }
    out[k] = 0;
    *len = (int)k;
    return out;
}

double kt_fisher_exact(int n11, int n12, int n21, int n22,
                       double *left, double *right, double *two) {
    return rv_oracle_fisher(n11, n12, n21, n22, left, right, two);
}
