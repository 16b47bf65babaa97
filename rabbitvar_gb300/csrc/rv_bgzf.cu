// BGZF/BAM decode on the GPU (the record side of RecordPreprocessor,
// src/recordPreprocessor.cpp:10-32,101-180, which the reference obtains from
// htslib's BGZF reader and record iterator).  Written from the SAM/BAM v1
// specification (BGZF 4.1, records 4.2) and RFC 1951.
//
//   host     walk the gzip member headers (18+ bytes each) -> member table
//   k_inflate          one warp per member (lanes in lockstep, parallel
//                      table fills and match copies), tables in shared memory
//   host     BAM header (reference names/lengths) from the stream's first bytes
//   k_bam_chunks       one warp per member-sized chunk of the stream: the
//                      first plausible record start (a lane per candidate
//                      offset, three chained records checked), then the
//                      chain of block_size fields to the chunk's end
//   host     verify the chunk starts as one chain from the header's end (a
//            chunk whose start disagrees is re-walked from the right offset)
//   k_bam_index        record offsets, one thread per chunk
//   k_bam_fields       fixed fields + NM tag, one thread per record
//   host     select one contig's records, prefix sums of CIGAR words and
//            32-aligned base slots (per-read fields are mirrored on the host,
//            which lays out regions and tiles from them)
//   k_bam_unpack       CIGAR words, 4-bit bases and qualities, one warp per read
//
// Every device access is bounded: members by their compressed length and
// ISIZE, records by the chain-verified block_size, aux fields by the record.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "rv_bam_internal.h"
#include "rv_inflate.cuh"
#include "rvgpu_io.h"

namespace {

// phase times on stderr with RV_TRACE set
struct Lap {
    bool on = getenv("RV_TRACE") != nullptr;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void operator()(const char *phase) {
        if (!on) return;
        auto n = std::chrono::steady_clock::now();
        fprintf(stderr, "trace bam_gpu %s %.3f\n", phase, std::chrono::duration<double, std::milli>(n - t).count());
        t = n;
    }
};

constexpr int kInflateWarps = 4;  // members per block (one warp each; tables 4 x 2.5 KB of shared memory)

struct ChunkOut {
    int64_t first;   // first record start found in the chunk, -1 none
    int64_t end;     // first record start at or after the chunk's end (walk end)
    int32_t count;   // records starting in the chunk
    int32_t status;  // 1: the walk met an impossible block_size
};

__global__ void __launch_bounds__(kInflateWarps * 32) k_inflate(const uint8_t *in, uint64_t in_bytes,
                                                                const BgzfMember *m, int n, uint8_t *out,
                                                                int32_t *err) {
    __shared__ rvz::Tables tabs[kInflateWarps];
    const int wib = threadIdx.x >> 5;
    const int i = blockIdx.x * kInflateWarps + wib;
    if (i >= n) return;  // whole warps leave together
    const BgzfMember mb = m[i];
    if (mb.out_len == 0) return;
    const rvz::Lanes w{(int)(threadIdx.x & 31), 32};
    const int e = rvz::inflate(in + mb.in_off, mb.in_len, in + in_bytes, out + mb.out_off, mb.out_len, tabs[wib], w);
    if (e && w.lane == 0) atomicCAS(err, 0, (e << 24) | (i & 0xFFFFFF));
}

__device__ void walk_chunk(const uint8_t *d, uint64_t total, uint64_t start, uint64_t E, ChunkOut &c) {
    uint64_t o = start;
    int32_t cnt = 0;
    c.status = 0;
    while (o < E) {
        if (o + 4 > total) break;  // trailing bytes shorter than a block_size field
        const uint32_t bs = rvz::rd32(d + o);
        if (bs < 32 || bs > total - o - 4) {
            c.status = 1;
            break;
        }
        o += 4 + (uint64_t)bs;
        cnt++;
    }
    c.first = (int64_t)start;
    c.end = (int64_t)o;
    c.count = cnt;
}

__device__ bool chain_plausible(const uint8_t *d, uint64_t total, uint64_t o, int32_t n_ref) {
    for (int k = 0; k < 3; k++) {
        if (o == total) return true;
        uint32_t bs;
        if (!rvz::record_plausible(d, total, o, n_ref, &bs)) return false;
        o += 4 + (uint64_t)bs;
    }
    return true;
}

// One warp per chunk (chunk = one member's output range).
__global__ void k_bam_chunks(const uint8_t *d, uint64_t total, uint64_t header_end, int32_t n_ref,
                             const BgzfMember *m, int n, ChunkOut *out) {
    const int lane = threadIdx.x & 31;
    const int c = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    if (c >= n) return;
    const uint64_t S = m[c].out_off, E = S + m[c].out_len;
    ChunkOut r;
    r.first = -1;
    r.end = (int64_t)E;
    r.count = 0;
    r.status = 0;
    int64_t start = -1;
    if (E > header_end && E > S) {
        if (S <= header_end) {
            start = (int64_t)header_end;
        } else {
            for (uint64_t base = S; base < E && start < 0; base += 32) {
                const uint64_t o = base + lane;
                const bool ok = o < E && chain_plausible(d, total, o, n_ref);
                const unsigned bal = __ballot_sync(0xFFFFFFFFu, ok);
                if (bal) start = (int64_t)(base + __ffs(bal) - 1);
            }
        }
    }
    if (lane == 0) {
        if (start >= 0) walk_chunk(d, total, (uint64_t)start, E, r);
        out[c] = r;
    }
}

// Re-walk of one chunk from a known start (the chain's).
__global__ void k_bam_walk(const uint8_t *d, uint64_t total, uint64_t start, uint64_t E, ChunkOut *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    ChunkOut r;
    walk_chunk(d, total, start, E, r);
    *out = r;
}

// Record offsets: one thread per chunk walks its verified chain again.
__global__ void k_bam_index(const uint8_t *d, uint64_t total, const int64_t *first, const int64_t *base,
                            const int32_t *count, int n, uint64_t *rec) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || first[c] < 0) return;
    uint64_t o = (uint64_t)first[c];
    uint64_t *w = rec + base[c];
    for (int k = 0; k < count[c]; k++) {
        w[k] = o;
        o += 4 + (uint64_t)rvz::rd32(d + o);
    }
}

// Fixed fields and the NM tag of every record.  status bit 1: a record whose
// block_size does not hold its name, CIGAR and sequence.
__global__ void k_bam_fields(const uint8_t *d, const uint64_t *rec, int64_t n, int32_t *tid, int32_t *pos,
                             int32_t *mpos, int32_t *nm, int32_t *lq, uint16_t *flag, uint16_t *nc, uint8_t *mapq,
                             int32_t *status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t o = rec[i];
        const uint32_t bs = rvz::rd32(d + o);
        const uint8_t *r = d + o + 4;
        const uint32_t lrn = r[8], ncig = rvz::rd16(r + 12);
        const int32_t l = (int32_t)rvz::rd32(r + 16);
        tid[i] = (int32_t)rvz::rd32(r);
        pos[i] = (int32_t)rvz::rd32(r + 4);
        mapq[i] = r[9];
        nc[i] = (uint16_t)ncig;
        flag[i] = (uint16_t)rvz::rd16(r + 14);
        lq[i] = l;
        mpos[i] = (int32_t)rvz::rd32(r + 24);
        int32_t v = INT32_MIN;
        const uint64_t fixed = 32ull + lrn + 4ull * ncig + (l < 0 ? 0ull : ((uint64_t)l + 1) / 2 + (uint64_t)l);
        if (l < 0 || fixed > bs) {
            atomicOr(status, 1);
            nm[i] = v;
            lq[i] = 0;
            nc[i] = 0;
            continue;
        }
        // optional fields: tag[2] type value ...
        uint64_t a = fixed;
        while (a + 3 <= bs) {
            const uint8_t t = r[a + 2];
            const uint64_t val = a + 3;
            const int sz = (t == 'A' || t == 'c' || t == 'C') ? 1
                           : (t == 's' || t == 'S')           ? 2
                           : (t == 'i' || t == 'I' || t == 'f') ? 4
                                                                : -1;
            if (r[a] == 'N' && r[a + 1] == 'M' && sz > 0) {
                if (val + sz > bs) break;
                switch (t) {
                case 'c': v = (int8_t)r[val]; break;
                case 'C': v = r[val]; break;
                case 's': v = (int16_t)rvz::rd16(r + val); break;
                case 'S': v = (int32_t)rvz::rd16(r + val); break;
                case 'i':
                case 'I': v = (int32_t)rvz::rd32(r + val); break;
                default: v = 0; break;  // 'A' / 'f': counted as 0, as the host decoder does
                }
                break;
            }
            if (sz > 0) {
                a = val + sz;
            } else if (t == 'Z' || t == 'H') {
                uint64_t q = val;
                while (q < bs && r[q]) q++;
                a = q + 1;
            } else if (t == 'B') {
                if (val + 5 > bs) break;
                const uint8_t sub = r[val];
                const uint64_t cnt = rvz::rd32(r + val + 1);
                const int es = (sub == 'c' || sub == 'C') ? 1 : (sub == 's' || sub == 'S') ? 2 : 4;
                a = val + 5 + cnt * es;
            } else {
                break;
            }
        }
        nm[i] = v;
    }
}

// One warp per selected read: CIGAR words, packed bases and qualities.
__global__ void k_bam_unpack(const uint8_t *d, const uint64_t *rec, const int64_t *sel, int64_t n,
                             const uint32_t *cig_off, const uint64_t *base_off, uint32_t *cigar, uint8_t *seq,
                             uint8_t *qual) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; k < n; k += warps) {
        const uint8_t *r = d + rec[sel[k]] + 4;
        const uint32_t lrn = r[8], ncig = rvz::rd16(r + 12);
        const uint32_t l = rvz::rd32(r + 16);
        const uint8_t *c = r + 32 + lrn;
        uint32_t *cw = cigar + cig_off[k];
        for (uint32_t j = lane; j < ncig; j += 32) cw[j] = rvz::rd32(c + 4 * j);
        const uint8_t *s = c + 4ull * ncig;
        const uint64_t bo = base_off[k];
        uint8_t *so = seq + bo / 2;
        for (uint32_t j = lane; j < (l + 1) / 2; j += 32) so[j] = s[j];
        const uint8_t *q = s + (l + 1) / 2;
        uint8_t *qo = qual + bo;
        for (uint32_t j = lane; j < l; j += 32) qo[j] = q[j];
    }
}

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    T *get(size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T *)p;
    }
};

template <class T>
T *pinned_host(size_t n, std::vector<void *> &owned) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, std::max<size_t>(n, 1) * sizeof(T), cudaHostAllocDefault) != cudaSuccess) return nullptr;
    owned.push_back(p);
    return (T *)p;
}

#define BG_CUDA(x)                                                 \
    do {                                                           \
        cudaError_t e_ = (x);                                      \
        if (e_ != cudaSuccess) {                                   \
            fprintf(stderr, "rv_bam_read_gpu: %s\n", cudaGetErrorString(e_)); \
            return RV_ERR_CUDA;                                    \
        }                                                          \
    } while (0)

int grid_for(int64_t n, int per, int cap = 1 << 20) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, cap));
}

rv_status decode(const uint8_t *bgzf, size_t nbytes, int device, rv_bam *bam) {
    Lap lap;
    std::vector<BgzfMember> mem;
    uint64_t total = 0;
    if (!bgzf_members(bgzf, nbytes, mem, total)) return RV_ERR_FORMAT;
    const int M = (int)mem.size();
    lap("members");
    BG_CUDA(cudaSetDevice(device));
    cudaStream_t s;
    BG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};
    BamGpu *g = new BamGpu();
    bam->gpu = g;
    g->device = device;
    g->total = total;
    DevBuf tmp;
    // compressed bytes and the member table; the stream is padded so that
    // word loads and field reads past the last byte stay in the allocation
    const uint64_t in_pad = (nbytes + 15) / 16 * 16 + 16;
    uint8_t *d_in = tmp.get<uint8_t>(in_pad);
    BgzfMember *d_mem = tmp.get<BgzfMember>((size_t)M);
    int32_t *d_err = tmp.get<int32_t>(4);
    ChunkOut *d_chunk = tmp.get<ChunkOut>((size_t)M);
    if (!d_in || !d_mem || !d_err || !d_chunk) return RV_ERR_CUDA;
    BG_CUDA(cudaMalloc((void **)&g->d_data, total + 64));
    BG_CUDA(cudaMemsetAsync(g->d_data + total, 0, 64, s));
    BG_CUDA(cudaMemsetAsync(d_in + nbytes, 0, in_pad - nbytes, s));
    BG_CUDA(cudaMemsetAsync(d_err, 0, 16, s));
    BG_CUDA(cudaMemcpyAsync(d_in, bgzf, nbytes, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(d_mem, mem.data(), (size_t)M * sizeof(BgzfMember), cudaMemcpyHostToDevice, s));
    if (M > 0)
        k_inflate<<<(M + kInflateWarps - 1) / kInflateWarps, kInflateWarps * 32, 0, s>>>(d_in, nbytes, d_mem, M,
                                                                                      g->d_data, d_err);
    BG_CUDA(cudaGetLastError());
    int32_t err = 0;
    BG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, s));
    // the header from the stream's first bytes (more if it is longer)
    std::vector<uint8_t> head;
    uint64_t have = std::min<uint64_t>(total, 1 << 16);
    int64_t hdr = 0;
    for (;;) {
        head.resize(have);
        BG_CUDA(cudaMemcpyAsync(head.data(), g->d_data, have, cudaMemcpyDeviceToHost, s));
        BG_CUDA(cudaStreamSynchronize(s));
        if (err) {
            fprintf(stderr, "rv_bam_read_gpu: member %d: inflate error %d\n", err & 0xFFFFFF, err >> 24);
            return RV_ERR_FORMAT;
        }
        hdr = bam_parse_header(head.data(), have, total, bam);
        if (hdr != 0) break;
        have = std::min<uint64_t>(total, have * 4);
    }
    if (hdr < 0) return RV_ERR_FORMAT;
    lap("upload+inflate+header");
    const int32_t n_ref = (int32_t)bam->names.size();
    // record starts per chunk, then the chain check on the host
    if (M > 0) k_bam_chunks<<<grid_for((int64_t)M * 32, 256), 256, 0, s>>>(g->d_data, total, (uint64_t)hdr, n_ref,
                                                                           d_mem, M, d_chunk);
    BG_CUDA(cudaGetLastError());
    std::vector<ChunkOut> ch((size_t)M);
    BG_CUDA(cudaMemcpyAsync(ch.data(), d_chunk, (size_t)M * sizeof(ChunkOut), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    lap("chunks");
    std::vector<int64_t> first((size_t)M, -1), base((size_t)M + 1, 0);
    std::vector<int32_t> count((size_t)M, 0);
    uint64_t expect = (uint64_t)hdr;
    for (int c = 0; c < M; c++) {
        const uint64_t S = mem[c].out_off, E = S + mem[c].out_len;
        base[c + 1] = base[c];
        if (E <= expect) continue;  // no record starts here (inside the header or a long record)
        ChunkOut r = ch[c];
        if (r.first != (int64_t)expect || r.status) {
            k_bam_walk<<<1, 32, 0, s>>>(g->d_data, total, expect, E, d_chunk + c);
            BG_CUDA(cudaGetLastError());
            BG_CUDA(cudaMemcpyAsync(&r, d_chunk + c, sizeof r, cudaMemcpyDeviceToHost, s));
            BG_CUDA(cudaStreamSynchronize(s));
            if (r.status) return RV_ERR_FORMAT;
        }
        first[c] = (int64_t)expect;
        count[c] = r.count;
        base[c + 1] = base[c] + r.count;
        expect = (uint64_t)r.end;
    }
    if (expect > total) return RV_ERR_FORMAT;
    lap("verify");
    const int64_t N = base[(size_t)M];
    g->n_rec = N;
    BG_CUDA(cudaMalloc((void **)&g->d_rec, (size_t)std::max<int64_t>(N, 1) * 8));
    int64_t *d_first = tmp.get<int64_t>((size_t)M), *d_base = tmp.get<int64_t>((size_t)M + 1);
    int32_t *d_count = tmp.get<int32_t>((size_t)M);
    if (!d_first || !d_base || !d_count) return RV_ERR_CUDA;
    BG_CUDA(cudaMemcpyAsync(d_first, first.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(d_base, base.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(d_count, count.data(), (size_t)M * 4, cudaMemcpyHostToDevice, s));
    if (M > 0) k_bam_index<<<grid_for(M, 128), 128, 0, s>>>(g->d_data, total, d_first, d_base, d_count, M, g->d_rec);
    BG_CUDA(cudaGetLastError());
    // fixed fields of every record, mirrored to pinned host memory
    const size_t n1 = (size_t)std::max<int64_t>(N, 1);
    int32_t *d_tid = tmp.get<int32_t>(n1), *d_pos = tmp.get<int32_t>(n1), *d_mpos = tmp.get<int32_t>(n1),
            *d_nm = tmp.get<int32_t>(n1), *d_lq = tmp.get<int32_t>(n1);
    uint16_t *d_flag = tmp.get<uint16_t>(n1), *d_nc = tmp.get<uint16_t>(n1);
    uint8_t *d_mapq = tmp.get<uint8_t>(n1);
    if (!d_tid || !d_pos || !d_mpos || !d_nm || !d_lq || !d_flag || !d_nc || !d_mapq) return RV_ERR_CUDA;
    auto &ho = g->host_owned;
    g->h_tid = pinned_host<int32_t>(n1, ho);
    g->h_pos = pinned_host<int32_t>(n1, ho);
    g->h_mpos = pinned_host<int32_t>(n1, ho);
    g->h_nm = pinned_host<int32_t>(n1, ho);
    g->h_lq = pinned_host<int32_t>(n1, ho);
    g->h_flag = pinned_host<uint16_t>(n1, ho);
    g->h_nc = pinned_host<uint16_t>(n1, ho);
    g->h_mapq = pinned_host<uint8_t>(n1, ho);
    if (!g->h_tid || !g->h_pos || !g->h_mpos || !g->h_nm || !g->h_lq || !g->h_flag || !g->h_nc || !g->h_mapq)
        return RV_ERR_CAPACITY;
    if (N > 0)
        k_bam_fields<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(g->d_data, g->d_rec, N, d_tid, d_pos, d_mpos, d_nm,
                                                                 d_lq, d_flag, d_nc, d_mapq, d_err + 1);
    BG_CUDA(cudaGetLastError());
    BG_CUDA(cudaMemcpyAsync(g->h_tid, d_tid, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_pos, d_pos, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_mpos, d_mpos, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_nm, d_nm, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_lq, d_lq, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_flag, d_flag, (size_t)N * 2, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_nc, d_nc, (size_t)N * 2, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_mapq, d_mapq, (size_t)N, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(&err, d_err + 1, 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    lap("index+fields");
    if (err) return RV_ERR_FORMAT;
    return RV_OK;
}

}  // namespace

rv_status bam_gpu_batch(rv_bam *bam, int tid, rv_read_batch *out, bool host_bases) {
    BamGpu *g = bam->gpu;
    const int64_t N = g->n_rec;
    // this contig's records in file order; CIGAR and 32-aligned base slots
    std::vector<int64_t> sel;
    for (int64_t i = 0; i < N; i++)
        if (g->h_tid[i] == tid) sel.push_back(i);
    const int64_t n = (int64_t)sel.size();
    auto &own = bam->owned;
    int32_t *pos = pinned_host<int32_t>(n, own), *mpos = pinned_host<int32_t>(n, own),
            *nm = pinned_host<int32_t>(n, own), *lq = pinned_host<int32_t>(n, own);
    uint16_t *flag = pinned_host<uint16_t>(n, own), *nc = pinned_host<uint16_t>(n, own);
    uint8_t *mapq = pinned_host<uint8_t>(n, own);
    uint32_t *coff = pinned_host<uint32_t>(n, own);
    uint64_t *boff = pinned_host<uint64_t>(n, own);
    if (!pos || !mpos || !nm || !lq || !flag || !nc || !mapq || !coff || !boff) return RV_ERR_CAPACITY;
    int64_t ci = 0, bi = 0;
    for (int64_t k = 0; k < n; k++) {
        const int64_t i = sel[k];
        pos[k] = g->h_pos[i];
        mpos[k] = g->h_mpos[i];
        nm[k] = g->h_nm[i];
        lq[k] = g->h_lq[i];
        flag[k] = g->h_flag[i];
        nc[k] = g->h_nc[i];
        mapq[k] = g->h_mapq[i];
        coff[k] = (uint32_t)ci;
        boff[k] = (uint64_t)bi;
        ci += nc[k];
        bi += ((int64_t)lq[k] + 31) / 32 * 32;
    }
    if (ci > (int64_t)UINT32_MAX) return RV_ERR_UNSUPPORTED;
    uint32_t *cig = pinned_host<uint32_t>((size_t)ci, own);
    if (!cig) return RV_ERR_CAPACITY;
    BG_CUDA(cudaSetDevice(g->device));
    cudaStream_t s;
    BG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};
    DevBuf tmp;
    int64_t *d_sel = tmp.get<int64_t>((size_t)n);
    uint32_t *d_coff = tmp.get<uint32_t>((size_t)n), *d_cig = tmp.get<uint32_t>((size_t)ci);
    uint64_t *d_boff = tmp.get<uint64_t>((size_t)n);
    if (!d_sel || !d_coff || !d_cig || !d_boff) return RV_ERR_CUDA;
    // bases and qualities stay on the device with the batch (zeroed slots)
    uint8_t *d_seq = nullptr, *d_qual = nullptr;
    BG_CUDA(cudaMalloc((void **)&d_seq, (size_t)bi / 2 + 16));
    g->dev_owned.push_back(d_seq);
    BG_CUDA(cudaMalloc((void **)&d_qual, (size_t)bi + 32));
    g->dev_owned.push_back(d_qual);
    BG_CUDA(cudaMemsetAsync(d_seq, 0, (size_t)bi / 2 + 16, s));
    BG_CUDA(cudaMemsetAsync(d_qual, 0, (size_t)bi + 32, s));
    BG_CUDA(cudaMemcpyAsync(d_sel, sel.data(), (size_t)n * 8, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(d_coff, coff, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(d_boff, boff, (size_t)n * 8, cudaMemcpyHostToDevice, s));
    if (n > 0)
        k_bam_unpack<<<grid_for(n * 32, 256, 152 * 16), 256, 0, s>>>(g->d_data, g->d_rec, d_sel, n, d_coff, d_boff,
                                                                     d_cig, d_seq, d_qual);
    BG_CUDA(cudaGetLastError());
    BG_CUDA(cudaMemcpyAsync(cig, d_cig, (size_t)ci * 4, cudaMemcpyDeviceToHost, s));
    const uint8_t *seq = d_seq, *qual = d_qual;
    if (host_bases) {
        uint8_t *hs = pinned_host<uint8_t>((size_t)bi / 2 + 16, own), *hq = pinned_host<uint8_t>((size_t)bi + 32, own);
        if (!hs || !hq) return RV_ERR_CAPACITY;
        BG_CUDA(cudaMemcpyAsync(hs, d_seq, (size_t)bi / 2 + 16, cudaMemcpyDeviceToHost, s));
        BG_CUDA(cudaMemcpyAsync(hq, d_qual, (size_t)bi + 32, cudaMemcpyDeviceToHost, s));
        seq = hs;
        qual = hq;
    }
    BG_CUDA(cudaStreamSynchronize(s));
    out->n_reads = n;
    out->pos = pos;
    out->flag = flag;
    out->mapq = mapq;
    out->mpos = mpos;
    out->nm = nm;
    out->n_cigar = nc;
    out->cig_off = coff;
    out->cigar = cig;
    out->n_cigar_words = ci;
    out->l_qseq = lq;
    out->base_off = boff;
    out->seq = seq;
    out->qual = qual;
    out->n_bases = bi;
    return RV_OK;
}

void bam_gpu_free(BamGpu *g) {
    if (!g) return;
    cudaSetDevice(g->device);
    cudaFree(g->d_data);
    cudaFree(g->d_rec);
    for (void *p : g->dev_owned) cudaFree(p);
    for (void *p : g->host_owned) cudaFreeHost(p);
    delete g;
}

extern "C" rv_status rv_bam_read_gpu(const uint8_t *bgzf, size_t n, int device, rv_bam **out) {
    if (!bgzf || !out) return RV_ERR_ARG;
    *out = nullptr;
    rv_bam *bam = new rv_bam();
    const rv_status st = decode(bgzf, n, device, bam);
    if (st != RV_OK) {
        rv_bam_free(bam);
        return st;
    }
    *out = bam;
    return RV_OK;
}
