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
//   host     prefix sums of CIGAR words and 32-aligned base slots over all
//            records (host threads; the per-read fields are mirrored on the
//            host, which lays out regions and tiles from them), and each
//            reference id's span of records
//   k_bam_unpack       CIGAR words, 4-bit bases and qualities of every record
//                      into that layout, one warp per read
//   rv_bam_batch       a contig whose records are contiguous (a sorted BAM)
//                      is a window of the layout; otherwise its records are
//                      gathered by a second k_bam_unpack
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
#include "rv_pool.h"
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

constexpr int kInflateWarps = 2;  // warps (members) per block

struct ChunkOut {
    int64_t first;   // first record start found in the chunk, -1 none
    int64_t end;     // first record start at or after the chunk's end (walk end)
    int32_t count;   // records starting in the chunk
    int32_t status;  // 1: the walk met an impossible block_size
};

// One warp per member: its lanes run the bit-level decoder in lockstep and
// share table fills and match copies; its tables live in shared memory.
__global__ void __launch_bounds__(kInflateWarps * 32) k_inflate(const uint8_t *in, uint64_t in_bytes,
                                                                const BgzfMember *m, int n, uint8_t *out,
                                                                int32_t *err) {
    __shared__ rvz::Tables tabs[kInflateWarps];
    const int wib = threadIdx.x >> 5;
    const int i = blockIdx.x * kInflateWarps + wib;
    if (i >= n) return;  // whole warps leave together
    const BgzfMember mb = m[i];
    if (mb.out_len == 0) return;
    const rvz::Lanes w{(int)(threadIdx.x & 31), 32, 0xFFFFFFFFu};
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

// One warp per selected read (every read when sel is null): CIGAR words,
// packed bases and qualities.
__global__ void k_bam_unpack(const uint8_t *d, const uint64_t *rec, const int64_t *sel, int64_t n,
                             const uint32_t *cig_off, const uint64_t *base_off, uint32_t *cigar, uint8_t *seq,
                             uint8_t *qual) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; k < n; k += warps) {
        const uint8_t *r = d + rec[sel ? sel[k] : k] + 4;
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

#define BG_CUDA(x)                                                            \
    do {                                                                      \
        cudaError_t e_ = (x);                                                 \
        if (e_ != cudaSuccess) {                                              \
            fprintf(stderr, "rv_bam_read_gpu: %s\n", cudaGetErrorString(e_)); \
            return RV_ERR_CUDA;                                               \
        }                                                                     \
    } while (0)

int grid_for(int64_t n, int per, int cap = 1 << 20) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, cap));
}

template <class T>
T *pinned_host(size_t n, std::vector<void *> &owned) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, std::max<size_t>(n, 1) * sizeof(T), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    owned.push_back(p);
    return (T *)p;
}

template <class T>
T *device_buf(size_t n, std::vector<void *> &owned) {
    void *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    owned.push_back(p);
    return (T *)p;
}

rv_status decode(const uint8_t *bgzf, size_t nbytes, rv_bam *bam) {
    Lap lap;
    BamGpu *g = bam->gpu;
    std::vector<BgzfMember> mem;
    uint64_t total = 0;
    if (!bgzf_members(bgzf, nbytes, mem, total)) return RV_ERR_FORMAT;
    const int M = (int)mem.size();
    lap("members");
    BG_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = g->stream;
    g->total = total;
    g->n_rec = g->n_cig = g->n_bases = 0;
    // compressed bytes and the member table; the stream is padded so that
    // word loads and field reads past the last byte stay in the allocation
    const uint64_t in_pad = (nbytes + 15) / 16 * 16 + 16;
    if (!g->d_in.grow(in_pad) || !g->d_mem.grow((size_t)M) || !g->d_err.grow(4) ||
        !g->d_chunk.grow((size_t)M * 3) || !g->d_data.grow(total + 64))
        return RV_ERR_CUDA;
    uint8_t *d_in = g->d_in.p, *d_data = g->d_data.p;
    BgzfMember *d_mem = g->d_mem.p;
    int32_t *d_err = g->d_err.p;
    ChunkOut *d_chunk = (ChunkOut *)g->d_chunk.p;
    static_assert(sizeof(ChunkOut) == 24, "ChunkOut is three words");
    BG_CUDA(cudaMemsetAsync(d_data + total, 0, 64, s));
    BG_CUDA(cudaMemsetAsync(d_in + nbytes, 0, in_pad - nbytes, s));
    BG_CUDA(cudaMemsetAsync(d_err, 0, 16, s));
    BG_CUDA(cudaMemcpyAsync(d_in, bgzf, nbytes, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(d_mem, mem.data(), (size_t)M * sizeof(BgzfMember), cudaMemcpyHostToDevice, s));
    if (lap.on) {
        BG_CUDA(cudaStreamSynchronize(s));
        lap("upload");
    }
    if (M > 0)
        k_inflate<<<(M + kInflateWarps - 1) / kInflateWarps, kInflateWarps * 32, 0, s>>>(d_in, nbytes, d_mem, M,
                                                                                      d_data, d_err);
    BG_CUDA(cudaGetLastError());
    int32_t err = 0;
    BG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, s));
    // the header from the stream's first bytes (more if it is longer)
    std::vector<uint8_t> head;
    uint64_t have = std::min<uint64_t>(total, 1 << 16);
    int64_t hdr = 0;
    for (;;) {
        head.resize(have);
        BG_CUDA(cudaMemcpyAsync(head.data(), d_data, have, cudaMemcpyDeviceToHost, s));
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
    lap("inflate+header");
    const int32_t n_ref = (int32_t)bam->names.size();
    // record starts per chunk, then the chain check on the host
    if (M > 0) k_bam_chunks<<<grid_for((int64_t)M * 32, 256), 256, 0, s>>>(d_data, total, (uint64_t)hdr, n_ref,
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
            k_bam_walk<<<1, 32, 0, s>>>(d_data, total, expect, E, d_chunk + c);
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
    const size_t n1 = (size_t)std::max<int64_t>(N, 1);
    if (!g->d_first.grow((size_t)M) || !g->d_base.grow((size_t)M + 1) || !g->d_count.grow((size_t)M) ||
        !g->d_rec.grow(n1) || !g->d_tid.grow(n1) || !g->d_pos.grow(n1) || !g->d_mpos.grow(n1) ||
        !g->d_nm.grow(n1) || !g->d_lq.grow(n1) || !g->d_flag.grow(n1) || !g->d_nc.grow(n1) ||
        !g->d_mapq.grow(n1) || !g->d_cigoff.grow(n1) || !g->d_boff.grow(n1))
        return RV_ERR_CUDA;
    if (!g->h_tid.grow(n1) || !g->h_pos.grow(n1) || !g->h_mpos.grow(n1) || !g->h_nm.grow(n1) ||
        !g->h_lq.grow(n1) || !g->h_flag.grow(n1) || !g->h_nc.grow(n1) || !g->h_mapq.grow(n1) ||
        !g->h_cigoff.grow(n1) || !g->h_boff.grow(n1))
        return RV_ERR_CAPACITY;
    BG_CUDA(cudaMemcpyAsync(g->d_first.p, first.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g->d_base.p, base.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g->d_count.p, count.data(), (size_t)M * 4, cudaMemcpyHostToDevice, s));
    if (M > 0)
        k_bam_index<<<grid_for(M, 128), 128, 0, s>>>(d_data, total, g->d_first.p, g->d_base.p, g->d_count.p, M,
                                                     g->d_rec.p);
    BG_CUDA(cudaGetLastError());
    if (N > 0)
        k_bam_fields<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(d_data, g->d_rec.p, N, g->d_tid.p, g->d_pos.p,
                                                                 g->d_mpos.p, g->d_nm.p, g->d_lq.p, g->d_flag.p,
                                                                 g->d_nc.p, g->d_mapq.p, d_err + 1);
    BG_CUDA(cudaGetLastError());
    BG_CUDA(cudaMemcpyAsync(g->h_tid.p, g->d_tid.p, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_nc.p, g->d_nc.p, (size_t)N * 2, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_lq.p, g->d_lq.p, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(&err, d_err + 1, 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    if (err) return RV_ERR_FORMAT;
    // the rest of the per-read fields come back while the host lays out the batch
    BG_CUDA(cudaMemcpyAsync(g->h_pos.p, g->d_pos.p, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_mpos.p, g->d_mpos.p, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_nm.p, g->d_nm.p, (size_t)N * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_flag.p, g->d_flag.p, (size_t)N * 2, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(g->h_mapq.p, g->d_mapq.p, (size_t)N, cudaMemcpyDeviceToHost, s));
    lap("index+fields");
    // batch layout over all records in file order: CIGAR word offsets and
    // 32-aligned base slots (prefix sums on the host threads); the records
    // of each reference id
    {
        const int64_t nch = rv::chunks_for(N, 1 << 16);
        std::vector<int64_t> cs((size_t)nch + 1, 0), bs((size_t)nch + 1, 0);
        struct Run {
            int32_t tid;
            int64_t lo, hi, n;
        };
        std::vector<std::vector<Run>> runs((size_t)nch);
        rv::parallel_chunks(N, 1 << 16, [&](int64_t k, int64_t a, int64_t e) {
            int64_t c = 0, b = 0;
            std::vector<Run> &rk = runs[(size_t)k];
            for (int64_t i = a; i < e; i++) {
                c += g->h_nc.p[i];
                b += ((int64_t)g->h_lq.p[i] + 31) / 32 * 32;
                const int32_t t = g->h_tid.p[i];
                if (rk.empty() || rk.back().tid != t) rk.push_back(Run{t, i, i + 1, 1});
                else {
                    rk.back().hi = i + 1;
                    rk.back().n++;
                }
            }
            cs[(size_t)k + 1] = c;
            bs[(size_t)k + 1] = b;
        });
        for (int64_t k = 0; k < nch; k++) {
            cs[(size_t)k + 1] += cs[(size_t)k];
            bs[(size_t)k + 1] += bs[(size_t)k];
        }
        if (cs[(size_t)nch] > (int64_t)UINT32_MAX) return RV_ERR_UNSUPPORTED;
        rv::parallel_chunks(N, 1 << 16, [&](int64_t k, int64_t a, int64_t e) {
            int64_t c = cs[(size_t)k], b = bs[(size_t)k];
            for (int64_t i = a; i < e; i++) {
                g->h_cigoff.p[i] = (uint32_t)c;
                g->h_boff.p[i] = (uint64_t)b;
                c += g->h_nc.p[i];
                b += ((int64_t)g->h_lq.p[i] + 31) / 32 * 32;
            }
        });
        g->n_cig = cs[(size_t)nch];
        g->n_bases = bs[(size_t)nch];
        // each reference id's span from the runs of equal ids (file order)
        g->tid_lo.assign((size_t)n_ref + 1, -1);
        g->tid_hi.assign((size_t)n_ref + 1, -1);
        g->tid_n.assign((size_t)n_ref + 1, 0);
        for (const auto &rk : runs)
            for (const Run &r : rk) {
                if (r.tid < -1 || r.tid >= n_ref) continue;  // cannot happen: fields were range-checked
                const size_t k = (size_t)(r.tid + 1);
                if (g->tid_lo[k] < 0) g->tid_lo[k] = r.lo;
                g->tid_hi[k] = r.hi;
                g->tid_n[k] += r.n;
            }
    }
    lap("layout");
    if (!g->d_cig.grow((size_t)g->n_cig) || !g->d_seq.grow((size_t)g->n_bases / 2 + 16) ||
        !g->d_qual.grow((size_t)g->n_bases + 32) || !g->h_cig.grow((size_t)g->n_cig))
        return RV_ERR_CUDA;
    BG_CUDA(cudaMemcpyAsync(g->d_cigoff.p, g->h_cigoff.p, (size_t)N * 4, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g->d_boff.p, g->h_boff.p, (size_t)N * 8, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemsetAsync(g->d_seq.p, 0, (size_t)g->n_bases / 2 + 16, s));
    BG_CUDA(cudaMemsetAsync(g->d_qual.p, 0, (size_t)g->n_bases + 32, s));
    if (N > 0)
        k_bam_unpack<<<grid_for(N * 32, 256, 152 * 16), 256, 0, s>>>(d_data, g->d_rec.p, nullptr, N, g->d_cigoff.p,
                                                                     g->d_boff.p, g->d_cig.p, g->d_seq.p, g->d_qual.p);
    BG_CUDA(cudaGetLastError());
    BG_CUDA(cudaMemcpyAsync(g->h_cig.p, g->d_cig.p, (size_t)g->n_cig * 4, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    g->n_rec = N;
    lap("unpack");
    return RV_OK;
}

}  // namespace

void bam_gpu_drop_batches(BamGpu *g) {
    for (void *p : g->batch_dev) cudaFree(p);
    for (void *p : g->batch_host) cudaFreeHost(p);
    g->batch_dev.clear();
    g->batch_host.clear();
}

rv_status bam_gpu_batch(rv_bam *bam, int tid, rv_read_batch *out, bool host_bases) {
    BamGpu *g = bam->gpu;
    const int64_t N = g->n_rec;
    BG_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = g->stream;
    const int64_t k = (int64_t)tid + 1;
    const bool known = k >= 0 && k < (int64_t)g->tid_n.size();
    const int64_t n = known ? g->tid_n[(size_t)k] : 0;
    const int64_t lo = n > 0 ? g->tid_lo[(size_t)k] : 0;
    memset(out, 0, sizeof *out);
    out->n_reads = n;
    if (n == 0 || g->tid_hi[(size_t)k] - lo == n) {
        // the contig's records are contiguous in the file (a sorted BAM):
        // the batch is a window of the all-records layout
        const int64_t hi = lo + n;
        const uint32_t c0 = n ? g->h_cigoff.p[lo] : 0;
        const uint64_t b0 = n ? g->h_boff.p[lo] : 0;
        const int64_t c1 = hi < N ? (int64_t)g->h_cigoff.p[hi] : g->n_cig;
        const int64_t b1 = hi < N ? (int64_t)g->h_boff.p[hi] : g->n_bases;
        out->pos = g->h_pos.p + lo;
        out->flag = g->h_flag.p + lo;
        out->mapq = g->h_mapq.p + lo;
        out->mpos = g->h_mpos.p + lo;
        out->nm = g->h_nm.p + lo;
        out->n_cigar = g->h_nc.p + lo;
        out->l_qseq = g->h_lq.p + lo;
        out->cigar = g->h_cig.p + c0;
        out->n_cigar_words = c1 - (int64_t)c0;
        out->n_bases = b1 - (int64_t)b0;
        if (lo == 0) {
            out->cig_off = g->h_cigoff.p;
            out->base_off = g->h_boff.p;
        } else {
            uint32_t *co = pinned_host<uint32_t>((size_t)n, g->batch_host);
            uint64_t *bo = pinned_host<uint64_t>((size_t)n, g->batch_host);
            if (!co || !bo) return RV_ERR_CAPACITY;
            for (int64_t i = 0; i < n; i++) {
                co[i] = g->h_cigoff.p[lo + i] - c0;
                bo[i] = g->h_boff.p[lo + i] - b0;
            }
            out->cig_off = co;
            out->base_off = bo;
        }
        out->seq = g->d_seq.p + b0 / 2;
        out->qual = g->d_qual.p + b0;
    } else {
        // records of the contig scattered through the file: gather them
        std::vector<int64_t> sel;
        sel.reserve((size_t)n);
        for (int64_t i = g->tid_lo[(size_t)k]; i < g->tid_hi[(size_t)k]; i++)
            if (g->h_tid.p[i] == tid) sel.push_back(i);
        auto &own = g->batch_host;
        int32_t *pos = pinned_host<int32_t>(n, own), *mpos = pinned_host<int32_t>(n, own),
                *nm = pinned_host<int32_t>(n, own), *lq = pinned_host<int32_t>(n, own);
        uint16_t *flag = pinned_host<uint16_t>(n, own), *nc = pinned_host<uint16_t>(n, own);
        uint8_t *mapq = pinned_host<uint8_t>(n, own);
        uint32_t *coff = pinned_host<uint32_t>(n, own);
        uint64_t *boff = pinned_host<uint64_t>(n, own);
        if (!pos || !mpos || !nm || !lq || !flag || !nc || !mapq || !coff || !boff) return RV_ERR_CAPACITY;
        int64_t ci = 0, bi = 0;
        for (int64_t j = 0; j < n; j++) {
            const int64_t i = sel[(size_t)j];
            pos[j] = g->h_pos.p[i];
            mpos[j] = g->h_mpos.p[i];
            nm[j] = g->h_nm.p[i];
            lq[j] = g->h_lq.p[i];
            flag[j] = g->h_flag.p[i];
            nc[j] = g->h_nc.p[i];
            mapq[j] = g->h_mapq.p[i];
            coff[j] = (uint32_t)ci;
            boff[j] = (uint64_t)bi;
            ci += nc[j];
            bi += ((int64_t)lq[j] + 31) / 32 * 32;
        }
        uint32_t *cig = pinned_host<uint32_t>((size_t)ci, own);
        int64_t *d_sel = device_buf<int64_t>((size_t)n, g->batch_dev);
        uint32_t *d_coff = device_buf<uint32_t>((size_t)n, g->batch_dev), *d_cig = device_buf<uint32_t>((size_t)ci, g->batch_dev);
        uint64_t *d_boff = device_buf<uint64_t>((size_t)n, g->batch_dev);
        uint8_t *d_seq = device_buf<uint8_t>((size_t)bi / 2 + 16, g->batch_dev);
        uint8_t *d_qual = device_buf<uint8_t>((size_t)bi + 32, g->batch_dev);
        if (!cig || !d_sel || !d_coff || !d_cig || !d_boff || !d_seq || !d_qual) return RV_ERR_CAPACITY;
        BG_CUDA(cudaMemsetAsync(d_seq, 0, (size_t)bi / 2 + 16, s));
        BG_CUDA(cudaMemsetAsync(d_qual, 0, (size_t)bi + 32, s));
        BG_CUDA(cudaMemcpyAsync(d_sel, sel.data(), (size_t)n * 8, cudaMemcpyHostToDevice, s));
        BG_CUDA(cudaMemcpyAsync(d_coff, coff, (size_t)n * 4, cudaMemcpyHostToDevice, s));
        BG_CUDA(cudaMemcpyAsync(d_boff, boff, (size_t)n * 8, cudaMemcpyHostToDevice, s));
        k_bam_unpack<<<grid_for(n * 32, 256, 152 * 16), 256, 0, s>>>(g->d_data.p, g->d_rec.p, d_sel, n, d_coff,
                                                                     d_boff, d_cig, d_seq, d_qual);
        BG_CUDA(cudaGetLastError());
        BG_CUDA(cudaMemcpyAsync(cig, d_cig, (size_t)ci * 4, cudaMemcpyDeviceToHost, s));
        BG_CUDA(cudaStreamSynchronize(s));
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
        out->seq = d_seq;
        out->qual = d_qual;
        out->n_bases = bi;
    }
    if (host_bases) {
        const size_t ns = (size_t)(out->n_bases + 1) / 2, nq = (size_t)out->n_bases;
        uint8_t *hs = pinned_host<uint8_t>(ns + 16, g->batch_host), *hq = pinned_host<uint8_t>(nq + 32, g->batch_host);
        if (!hs || !hq) return RV_ERR_CAPACITY;
        BG_CUDA(cudaMemcpyAsync(hs, out->seq, ns, cudaMemcpyDeviceToHost, s));
        BG_CUDA(cudaMemcpyAsync(hq, out->qual, nq, cudaMemcpyDeviceToHost, s));
        BG_CUDA(cudaStreamSynchronize(s));
        out->seq = hs;
        out->qual = hq;
    }
    return RV_OK;
}

void bam_gpu_free(BamGpu *g) {
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    bam_gpu_drop_batches(g);
    g->d_in.release();
    g->d_data.release();
    g->d_mem.release();
    g->d_chunk.release();
    g->d_first.release();
    g->d_base.release();
    g->d_count.release();
    g->d_err.release();
    g->d_rec.release();
    g->d_boff.release();
    g->d_tid.release();
    g->d_pos.release();
    g->d_mpos.release();
    g->d_nm.release();
    g->d_lq.release();
    g->d_flag.release();
    g->d_nc.release();
    g->d_mapq.release();
    g->d_seq.release();
    g->d_qual.release();
    g->d_cigoff.release();
    g->d_cig.release();
    g->h_tid.release();
    g->h_pos.release();
    g->h_mpos.release();
    g->h_nm.release();
    g->h_lq.release();
    g->h_flag.release();
    g->h_nc.release();
    g->h_mapq.release();
    g->h_cigoff.release();
    g->h_cig.release();
    g->h_boff.release();
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

extern "C" rv_status rv_bam_read_gpu(const uint8_t *bgzf, size_t n, int device, rv_bam **out) {
    if (!bgzf || !out) return RV_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return RV_ERR_CUDA;
    }
    rv_bam *bam = new rv_bam();
    bam->gpu = new BamGpu();
    bam->gpu->device = device;
    if (cudaStreamCreateWithFlags(&bam->gpu->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        bam->gpu->stream = nullptr;
        rv_bam_free(bam);
        return RV_ERR_CUDA;
    }
    const rv_status st = decode(bgzf, n, bam);
    if (st != RV_OK) {
        rv_bam_free(bam);
        return st;
    }
    *out = bam;
    return RV_OK;
}

extern "C" rv_status rv_bam_reread_gpu(rv_bam *bam, const uint8_t *bgzf, size_t n) {
    if (!bam || !bam->gpu || !bgzf) return RV_ERR_ARG;
    if (cudaSetDevice(bam->gpu->device) != cudaSuccess) {
        cudaGetLastError();
        return RV_ERR_CUDA;
    }
    cudaStreamSynchronize(bam->gpu->stream);
    bam_gpu_drop_batches(bam->gpu);
    bam->gpu->tid_n.clear();
    bam->gpu->n_rec = 0;
    return decode(bgzf, n, bam);
}
