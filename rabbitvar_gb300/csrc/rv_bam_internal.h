// rv_bam_internal.h -- the rv_bam handle shared by the host BGZF/BAM decoder
// (rv_bam.cpp) and the device decoder (rv_bgzf.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "rvgpu_io.h"

// BGZF members of a whole file: compressed payload [in_off, in_off + in_len)
// inflating to [out_off, out_off + out_len) of the stream.
struct BgzfMember {
    uint64_t in_off, out_off;
    uint32_t in_len, out_len;
};

// Grow-only buffers (device / pinned host) reused across decodes.
template <class T>
struct DArr {
    T *p = nullptr;
    size_t cap = 0;
    bool grow(size_t n) {
        if (p && n <= cap) return true;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t c = std::max<size_t>(n, 1) + n / 8;
        if (cudaMalloc((void **)&p, c * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = c;
        return true;
    }
    void release() {
        cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};
template <class T>
struct HArr {
    T *p = nullptr;
    size_t cap = 0;
    bool grow(size_t n) {
        if (p && n <= cap) return true;
        cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t c = std::max<size_t>(n, 1) + n / 8;
        if (cudaHostAlloc((void **)&p, c * sizeof(T), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = c;
        return true;
    }
    void release() {
        cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// State of a BAM decoded on the GPU (rv_bam_read_gpu): the inflated stream,
// the record offsets, every record's fixed fields, CIGAR words, bases and
// qualities in a batch layout over all records in file order (device); the
// per-read fields, CIGAR words and layout offsets mirrored in pinned host
// memory (the host lays out regions and tiles from them).  Buffers only grow,
// so a second decode into the same handle allocates nothing.
struct BamGpu {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t total = 0;
    int64_t n_rec = 0, n_cig = 0, n_bases = 0;
    DArr<uint8_t> d_in, d_data;
    DArr<BgzfMember> d_mem;
    DArr<int64_t> d_chunk;  // ChunkOut records (3 words each)
    DArr<int64_t> d_first, d_base;
    DArr<int32_t> d_count, d_err;
    DArr<uint64_t> d_rec, d_boff;
    DArr<int32_t> d_tid, d_pos, d_mpos, d_nm, d_lq;
    DArr<uint16_t> d_flag, d_nc;
    DArr<uint8_t> d_mapq, d_seq, d_qual;
    DArr<uint32_t> d_cigoff, d_cig;
    HArr<int32_t> h_tid, h_pos, h_mpos, h_nm, h_lq;
    HArr<uint16_t> h_flag, h_nc;
    HArr<uint8_t> h_mapq;
    HArr<uint32_t> h_cigoff, h_cig;
    HArr<uint64_t> h_boff;
    // records of each reference id: [lo, hi) span in file order and count
    // (index 0 is tid -1)
    std::vector<int64_t> tid_lo, tid_hi, tid_n;
    std::vector<void *> batch_dev, batch_host;  // per-batch buffers (gathered or rebased batches)
};

struct rv_bam {
    std::vector<std::string> names;
    std::vector<int32_t> lens;
    std::vector<const char *> name_ptrs;
    std::vector<uint8_t> data;        // inflated BAM stream (host decoder)
    std::vector<size_t> rec_off;      // record offsets (block_size field)
    std::vector<int32_t> rec_tid;
    std::vector<void *> owned;        // batch buffers
    std::string err;
    BamGpu *gpu = nullptr;            // set by rv_bam_read_gpu
};

// Walks the gzip member headers (BC extra subfield = member size - 1);
// false on a malformed header or an ISIZE above 64 KiB.
bool bgzf_members(const uint8_t *raw, size_t n, std::vector<BgzfMember> &out, uint64_t &total);

// Reference names and lengths of a BAM header held in `d` (the first `n`
// bytes of the stream); returns the header's length in bytes, 0 when `n` is
// too short (needs more bytes), -1 when malformed.
int64_t bam_parse_header(const uint8_t *d, uint64_t n, uint64_t total, rv_bam *bam);

// Device-decoded batches (rv_bgzf.cu).
rv_status bam_gpu_batch(rv_bam *bam, int tid, rv_read_batch *out, bool host_bases);
void bam_gpu_free(BamGpu *g);
void bam_gpu_drop_batches(BamGpu *g);
