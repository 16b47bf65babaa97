// rv_bam_internal.h -- the rv_bam handle shared by the host BGZF/BAM decoder
// (rv_bam.cpp) and the device decoder (rv_bgzf.cu).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "rvgpu_io.h"

// State of a BAM decoded on the GPU (rv_bam_read_gpu): the inflated stream,
// the record offsets and the per-record fixed fields stay on the device; the
// fields the host needs to lay out a batch are mirrored in pinned memory.
struct BamGpu {
    int device = 0;
    uint8_t *d_data = nullptr;     // inflated stream, zero-padded
    uint64_t total = 0;
    uint64_t *d_rec = nullptr;     // record offsets (block_size field)
    int64_t n_rec = 0;
    // per record, in file order (host mirrors, pinned)
    int32_t *h_tid = nullptr, *h_pos = nullptr, *h_mpos = nullptr, *h_nm = nullptr, *h_lq = nullptr;
    uint16_t *h_flag = nullptr, *h_nc = nullptr;
    uint8_t *h_mapq = nullptr;
    std::vector<void *> dev_owned;  // device buffers of batches handed out
    std::vector<void *> host_owned; // pinned buffers of this state
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

// BGZF members of a whole file: compressed payload [in_off, in_off + in_len)
// inflating to [out_off, out_off + out_len) of the stream.
struct BgzfMember {
    uint64_t in_off, out_off;
    uint32_t in_len, out_len;
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
