// Host mirror of the device-built maps as the local realigner reads them:
// one allele key's statistics (include/Variation.h:12-82), a soft-clip
// aggregate with its per-offset base counts (include/Sclip.h:10-39), and the
// transfers that fill them from the device.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "rv_ctx.h"

namespace rv {

// Statistics of one allele key as the host realigner sees it.
struct HVar {
    int cnt = 0, fwd = 0, rev = 0, hi = 0, lo = 0, extracnt = 0;
    double tp = 0, q = 0, mq = 0, nm = 0;
    bool pstd = false, qstd = false;
    int64_t slot = -1;   // hash slot, or -1 for a cell key
    int64_t cell = -1;
    int base = -1;
    bool dirty = false, erased = false, force_std = false;
};

struct HClip {
    HVar agg;
    std::map<int, std::map<char, std::pair<int, double>>> nt;  // idx -> ch -> (count, quality sum)
    std::string cons;
    bool used = false;
};

// one per-offset base count of a soft clip
struct NtCount {
    int idx;
    char ch;
    int cnt;
    double q;
};
// findconseq (include/VariationUtils.h:403-509) over counts sorted by sort_nt
std::string consensus_of(const std::vector<NtCount> &nt, int agg_cnt, bool &used);
void sort_nt(std::vector<NtCount> &nt);
// findconseq cached in the clip
std::string clip_consensus(HClip &sc);
// adjCnt(to, v) (include/VariationUtils.h:338-352)
void add_into(HVar &to, const HVar &v);
bool is_mnv(const std::string &k);
HVar from_cell(const CellView &v, int b, int64_t cell);
HVar from_slot(const Slot &s, int64_t slot);
std::string slot_key(const rv_ctx *ctx, const Slot &s);
// every used slot and the key arena
rv_status fetch_slots(rv_ctx *ctx, std::vector<Slot> &slots, std::vector<uint32_t> &idx);
rv_status fetch_cells(rv_ctx *ctx, const std::vector<int64_t> &cells, std::vector<CellView> &out);
// copies patches (and the key bytes of type-5 patches) to the device and applies them
rv_status apply_patches(rv_ctx *ctx, const std::vector<Patch> &patches, const std::string &keys);
// the used part of the key arena into ctx->h_arena
rv_status pull_arena(rv_ctx *ctx);

// a device scratch array of at least `need` elements (grown by half again)
template <class T>
rv_status ensure(rv_ctx *ctx, T *&p, size_t &cap, size_t need) {
    if (p && need <= cap) return RV_OK;
    if (p) cudaFree(p);
    p = nullptr;
    size_t n = need + need / 2 > 256 ? need + need / 2 : 256;
    cudaError_t e = cudaMalloc((void **)&p, n * sizeof(T));
    if (e != cudaSuccess) {
        ctx->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return RV_ERR_CUDA;
    }
    cap = n;
    return RV_OK;
}

}  // namespace rv
