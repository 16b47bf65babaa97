// Batch preparation on the device, from the uploaded read arrays: each
// read's span (the positions its walk can touch, as read_span computes it)
// and walk-cost class, the batch's longest span and read, and per region its
// bounds (lowest/highest span, reach, the edge-read flag), its read list
// (reads grouped by class, file order within a class) and its tiles over
// that list with their shared-memory window starts.  The host keeps only
// the region records it derives from the sorted positions.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "rv_ctx.h"
#include "rv_internal.h"

namespace rv {

namespace {

__device__ __forceinline__ int warp_max(int v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_min(int v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum(long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

constexpr int kPrepThreads = 256;
constexpr int kPrepWarps = kPrepThreads / 32;

}  // namespace

// One thread per read (grid-stride).  words[PREP_MAX_SPAN], words[PREP_MAX_LQ]
// start at 1, words[PREP_MISALIGNED] at 0.
__global__ void __launch_bounds__(kPrepThreads) k_read_prep(ReadPrepIn in, ReadPrepOut out) {
    int msp = 1, mlq = 1, bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < in.n; i += (int64_t)gridDim.x * blockDim.x) {
        bad |= (in.base_off[i] & 31u) != 0u ? 1 : 0;
        int nc = in.n_cigar[i];
        const int lq = in.l_qseq[i];
        if ((int64_t)in.cig_off[i] + nc > in.n_cigar_words) {
            bad |= 2;
            nc = 0;  // not read: the batch is refused
        }
        if (lq < 0 || (int64_t)in.base_off[i] + lq > in.n_bases) bad |= 4;
        const uint32_t *c = in.cigar + in.cig_off[i];
        int sp = 0, ins = 0, clip5 = 0, clip3 = 0;
        for (int q = 0; q < nc; q++) {
            const uint32_t w = c[q];
            const int o = (int)(w & 15u);
            if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) sp += (int)(w >> 4);
            if (o == 1) ins += (int)(w >> 4);
        }
        uint8_t cls = 2;
        if (nc > 0) {
            const uint32_t w0 = c[0], wl = c[nc - 1];
            if ((w0 & 15u) == 4u || (w0 & 15u) == 1u) clip5 = (int)(w0 >> 4);
            if ((wl & 15u) == 4u || (wl & 15u) == 1u) clip3 = (int)(wl >> 4);
            // walk-cost class: one M op; soft clips around one M op; anything else
            const uint32_t o0 = w0 & 15u;
            if (nc == 1 && o0 == 0u) cls = 0;
            else if (nc == 2 && ((o0 == 4u && (c[1] & 15u) == 0u) || (o0 == 0u && (c[1] & 15u) == 4u))) cls = 1;
            else if (nc == 3 && o0 == 4u && (c[1] & 15u) == 0u && (c[2] & 15u) == 4u) cls = 1;
        }
        if (!in.widen) ins = 0;
        const int pos1 = in.pos[i] + 1;
        out.span_lo[i] = pos1 - clip5 - 1 - ins;
        out.span_hi[i] = pos1 + sp + clip3 + ins;
        out.cost[i] = cls;
        msp = max(msp, sp);
        mlq = max(mlq, lq);
    }
    msp = warp_max(msp);
    mlq = warp_max(mlq);
    for (int o = 16; o > 0; o >>= 1) bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out.words[PREP_MAX_SPAN], msp);
        atomicMax(&out.words[PREP_MAX_LQ], mlq);
        if (bad) atomicOr(&out.words[PREP_MISALIGNED], bad);
    }
}

// One block per region: its span bounds, reach and edge-read flag (into the
// region record), its read counts per class and, per class, the reads per
// tile (sized so a tile's window fits kTileW positions) and the tile count.
__global__ void __launch_bounds__(kPrepThreads) k_region_prep(RegionPrepArgs a) {
    __shared__ int s_lo[kPrepWarps], s_hi[kPrepWarps], s_reach[kPrepWarps];
    __shared__ long long s_cnt[3][kPrepWarps];
    Region &R = a.regions[blockIdx.x];
    int lo = INT_MAX, hi = INT_MIN, reach = 0;
    long long cnt[3] = {0, 0, 0};
    for (int64_t i = R.r0 + threadIdx.x; i < R.r1; i += blockDim.x) {
        const int sl = a.span_lo[i], sh = a.span_hi[i];
        lo = min(lo, max(sl, 1));
        hi = max(hi, sh);
        reach = max(reach, sh - (a.pos[i] + 1));
        cnt[a.cost[i]]++;
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    lo = warp_min(lo);
    hi = warp_max(hi);
    reach = warp_max(reach);
    for (int c = 0; c < 3; c++) cnt[c] = warp_sum(cnt[c]);
    if (lane == 0) {
        s_lo[w] = lo;
        s_hi[w] = hi;
        s_reach[w] = reach;
        for (int c = 0; c < 3; c++) s_cnt[c][w] = cnt[c];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 1; k < kPrepWarps; k++) {
        lo = min(lo, s_lo[k]);
        hi = max(hi, s_hi[k]);
        reach = max(reach, s_reach[k]);
    }
    RegionTiles t;
    long long start = 0;
    int n_tiles = 0;
    for (int c = 0; c < 3; c++) {
        long long n = 0;
        for (int k = 0; k < kPrepWarps; k++) n += s_cnt[c][k];
        t.start[c] = start;
        t.count[c] = n;
        t.tile0[c] = n_tiles;
        t.per[c] = 1;
        if (n > 0) {
            const double len = (double)(R.end - R.start + 1 + 2 * a.max_lq);
            const double usable = (double)kTileW - a.max_span - a.max_lq - 16.0;  // window = start span + read extent
            const long long tr = (long long)fmax(32.0, fmin((double)kTileReads, usable * ((double)n / len)));
            t.per[c] = tr;
            n_tiles += (int)((n + tr - 1) / tr);
        }
        start += n;
    }
    t.n_tiles = n_tiles;
    a.rtiles[blockIdx.x] = t;
    if (R.r1 > R.r0) {
        R.span_lo = lo;
        R.span_hi = hi;
        R.reach = reach;
        R.serial = hi + kEdgeMargin > R.we ? 1 : 0;
        if (lo < R.clo || hi > R.chi) atomicOr(&a.words[PREP_SPAN_BAD], 1);
    }
}

// Exclusive scan of the regions' tile counts (one block); the total to
// words[PREP_N_TILES].
__global__ void __launch_bounds__(1024) k_tile_scan(RegionTiles *rt, int n_regions, int *words) {
    __shared__ int s_warp[32];
    __shared__ int s_carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int b = 0; b < n_regions; b += blockDim.x) {
        const int r = b + threadIdx.x;
        int v = r < n_regions ? rt[r].n_tiles : 0;
        const int x = v;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v += y;
        }
        if (lane == 31) s_warp[w] = v;
        __syncthreads();
        if (w == 0) {
            int u = lane < nw ? s_warp[lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, u, d);
                if (lane >= d) u += y;
            }
            if (lane < nw) s_warp[lane] = u;
        }
        __syncthreads();
        const int incl = s_carry + (w ? s_warp[w - 1] : 0) + v;
        if (r < n_regions) rt[r].base = incl - x;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) words[PREP_N_TILES] = s_carry;
}

// One block per region: the tile records, then the reads into the region's
// list by class (ballot prefixes keep file order within a class), each read
// lowering its tile's window start unless it is an edge read.
__global__ void __launch_bounds__(kPrepThreads) k_region_fill(RegionFillArgs a) {
    __shared__ int s_cnt[3][kPrepWarps];
    const int r = blockIdx.x;
    const Region &R = a.regions[r];
    const RegionTiles t = a.rtiles[r];
    const int64_t lb = a.list_begin[r];
    for (int k = threadIdx.x; k < t.n_tiles; k += blockDim.x) {
        int c = 0;
        while (c < 2 && k >= t.tile0[c + 1]) c++;
        const long long j = k - t.tile0[c];
        Tile tl;
        tl.region = r;
        tl.wlo = INT_MAX;
        tl.r0 = lb + t.start[c] + j * t.per[c];
        tl.r1 = lb + t.start[c] + min(t.count[c], (j + 1) * t.per[c]);
        a.tiles[t.base + k] = tl;
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    long long next[3] = {t.start[0], t.start[1], t.start[2]};
    for (int64_t i0 = R.r0; i0 < R.r1; i0 += blockDim.x) {
        const int64_t i = i0 + threadIdx.x;
        const int c = i < R.r1 ? (int)a.cost[i] : 3;
        unsigned m[3];
        for (int cc = 0; cc < 3; cc++) {
            m[cc] = __ballot_sync(0xffffffffu, c == cc);
            if (lane == 0) s_cnt[cc][w] = __popc(m[cc]);
        }
        __syncthreads();
        // the warp's lanes of one tile (consecutive entries of a class)
        // lower its window start with one atomic
        int jt = -1, v = INT_MAX;
        if (c < 3) {
            long long p = next[c] + __popc(m[c] & lt);
            for (int k = 0; k < w; k++) p += s_cnt[c][k];
            a.list[lb + p] = (uint32_t)i;
            jt = t.tile0[c] + (int)((p - t.start[c]) / t.per[c]);
            if (a.span_hi[i] + kEdgeMargin <= R.we) v = a.span_lo[i];
        }
        const unsigned peers = __match_any_sync(0xffffffffu, jt);
        v = __reduce_min_sync(peers, v);
        if (jt >= 0 && v != INT_MAX && lane == __ffs(peers) - 1) atomicMin(&a.tiles[t.base + jt].wlo, v);
        for (int cc = 0; cc < 3; cc++)
            for (int k = 0; k < kPrepWarps; k++) next[cc] += s_cnt[cc][k];
        __syncthreads();
    }
    for (int k = threadIdx.x; k < t.n_tiles; k += blockDim.x) {
        Tile &tl = a.tiles[t.base + k];
        tl.wlo = max(tl.wlo, R.clo);
    }
}

void launch_read_prep(const ReadPrepIn &in, const ReadPrepOut &out, int sm_count, cudaStream_t s) {
    if (in.n <= 0) return;
    const int64_t blocks = std::min<int64_t>((in.n + kPrepThreads - 1) / kPrepThreads, (int64_t)sm_count * 16);
    k_read_prep<<<(int)blocks, kPrepThreads, 0, s>>>(in, out);
}

void launch_region_prep(const RegionPrepArgs &a, int n_regions, cudaStream_t s) {
    if (n_regions <= 0) return;
    k_region_prep<<<n_regions, kPrepThreads, 0, s>>>(a);
    k_tile_scan<<<1, 1024, 0, s>>>(a.rtiles, n_regions, a.words);
}

void launch_region_fill(const RegionFillArgs &a, int n_regions, cudaStream_t s) {
    if (n_regions > 0) k_region_fill<<<n_regions, kPrepThreads, 0, s>>>(a);
}

}  // namespace rv
