// Small data-movement kernels at the realigner boundary: compact the used
// hash slots, gather cells for the host realigner, apply its patches.
#include <cuda_runtime.h>

#include <algorithm>

#include "rv_ctx.h"
#include "rv_hash.cuh"

namespace rv {

__global__ void k_compact_slots(DevState st, uint32_t *out, unsigned int *n_out) {
    unsigned long long n = used_count(st.hash);
    for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < n;
         u += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = st.hash.used[u];
        if (st.hash.slots[i].fp != 0ULL) out[atomicAdd(n_out, 1u)] = i;
    }
}

__global__ void k_gather_slots(const Slot *slots, const uint32_t *idx, int64_t n, Slot *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = slots[idx[i]];
}

__global__ void k_gather_cells(DevState st, const int64_t *cells, int64_t n, CellView *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = cells[i];
        CellView v;
        for (int b = 0; b < 4; b++) {
            int64_t g = 4 * c + b;
            v.fwd[b] = st.cells.fwd[g];
            v.rev[b] = st.cells.rev[g];
            v.hi[b] = st.cells.hi[g];
            v.tp[b] = st.cells.tp[g];
            v.q[b] = st.cells.q[g];
            v.mq[b] = st.cells.mq[g];
            v.nm[b] = st.cells.nm[g];
            v.first[b] = st.cells.first[g];
        }
        v.cov = st.cells.cov[c];
        v.kflags = st.cells.kflags[c];
        out[i] = v;
    }
}

// Realigned statistics of one key (SF_OVR: the count rides in first_tp, the
// fractional sums as double bits).
__device__ void set_override(Slot &s, const Patch &q) {
    s.fwd = q.fwd;
    s.rev = q.rev;
    s.hi = q.hi;
    s.lo = q.lo;
    s.extracnt = q.extracnt;
    s.first_tp = q.cnt;
    s.tp_sum = __double_as_longlong(q.tp);
    s.mq_sum = __double_as_longlong(q.mq);
    s.nm_sum = __double_as_longlong(q.nm);
    s.q_sum = q.q_sum;
    s.flags = (s.flags & ~(SF_ERASED | SF_NOMAP | SF_PDIFF | SF_QDIFF | SF_FORCE_STD)) | SF_OVR | (uint32_t)q.flags_or;
}

// Finds or creates the slot of a key the realigner added, sets its
// statistics and links a new slot into its position's list.
__device__ void create_slot(const DevState &st, const Patch &q, const uint8_t *keys) {
    const char *k = (const char *)keys + q.key_off;
    unsigned long long h1, h2;
    key_hashes(q.region, q.kind, q.pos, k, q.klen, h1, h2);
    const Hash &H = st.hash;
    unsigned long long i = h1 & H.mask;
    for (int step = 0; step <= 4096; step++) {
        Slot &s = H.slots[i];
        unsigned long long old = atomicCAS(&s.fp, 0ULL, h1);
        if (old == 0ULL) {
            s.region = q.region;
            s.pos = q.pos;
            s.kind = (uint16_t)q.kind;
            s.klen = (uint16_t)q.klen;
            unsigned long long off = q.klen ? atomicAdd(H.arena_used, (unsigned long long)q.klen) : 0ULL;
            if (off + q.klen > H.arena_cap) {
                atomicOr(st.err, ERR_ARENA_FULL);
                s.koff = 0;
                s.klen = 0;
            } else {
                s.koff = (uint32_t)off;
                for (int j = 0; j < q.klen; j++) H.arena[off + j] = (uint8_t)k[j];
            }
            note_used(H, i);
            s.h2x = h2;
            set_override(s, q);
            const Region &R = st.regions[q.region];
            if (q.pos >= R.clo && q.pos <= R.chi) {
                int64_t c = R.cell_base + (q.pos - R.clo);
                bool clip = q.kind != KIND_NONINS && q.kind != KIND_INS;
                s.next = atomicExch(clip ? &st.head_sc[c] : &st.head[c], (uint32_t)i);
            }
            return;
        }
        if (old == h1) {
            set_override(s, q);
            return;
        }
        i = (i + 1) & H.mask;
    }
    atomicOr(st.err, ERR_HASH_FULL);
}

// Patches are applied by one thread each; a slot or cell key is named by at
// most one statistics patch, and coverage additions use atomics.
__global__ void k_apply_patches(DevState st, const Patch *p, int64_t n, const uint8_t *keys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const Patch &q = p[i];
        if (q.type == 0) {
            Slot &s = st.hash.slots[q.target];
            s.fwd = q.fwd;
            s.rev = q.rev;
            s.hi = q.hi;
            s.lo = q.lo;
            s.extracnt = q.extracnt;
            s.tp_sum = q.tp_sum;
            s.mq_sum = q.mq_sum;
            s.nm_sum = q.nm_sum;
            s.q_sum = q.q_sum;
            s.flags |= (uint32_t)q.flags_or;
        } else if (q.type == 1) {
            atomicOr(&st.hash.slots[q.target].flags, SF_ERASED | (uint32_t)q.flags_or);
        } else if (q.type == 2) {
            int64_t c = q.target;
            atomicOr((unsigned int *)&st.cells.kflags[c & ~3LL], 1u << (4 + q.base + 8 * (c & 3)));
        } else if (q.type == 3) {
            atomicAdd(&st.cells.cov[q.target], (uint32_t)q.cov_add);
        } else if (q.type == 4) {
            set_override(st.hash.slots[q.target], q);
        } else if (q.type == 5) {
            if (keys) create_slot(st, q, keys);
        } else if (q.type == 6) {
            int64_t c = q.target;
            atomicAnd((unsigned int *)&st.cells.kflags[c & ~3LL], ~(0xFFu << (8 * (c & 3))));
        }
    }
}

// ---------------------------------------------------------------------------
// Flattened key lists for the -k 1 realigner's host mirror: the keys of cell
// c (its allele-key list, then its soft-clip list, each in list order) land
// in out[off[c] .. off[c + 1]).
// ---------------------------------------------------------------------------
constexpr int kListLimit = 1 << 20;  // longest list walked (a corrupt list sets ERR_UNSUPPORTED)

__global__ void k_list_count(DevState st, uint32_t *cnt) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < st.cells.n_cells;
         c += (int64_t)gridDim.x * blockDim.x) {
        int n = 0;
        for (int l = 0; l < 2; l++)
            for (uint32_t s = l ? st.head_sc[c] : st.head[c]; s != 0xFFFFFFFFu; s = st.hash.slots[s].next) {
                if (++n > kListLimit) {
                    atomicOr(st.err, ERR_UNSUPPORTED);
                    break;
                }
            }
        cnt[c] = (uint32_t)(n > kListLimit ? 0 : n);
    }
}

// exclusive scan of n values in blocks of 1024 (block sums to bsum)
__global__ void k_scan_blocks(uint32_t *v, int64_t n, uint32_t *bsum) {
    __shared__ uint32_t sh[1024];
    int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    uint32_t x = i < n ? v[i] : 0u;
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        uint32_t y = threadIdx.x >= (unsigned)d ? sh[threadIdx.x - d] : 0u;
        __syncthreads();
        sh[threadIdx.x] += y;
        __syncthreads();
    }
    if (i < n) v[i] = sh[threadIdx.x] - x;
    if (threadIdx.x == 1023) bsum[blockIdx.x] = sh[1023];
}

// exclusive scan of the block sums (one block, chunks of 1024 with a carry);
// bsum[nb] = total
__global__ void k_scan_sums(uint32_t *bsum, int64_t nb) {
    __shared__ uint32_t sh[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
        int64_t i = b0 + threadIdx.x;
        uint32_t x = i < nb ? bsum[i] : 0u;
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int d = 1; d < 1024; d <<= 1) {
            uint32_t y = threadIdx.x >= (unsigned)d ? sh[threadIdx.x - d] : 0u;
            __syncthreads();
            sh[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + sh[threadIdx.x] - x;
        __syncthreads();
        if (threadIdx.x == 0) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void k_scan_add(uint32_t *v, int64_t n, const uint32_t *bsum) {
    int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    if (i < n) v[i] += bsum[blockIdx.x];
    if (i == 0) v[n] = bsum[gridDim.x];
}

__global__ void k_list_fill(DevState st, const uint32_t *off, Slot *out, uint32_t *out_idx) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < st.cells.n_cells;
         c += (int64_t)gridDim.x * blockDim.x) {
        uint32_t k = off[c], e = off[c + 1];
        for (int l = 0; l < 2; l++)
            for (uint32_t s = l ? st.head_sc[c] : st.head[c]; s != 0xFFFFFFFFu && k < e; s = st.hash.slots[s].next) {
                out[k] = st.hash.slots[s];
                out_idx[k] = s;
                k++;
            }
    }
}

// ---------------------------------------------------------------------------
// Soft-clip consensus (findconseq, include/VariationUtils.h:403-509) of every
// clip aggregate in the flattened lists, for the -k 1 realigner.  For an
// aggregate at list index i: meta[i] = bit 31 computed | bit 30 the clip is
// marked used (a low-complexity consensus) | bits 16-29 offset of its
// characters from off[c] in `cons` | bits 0-15 length.  Clips with more than
// kMaxNt per-offset base counts are left to the host (meta[i] = 0).
// ---------------------------------------------------------------------------
constexpr int kMaxNt = 256;

__device__ __forceinline__ int clip_rank_d(char c) {
    // measured iteration order of the reference's hash map over soft-clip
    // bases: N, A, T, G, C
    switch (c) {
    case 'N': return 0;
    case 'A': return 1;
    case 'T': return 2;
    case 'G': return 3;
    case 'C': return 4;
    default: return 5 + (unsigned char)c;
    }
}

// One warp per cell: the lanes zero the cell's meta words and look for clip
// aggregates together (most cells have none); for each aggregate, in list
// order, the lanes gather its per-offset base counts into shared memory
// (list order kept by ballot prefixes), rank them by (offset, base rank) —
// each lane places its entries by counting smaller keys, ties by list
// order, which is the stable order — and lane 0 walks the ranked counts.
constexpr int kConsWarps = 4;
__global__ void __launch_bounds__(32 * kConsWarps)
    k_clip_consensus(const Slot *list, const uint32_t *off, int64_t n_cells, const uint8_t *arena,
                     const unsigned long long *arena_used, uint32_t *meta, uint8_t *cons) {
    __shared__ uint32_t s_key[kConsWarps][kMaxNt];  // offset << 9 | base rank
    __shared__ int s_cnt[kConsWarps][kMaxNt];
    __shared__ double s_q[kConsWarps][kMaxNt];
    __shared__ char s_ch[kConsWarps][kMaxNt];
    __shared__ uint16_t s_ord[kConsWarps][kMaxNt];  // ranked position -> gathered entry
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    uint32_t *key = s_key[wl];
    int *cnt = s_cnt[wl];
    double *q = s_q[wl];
    char *ch = s_ch[wl];
    uint16_t *ord = s_ord[wl];
    const unsigned long long used_bytes = *arena_used;
    const int64_t warps = (int64_t)gridDim.x * kConsWarps;
    for (int64_t c = blockIdx.x * (int64_t)kConsWarps + wl; c < n_cells; c += warps) {
        const uint32_t b = off[c], e = off[c + 1];
        bool any = false;
        for (uint32_t i = b + lane; i < e; i += 32) {
            meta[i] = 0u;
            const int k = list[i].kind;
            any |= k == KIND_SC5 || k == KIND_SC3;
        }
        if (!__any_sync(0xffffffffu, any)) continue;
        __syncwarp();
        uint32_t written = 0;
        for (uint32_t i = b; i < e; i++) {
            const int kind = list[i].kind;
            if (kind != KIND_SC5 && kind != KIND_SC3) continue;
            const int seqk = kind == KIND_SC3 ? KIND_SC3_SEQ : KIND_SC5_SEQ;
            const int agg_cnt = list[i].fwd + list[i].rev;
            int n = 0;
            for (uint32_t j0 = b; j0 < e; j0 += 32) {
                const uint32_t j = j0 + lane;
                bool m = false;
                if (j < e) {
                    const Slot &t = list[j];
                    m = t.kind == seqk && t.klen == 3 && (unsigned long long)t.koff + 3 <= used_bytes;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, m);
                const int pos = n + __popc(bal & ((1u << lane) - 1u));
                if (m && pos < kMaxNt) {
                    const Slot &t = list[j];
                    const uint8_t *kb = arena + t.koff;
                    const char c2 = (char)kb[2];
                    key[pos] = ((uint32_t)(kb[0] | (kb[1] << 8)) << 9) | (uint32_t)clip_rank_d(c2);
                    ch[pos] = c2;
                    cnt[pos] = t.obs;
                    q[pos] = t.q_sum;
                }
                n += __popc(bal);
            }
            // more per-offset counts than the arrays hold: left to the host
            if (n > kMaxNt) continue;
            __syncwarp();
            for (int x = lane; x < n; x += 32) {
                const uint32_t kx = key[x];
                int r = 0;
                for (int y = 0; y < n; y++) {
                    const uint32_t ky = key[y];
                    r += ky < kx || (ky == kx && y < x);
                }
                ord[r] = (uint16_t)x;
            }
            __syncwarp();
            if (lane == 0 && written <= 16383u) {
                int nts = 0;
                for (int x = 0; x < n; x++)
                    if (x == 0 || (key[ord[x]] >> 9) != (key[ord[x - 1]] >> 9)) nts++;
                // the consensus characters go straight to this clip's output range
                uint8_t *out = cons + b + written;
                int total = 0, match = 0, sl = 0;
                bool flag = false;
                for (int x = 0; x < n;) {
                    const uint32_t ix = key[ord[x]] >> 9;
                    int y = x;
                    while (y < n && (key[ord[y]] >> 9) == ix) y++;
                    int maxc = 0, tt = 0;
                    double maxq = 0;
                    char chosen = 0;
                    for (int k = x; k < y; k++) {
                        const int o = ord[k];
                        tt += cnt[o];
                        if (cnt[o] > maxc || q[o] > maxq) {
                            maxc = cnt[o];
                            chosen = ch[o];
                            maxq = q[o];
                        }
                    }
                    if (ix == 3 && nts >= 6 && tt / (double)agg_cnt < 0.2 && tt <= 2) break;
                    if ((tt - maxc > 2 || maxc <= tt - maxc) && maxc / (double)tt < 0.8) {
                        if (flag) break;
                        flag = true;
                    }
                    total += tt;
                    match += maxc;
                    if (chosen != 0) out[sl++] = (uint8_t)chosen;
                    x = y;
                }
                bool keep = total != 0 && match / (double)total > 0.9 && sl / 1.5 > nts - sl &&
                            (sl / (double)nts > 0.8 || nts - sl < 10 || sl > 25);
                int len = sl;
                if (!keep) {
                    out[0] = (uint8_t)' ';
                    len = 1;
                }
                bool used = false;
                if (len > 12) {
                    bool a7 = true, t7 = true;
                    for (int k = 1; k < 8; k++) {
                        a7 = a7 && out[k] == 'A';
                        t7 = t7 && out[k] == 'T';
                    }
                    if (a7 || t7) used = true;
                    const char bases[4] = {'A', 'T', 'G', 'C'};
                    int kinds = 0;
                    bool low = false;
                    for (int m = 0; m < 4; m++) {
                        int cc = 0;
                        for (int k = 0; k < len; k++) cc += out[k] == (uint8_t)bases[m];
                        if (cc > 0) kinds++;
                        if (cc / (double)len > 0.75) low = true;
                    }
                    if (low || kinds < 3) used = true;
                }
                meta[i] = (1u << 31) | (used ? (1u << 30) : 0u) | (written << 16) | (uint32_t)len;
                written += (uint32_t)len;
            }
            written = __shfl_sync(0xffffffffu, written, 0);
        }
    }
}

void launch_clip_consensus(const DevState &st, const uint32_t *off, const Slot *list, uint32_t *meta, uint8_t *cons,
                           cudaStream_t s) {
    const int64_t n = st.cells.n_cells;
    if (n > 0)
        k_clip_consensus<<<(int)std::min<int64_t>((n + kConsWarps - 1) / kConsWarps, 152 * 32), 32 * kConsWarps, 0,
                           s>>>(list, off, n, st.hash.arena, st.hash.arena_used, meta, cons);
}

// MNP keys (A/C/G/T '&' A/C/G/T...) that the realigner's adjustMNP visits.
__global__ void k_select_mnv(DevState st, uint32_t *out, unsigned int *n_out) {
    unsigned long long n = used_count(st.hash);
    for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < n;
         u += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = st.hash.used[u];
        const Slot &s = st.hash.slots[i];
        if (s.fp == 0ULL || s.kind != KIND_NONINS || (s.flags & SF_ERASED) || s.obs <= 0 || s.klen < 3) continue;
        const uint8_t *k = st.hash.arena + s.koff;
        auto acgt = [](uint8_t c) { return c == 'A' || c == 'C' || c == 'G' || c == 'T'; };
        bool ok = k[1] == '&' && acgt(k[0]);
        for (int j = 2; ok && j < s.klen; j++) ok = acgt(k[j]);
        if (ok) out[atomicAdd(n_out, 1u)] = (uint32_t)i;
    }
}

// All keys linked at the requested cells (their per-position lists).
__global__ void k_gather_lists(DevState st, const int64_t *cells, int64_t n, uint32_t *out, unsigned int *n_out,
                               unsigned int cap) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int list = 0; list < 2; list++) {
            int steps = 0;
            uint32_t h = list == 0 ? st.head[cells[i]] : st.head_sc[cells[i]];
            for (uint32_t s = h; s != 0xFFFFFFFFu && steps < (1 << 20); s = st.hash.slots[s].next, steps++) {
                unsigned int k = atomicAdd(n_out, 1u);
                if (k < cap) out[k] = s;
            }
        }
    }
}

void launch_select_mnv(const DevState &st, uint32_t *out, unsigned int *n_out, cudaStream_t s) {
    k_select_mnv<<<592, 256, 0, s>>>(st, out, n_out);
}
void launch_gather_lists(const DevState &st, const int64_t *cells, int64_t n, uint32_t *out, unsigned int *n_out,
                         unsigned int cap, cudaStream_t s) {
    if (n > 0) k_gather_lists<<<(int)((n + 127) / 128 < 1024 ? (n + 127) / 128 : 1024), 128, 0, s>>>(st, cells, n, out, n_out, cap);
}

void launch_compact_slots(const DevState &st, uint32_t *out, unsigned int *n_out, cudaStream_t s) {
    k_compact_slots<<<592, 256, 0, s>>>(st, out, n_out);
}
void launch_gather_slots(const Slot *slots, const uint32_t *idx, int64_t n, Slot *out, cudaStream_t s) {
    if (n > 0) k_gather_slots<<<(int)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048), 256, 0, s>>>(slots, idx, n, out);
}
void launch_gather_cells(const DevState &st, const int64_t *cells, int64_t n, CellView *out, cudaStream_t s) {
    if (n > 0) k_gather_cells<<<(int)((n + 127) / 128 < 2048 ? (n + 127) / 128 : 2048), 128, 0, s>>>(st, cells, n, out);
}
// off has n_cells + 1 entries, bsum (n_cells + 1023) / 1024 + 1
void launch_list_offsets(const DevState &st, uint32_t *off, uint32_t *bsum, cudaStream_t s) {
    const int64_t n = st.cells.n_cells;
    if (n <= 0) return;
    k_list_count<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(st, off);
    const int64_t nb = (n + 1023) / 1024;
    k_scan_blocks<<<(unsigned)nb, 1024, 0, s>>>(off, n, bsum);
    k_scan_sums<<<1, 1024, 0, s>>>(bsum, nb);
    k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(off, n, bsum);
}

void launch_list_fill(const DevState &st, const uint32_t *off, Slot *out, uint32_t *out_idx, cudaStream_t s) {
    const int64_t n = st.cells.n_cells;
    if (n > 0) k_list_fill<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(st, off, out, out_idx);
}

void launch_apply_patches(const DevState &st, const Patch *p, int64_t n, const uint8_t *keys, cudaStream_t s) {
    if (n > 0) k_apply_patches<<<(int)((n + 127) / 128 < 2048 ? (n + 127) / 128 : 2048), 128, 0, s>>>(st, p, n, keys);
}

}  // namespace rv

namespace rv {

// find35match (src/VariationRealigner.cpp:1396-1428) for a batch of soft-clip
// consensus pairs, one thread per pair: pairs[4k..4k+3] = offset and length
// of the 5' clip's string, offset and length of the 3' clip's string in
// `strs`; res[3k..3k+2] = b5, b3, score (0, 0, 0 when no start passes).
// Every start (i, j) in the reference's order; the first that passes wins.
__global__ void k_find35(const int32_t *pairs, int64_t n, const char *strs, int32_t *res) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const char *s5 = strs + pairs[4 * k];
        const int l5 = pairs[4 * k + 1];
        const char *s3 = strs + pairs[4 * k + 2];
        const int l3 = pairs[4 * k + 3];
        int b5 = 0, b3 = 0, score = 0;
        for (int i = 0; i < l5 - 8 && score == 0; i++) {
            for (int j = 1; j < l3 - 8; j++) {
                int nm = 0, m = 0;
                while (m + j <= l3 && i + m <= l5) {
                    if (i + m == l5 || s3[l3 - j - m] != s5[i + m]) nm++;
                    if (nm > 2) break;
                    m++;
                }
                if (m - nm > 8 && nm / (double)m < 0.1 && (m + j >= l3 || i + m >= l5)) {
                    b5 = i;
                    b3 = j;
                    score = m - nm;
                    break;
                }
            }
        }
        res[3 * k] = b5;
        res[3 * k + 1] = b3;
        res[3 * k + 2] = score;
    }
}

void launch_find35(const int32_t *pairs, int64_t n, const char *strs, int32_t *res, cudaStream_t s) {
    if (n <= 0) return;
    const int64_t blocks = (n + 127) / 128;
    k_find35<<<(int)std::min<int64_t>(blocks, 152 * 64), 128, 0, s>>>(pairs, n, strs, res);
}

}  // namespace rv
