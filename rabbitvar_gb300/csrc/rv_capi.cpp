// C ABI of librvgpu (include/rvgpu.h): context, device memory, batch upload,
// and the stage sequence pileup -> realign -> score -> format.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <iterator>
#include <cstdlib>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "rv_ctx.h"
#include "rv_pool.h"

namespace rv {
rv_status host_realign_mnp(rv_ctx *ctx);
rv_status host_realign_full(rv_ctx *ctx);
rv_status host_format_records(rv_ctx *ctx, const char *sample, const char *gene, uint8_t *emitted = nullptr);
rv_status host_export_maps(rv_ctx *ctx, int region, const char *stages);
}  // namespace rv

using namespace rv;

#define RV_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);         \
            return RV_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

namespace {

template <class T>
rv_status grow(rv_ctx *ctx, T *&p, size_t &cap, size_t need) {
    if (need <= cap && p) return RV_OK;
    if (p) cudaFree(p);
    p = nullptr;
    size_t n = std::max<size_t>(need + need / 4, 1024);
    RV_CUDA(cudaMalloc((void **)&p, n * sizeof(T)));
    cap = n;
    return RV_OK;
}

// Pinned host buffer of at least `need` bytes (grown with headroom).
rv_status ensure_pinned(rv_ctx *ctx, void **p, size_t &cap, size_t need) {
    if (need <= cap && *p) return RV_OK;
    // a copy queued from the old buffer may still be running
    if (*p) {
        RV_CUDA(cudaDeviceSynchronize());
        cudaFreeHost(*p);
    }
    *p = nullptr;
    cap = 0;
    const size_t n = std::max<size_t>(need + need / 4, 4096);
    RV_CUDA(cudaHostAlloc(p, n, cudaHostAllocDefault));
    cap = n;
    return RV_OK;
}

unsigned long long next_pow2(unsigned long long x) {
    unsigned long long p = 1;
    while (p < x) p <<= 1;
    return p;
}

enum { CNT_TILE = 32, CNT_DEFER = 1, CNT_USED = 2, CNT_ERR = 3, CNT_CAND = 4, CNT_AUX = 5, CNT_FIX = 6,
       CNT_WIDE_INS = 7, CNT_WIDE_SCORE = 10 };

// (Re)allocates the hash table and its used-slot list with `cap` slots.
rv_status alloc_hash(rv_ctx *ctx, unsigned long long cap) {
    if (ctx->d_slots) cudaFree(ctx->d_slots);
    if (ctx->d_used) cudaFree(ctx->d_used);
    ctx->d_slots = nullptr;
    ctx->d_used = nullptr;
    ctx->hash_cap = 0;
    RV_CUDA(cudaMalloc((void **)&ctx->d_slots, cap * sizeof(Slot)));
    RV_CUDA(cudaMalloc((void **)&ctx->d_used, cap * sizeof(uint32_t)));
    ctx->hash_cap = cap;
    ctx->slots_fresh = true;
    return RV_OK;
}

rv_status alloc_arena(rv_ctx *ctx, unsigned long long cap) {
    if (ctx->d_arena) cudaFree(ctx->d_arena);
    ctx->d_arena = nullptr;
    ctx->arena_cap = 0;
    RV_CUDA(cudaMalloc((void **)&ctx->d_arena, cap));
    ctx->arena_cap = cap;
    return RV_OK;
}

rv_status alloc_deferred(rv_ctx *ctx, unsigned int cap) {
    if (ctx->d_deferred) cudaFree(ctx->d_deferred);
    ctx->d_deferred = nullptr;
    ctx->deferred_cap = 0;
    RV_CUDA(cudaMalloc((void **)&ctx->d_deferred, (size_t)cap * sizeof(Deferred)));
    ctx->deferred_cap = cap;
    return RV_OK;
}

rv_status alloc_fix(rv_ctx *ctx, unsigned int cap) {
    if (ctx->d_ofix) cudaFree(ctx->d_ofix);
    ctx->d_ofix = nullptr;
    ctx->ofix_cap = 0;
    RV_CUDA(cudaMalloc((void **)&ctx->d_ofix, (size_t)cap * sizeof(OrderFix)));
    ctx->ofix_cap = cap;
    return RV_OK;
}

}  // namespace

DevState rv_ctx::state() const {
    DevState s;
    s.batch.n_reads = n_reads;
    s.batch.pos = d_pos;
    s.batch.mpos = d_mpos;
    s.batch.nm = d_nm;
    s.batch.l_qseq = d_lq;
    s.batch.flag = d_flag;
    s.batch.n_cigar = d_ncig;
    s.batch.mapq = d_mapq;
    s.batch.cig_off = d_cigoff;
    s.batch.cigar = d_cigar;
    s.batch.base_off = d_boff;
    s.batch.seq = d_seq;
    s.batch.qual = d_qual;
    s.batch.skip = use_skip ? d_skip : nullptr;
    s.batch.max_lq = max_lq;
    s.regions = d_regions;
    s.n_regions = (int32_t)regions.size();
    s.tiles = d_tiles;
    s.n_tiles = (int32_t)n_tiles;
    s.tile_reads = d_tile_reads;
    s.tile_counter = d_counters + CNT_TILE;
    s.cells = cells;
    s.hash.slots = d_slots;
    s.hash.mask = hash_cap ? hash_cap - 1 : 0;
    s.hash.arena = d_arena;
    s.hash.arena_cap = arena_cap;
    s.hash.arena_used = (unsigned long long *)(d_counters + 8);
    s.hash.n_used = d_counters + CNT_USED;
    s.hash.used = d_used;
    s.deferred = d_deferred;
    s.n_deferred = d_counters + CNT_DEFER;
    s.deferred_cap = deferred_cap;
    s.ref = d_ref;
    s.ref_len = ref_len;
    s.err = d_counters + CNT_ERR;
    s.head = d_head;
    s.head_sc = d_head ? d_head + cap_cells : nullptr;
    s.score_base = d_score_base;
    s.n_score = n_score;
    s.cand = d_cand;
    s.n_cand = d_counters + CNT_CAND;
    s.cand_cap = cand_cap;
    s.logfact = d_logfact;
    s.ofix = d_ofix;
    s.n_ofix = d_counters + CNT_FIX;
    s.ofix_cap = ofix_cap;
    s.wide_ins = d_wide;
    s.wide_score = d_wide ? d_wide + wide_cap : nullptr;
    s.n_wide_ins = d_counters + CNT_WIDE_INS;
    s.n_wide_score = d_counters + CNT_WIDE_SCORE;
    s.wide_cap = wide_cap;
    return s;
}

namespace rv {

rv_status device_fisher(rv_ctx *ctx, const int32_t *tables, int64_t n, double *p2) {
    if (n <= 0) return RV_OK;
    RV_CUDA(cudaSetDevice(ctx->device));
    // tables (16 B each) followed by the p-values and ratios (16 B per table)
    size_t need = (size_t)n * 2;
    if (need > ctx->cap_ftab || !ctx->d_ftab) {
        if (ctx->d_ftab) cudaFree(ctx->d_ftab);
        ctx->d_ftab = nullptr;
        size_t cap = std::max<size_t>(need + need / 4, 4096);
        RV_CUDA(cudaMalloc((void **)&ctx->d_ftab, cap * 16));
        ctx->cap_ftab = cap;
    }
    double *dp = (double *)(ctx->d_ftab + 4 * n);
    // through a pinned staging buffer: pageable copies would each wait for the stream
    const size_t stage = (size_t)n * 24;
    if (!ctx->h_fstage || ctx->cap_fstage < stage) {
        if (ctx->h_fstage) cudaFreeHost(ctx->h_fstage);
        ctx->h_fstage = nullptr;
        size_t cap = std::max<size_t>(stage + stage / 4, 1 << 16);
        RV_CUDA(cudaHostAlloc(&ctx->h_fstage, cap, cudaHostAllocDefault));
        ctx->cap_fstage = cap;
    }
    char *hs = (char *)ctx->h_fstage;
    memcpy(hs, tables, (size_t)n * 16);
    RV_CUDA(cudaMemcpyAsync(ctx->d_ftab, hs, (size_t)n * 16, cudaMemcpyHostToDevice, ctx->stream));
    launch_fisher(ctx->d_ftab, n, dp, dp + n, ctx->stream, ctx->d_logfact);
    RV_CUDA(cudaGetLastError());
    RV_CUDA(cudaMemcpyAsync(hs + (size_t)n * 16, dp, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    RV_CUDA(cudaEventRecord(ctx->ev_block, ctx->stream));
    RV_CUDA(cudaEventSynchronize(ctx->ev_block));
    memcpy(p2, hs + (size_t)n * 16, (size_t)n * 8);
    ctx->io_h2d += n * 16;
    ctx->io_d2h += n * 8;
    ctx->kernels += 1;
    return RV_OK;
}

}  // namespace rv

namespace {

// counter words copied back after a scoring kernel
constexpr int kHdrWords = 12;
constexpr unsigned int kScoreRetryBits = ERR_CAND_FULL | ERR_WIDE_INS_SCRATCH | ERR_WIDE_SCORE_SCRATCH;

int64_t *wide_off(rv_ctx *ctx, int list) { return ctx->d_wide_off + (size_t)list * ((size_t)ctx->wide_cap + 1); }

int64_t wide_entries(const rv_ctx *ctx) {
    return ctx->d_wide_scratch ? (int64_t)(ctx->cap_wide_scratch / wide_entry_bytes()) : 0;
}

// The wide pass of one list (k_ins_adjust_wide for list 0, k_score_wide for
// list 1), queued on s behind the kernel that fills the list: the scratch
// offsets from the positions' allele counts (k_wide_offsets), then the
// kernel.  Nothing is read back; a pass whose scratch is too small sets its
// error bit and is run again by the caller after grow_wide_scratch.
void queue_wide(rv_ctx *ctx, int list, const DevParams &dp, cudaStream_t s) {
    DevState st = ctx->state();
    launch_wide_offsets(st, list, wide_off(ctx, list), s);
    if (list == 0) launch_ins_adjust_wide(st, wide_off(ctx, 0), ctx->d_wide_scratch, wide_entries(ctx), s);
    else launch_score_wide(st, dp, wide_off(ctx, 1), ctx->d_wide_scratch, wide_entries(ctx), s);
    ctx->kernels += 2;
}

// Grows the wide scratch to the larger of the two lists' totals (their
// offsets' last entries, from the passes that overflowed), with headroom.
rv_status grow_wide_scratch(rv_ctx *ctx, cudaStream_t s) {
    unsigned int n[2];
    RV_CUDA(cudaMemcpyAsync(&n[0], ctx->d_counters + CNT_WIDE_INS, 4, cudaMemcpyDeviceToHost, s));
    RV_CUDA(cudaMemcpyAsync(&n[1], ctx->d_counters + CNT_WIDE_SCORE, 4, cudaMemcpyDeviceToHost, s));
    RV_CUDA(cudaStreamSynchronize(s));
    int64_t need = 0;
    for (int l = 0; l < 2; l++) {
        int64_t t = 0;
        const unsigned int k = std::min(n[l], ctx->wide_cap);
        RV_CUDA(cudaMemcpyAsync(&t, wide_off(ctx, l) + k, 8, cudaMemcpyDeviceToHost, s));
        RV_CUDA(cudaStreamSynchronize(s));
        need = std::max(need, t);
    }
    const size_t bytes = (size_t)need * wide_entry_bytes();
    if (bytes > ctx->cap_wide_scratch || !ctx->d_wide_scratch) {
        if (ctx->d_wide_scratch) cudaFree(ctx->d_wide_scratch);
        ctx->d_wide_scratch = nullptr;
        ctx->cap_wide_scratch = 0;
        const size_t cap = std::max<size_t>(bytes + bytes / 2, 65536 * wide_entry_bytes());
        RV_CUDA(cudaMalloc(&ctx->d_wide_scratch, cap));
        ctx->cap_wide_scratch = cap;
    }
    return RV_OK;
}

// Grows the candidate buffer to `need` entries with headroom.
rv_status grow_cand(rv_ctx *ctx, unsigned long long need) {
    if (ctx->d_cand) cudaFree(ctx->d_cand);
    ctx->d_cand = nullptr;
    ctx->cand_cap = 0;
    const unsigned int cap = (unsigned int)std::min<unsigned long long>(INT32_MAX, need + need / 4 + 65536);
    RV_CUDA(cudaMalloc((void **)&ctx->d_cand, (size_t)cap * sizeof(CandVar)));
    ctx->cand_cap = cap;
    return RV_OK;
}

// The error bits every score step checks last.
rv_status score_errors(rv_ctx *ctx, const unsigned int *hdr, unsigned int n) {
    if (n > ctx->cand_cap || (hdr[CNT_ERR] & ERR_CAND_FULL)) {
        ctx->err = "candidate buffer overflow";
        return RV_ERR_CAPACITY;
    }
    if (hdr[CNT_ERR] & (ERR_WIDE_INS_SCRATCH | ERR_WIDE_SCORE_SCRATCH)) {
        ctx->err = "wide scratch still too small after regrowth";
        return RV_ERR_CAPACITY;
    }
    if (hdr[CNT_ERR] & ERR_WIDE_FULL) {
        ctx->err = "more positions with many alleles than the wide list holds";
        return RV_ERR_CAPACITY;
    }
    if (hdr[CNT_ERR] & (ERR_UNSUPPORTED | ERR_CELL_RANGE)) {
        char buf[96];
        snprintf(buf, sizeof buf, "score device error bits 0x%x", hdr[CNT_ERR]);
        ctx->err = buf;
        return RV_ERR_UNSUPPORTED;
    }
    return RV_OK;
}

// Scores the listed (region, position) pairs of `ctx` without screens and
// appends their CandVars to the host copy.
// score_list_a queues the kernel, its wide pass and the counters' copy to
// the pinned words; score_list_b waits for them and collects (two contexts'
// lists are queued before either is waited for).
rv_status score_list_a(rv_ctx *ctx, const std::vector<int2> &list) {
    if (list.empty()) return RV_OK;
    if (list.size() > ctx->cap_list || !ctx->d_list) {
        if (ctx->d_list) cudaFree(ctx->d_list);
        ctx->d_list = nullptr;
        size_t cap = std::max<size_t>(list.size() + list.size() / 4, 4096);
        RV_CUDA(cudaMalloc((void **)&ctx->d_list, cap * sizeof(int2)));
        ctx->cap_list = cap;
    }
    cudaStream_t s = ctx->stream;
    RV_CUDA(cudaMemcpyAsync(ctx->d_list, list.data(), list.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
    RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_WIDE_SCORE, 0, 4, s));
    launch_score_list(ctx->state(), ctx->dp, ctx->d_list, (int)list.size(), s);
    queue_wide(ctx, 1, ctx->dp, s);
    RV_CUDA(cudaGetLastError());
    RV_CUDA(cudaMemcpyAsync(ctx->h_cnt, ctx->d_counters, kHdrWords * 4, cudaMemcpyDeviceToHost, s));
    return RV_OK;
}

rv_status score_list_b(rv_ctx *ctx, const std::vector<int2> &list) {
    if (list.empty()) return RV_OK;
    cudaStream_t s = ctx->stream;
    RV_CUDA(cudaStreamSynchronize(s));
    unsigned int hdr[kHdrWords];
    std::memcpy(hdr, ctx->h_cnt, sizeof hdr);
    const unsigned int n0 = (unsigned int)ctx->h_cand.size();
    // a full candidate buffer or too little wide scratch: grow what
    // overflowed and score the list again (the candidates before n0 are
    // already on the host)
    for (int attempt = 0; attempt < 3 && (hdr[CNT_ERR] & kScoreRetryBits); attempt++) {
        rv_status g;
        if ((hdr[CNT_ERR] & ERR_CAND_FULL) && (g = grow_cand(ctx, hdr[CNT_CAND]))) return g;
        if ((hdr[CNT_ERR] & ERR_WIDE_SCORE_SCRATCH) && (g = grow_wide_scratch(ctx, s))) return g;
        RV_CUDA(cudaMemcpyAsync(ctx->d_counters + CNT_CAND, &n0, 4, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_WIDE_SCORE, 0, 4, s));
        DevState st = ctx->state();
        launch_clear_err_bits(st, ~kScoreRetryBits, s);
        launch_score_list(st, ctx->dp, ctx->d_list, (int)list.size(), s);
        queue_wide(ctx, 1, ctx->dp, s);
        RV_CUDA(cudaGetLastError());
        RV_CUDA(cudaMemcpyAsync(hdr, ctx->d_counters, sizeof hdr, cudaMemcpyDeviceToHost, s));
        RV_CUDA(cudaStreamSynchronize(s));
        ctx->kernels += 2;
    }
    const unsigned int n = hdr[CNT_CAND];
    rv_status e = score_errors(ctx, hdr, n);
    if (e) return e;
    ctx->h_cand.resize(n);
    if (n > n0) {
        RV_CUDA(cudaMemcpyAsync(ctx->h_cand.data() + n0, ctx->d_cand + n0, (size_t)(n - n0) * sizeof(CandVar),
                                cudaMemcpyDeviceToHost, s));
        RV_CUDA(cudaStreamSynchronize(s));
    }
    ctx->io_h2d += (int64_t)(list.size() * sizeof(int2));
    ctx->io_d2h += (int64_t)sizeof hdr + (int64_t)(n - n0) * (int64_t)sizeof(CandVar);
    ctx->kernels += 1;
    return RV_OK;
}

std::vector<int2> positions_of(const rv_ctx *ctx) {
    std::vector<int2> v;
    v.reserve(ctx->h_cand.size());
    for (const CandVar &c : ctx->h_cand) v.push_back(make_int2(c.region, c.pos));
    auto lt = [](const int2 &a, const int2 &b) { return a.x != b.x ? a.x < b.x : a.y < b.y; };
    std::sort(v.begin(), v.end(), lt);
    v.erase(std::unique(v.begin(), v.end(), [](const int2 &a, const int2 &b) { return a.x == b.x && a.y == b.y; }),
            v.end());
    return v;
}

// the positions of `a` missing from `b` (both sorted and unique)
std::vector<int2> missing(const std::vector<int2> &a, const std::vector<int2> &b) {
    std::vector<int2> out;
    auto lt = [](const int2 &x, const int2 &y) { return x.x != y.x ? x.x < y.x : x.y < y.y; };
    std::set_difference(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(out), lt);
    return out;
}

bool same_regions(const rv_ctx *a, const rv_ctx *b) {
    if (a->regions.size() != b->regions.size()) return false;
    for (size_t i = 0; i < a->regions.size(); i++)
        if (a->regions[i].start != b->regions[i].start || a->regions[i].end != b->regions[i].end) return false;
    return a->chr == b->chr && a->ref_len == b->ref_len;
}

}  // namespace

extern "C" {

void rv_default_params(rv_params *p) {
    memset(p, 0, sizeof *p);
    p->goodq = 22.5;
    p->vext = 2;
    p->mismatch = 8;
    p->local_realign = 1;
    p->freq = 0.01;
    p->minr = 2;
    p->read_pos_filter = 5;
    p->qratio = 1.5;
    p->mapq_filter = 0;
    p->min_mapq = 0;
    p->lofreq = 0.05;
    p->bias = 0.05;
    p->min_bias_reads = 2;
    p->samfilter = 0x504;
    p->ref_extension = 1200;
    p->svminlen = 1000;
}

const char *rv_last_error(const rv_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

rv_status rv_create(rv_ctx **out, const rv_params *p, int device, size_t hbm_budget) {
    if (!out || !p) return RV_ERR_ARG;
    *out = nullptr;
    rv_ctx *ctx = new rv_ctx();
    ctx->device = device;
    ctx->params = *p;
    ctx->budget = hbm_budget;
    cudaError_t e = cudaSetDevice(device);
    // the context's stream runs at the highest priority; only the tile
    // kernel is launched at the lowest (launch_pileup), so a realigner pass
    // or a scoring kernel queued while another batch's tile kernel runs takes
    // the block slots that kernel's retiring blocks free
    int least = 0, greatest = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    ctx->low_priority = least;
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_up, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    for (int i = 0; e == cudaSuccess && i < 12; i++) e = cudaEventCreate(&ctx->ev[i]);
    // a blocking-wait event for waits off the critical path (the record
    // formatter's Fisher batch): the waiting thread sleeps instead of spinning
    // on a core the host pool needs
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_block, cudaEventBlockingSync | cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_counters, 64 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&ctx->h_cnt, 64 * sizeof(unsigned int), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_prep, PREP_WORDS * sizeof(int));
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&ctx->h_prep, PREP_WORDS * sizeof(unsigned int), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_logfact, (size_t)kLogFact * sizeof(double));
    if (e == cudaSuccess) {
        launch_fill_logfact(ctx->d_logfact, ctx->stream);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        ctx->err = cudaGetErrorString(e);
        *out = ctx;
        return RV_ERR_CUDA;
    }
    DevParams &d = ctx->dp;
    memset(&d, 0, sizeof d);
    d.goodq = p->goodq;
    // the hot loops compare integer base qualities with an integer threshold
    // (FP64 compares are slow on this part)
    d.goodq_i = !(p->goodq > -1e9) ? INT32_MIN : (p->goodq > 1e9 ? INT32_MAX : (int32_t)std::ceil(p->goodq));
    d.freq = p->freq;
    d.qratio = p->qratio;
    d.mapq_filter = p->mapq_filter;
    d.lofreq = p->lofreq;
    d.bias = p->bias;
    d.vext = p->vext;
    d.mismatch = p->mismatch;
    d.local_realign = p->local_realign;
    d.minr = p->minr;
    d.read_pos_filter = p->read_pos_filter;
    d.min_mapq = p->min_mapq;
    d.min_bias_reads = p->min_bias_reads;
    d.samfilter = p->samfilter;
    d.trim_bases_after = p->trim_bases_after;
    d.minmatch = p->minmatch;
    d.dedup = p->dedup;
    d.unique_fwd = p->unique_fwd;
    d.unique_first = p->unique_first;
    d.do_pileup = p->do_pileup;
    d.fisher = p->fisher;
    d.move_indels_3 = p->move_indels_3;
    d.svminlen = p->svminlen;
    d.somatic = p->somatic;
    // -p changes nothing in somatic mode: ToVarsBuilder keeps every position
    // of a pair anyway (src/ToVarsBuilder.cpp:170-175, 228) and the somatic
    // writer does not read it (src/modes/somaticMode.cpp)
    if (p->somatic) d.do_pileup = 0;
    *out = ctx;
    return RV_OK;
}

void rv_destroy(rv_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    void *ptrs[] = {ctx->d_ref, ctx->d_pos, ctx->d_mpos, ctx->d_nm, ctx->d_lq, ctx->d_flag, ctx->d_ncig,
                    ctx->d_mapq, ctx->d_cigoff, ctx->d_cigar, ctx->d_boff, ctx->d_seq, ctx->d_qual,
                    ctx->d_regions, ctx->d_tiles, ctx->d_score_base, ctx->d_cellmem, ctx->d_head, ctx->d_slots,
                    ctx->d_arena, ctx->d_deferred, ctx->d_cand, ctx->d_counters, ctx->d_tmp_idx,
                    ctx->d_tmp_slots, ctx->d_tmp_cells, ctx->d_tmp_views, ctx->d_tmp_n, ctx->d_list,
                    ctx->d_ftab, ctx->d_logfact, ctx->d_skip, ctx->d_patches, ctx->d_patch_keys,
                    ctx->d_list_off, ctx->d_list_bsum, ctx->d_list_idx, ctx->d_list_slots,
                    ctx->d_cons_meta, ctx->d_cons, ctx->d_ofix, ctx->d_used, ctx->d_wide, ctx->d_wide_off,
                    ctx->d_wide_scratch, ctx->d_f35, ctx->d_tile_reads, ctx->d_span_lo, ctx->d_span_hi,
                    ctx->d_cost, ctx->d_list_begin, ctx->d_rtiles, ctx->d_prep};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (ctx->h_mirror) cudaFreeHost(ctx->h_mirror);
    if (ctx->h_mirror_slots) cudaFreeHost(ctx->h_mirror_slots);
    if (ctx->h_fstage) cudaFreeHost(ctx->h_fstage);
    if (ctx->h_cnt) cudaFreeHost(ctx->h_cnt);
    if (ctx->h_prep) cudaFreeHost(ctx->h_prep);
    if (ctx->h_meta) cudaFreeHost(ctx->h_meta);
    for (int i = 0; i < 12; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->ev_block) cudaEventDestroy(ctx->ev_block);
    if (ctx->pileup_exec) cudaGraphExecDestroy(ctx->pileup_exec);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->ev_up) cudaEventDestroy(ctx->ev_up);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

rv_status rv_upload_reference(rv_ctx *ctx, const char *chr, const char *bases, int64_t n) {
    if (!ctx || !bases || n <= 0 || n > INT32_MAX) return RV_ERR_ARG;
    RV_CUDA(cudaSetDevice(ctx->device));
    ctx->chr = chr ? chr : "";
    ctx->ref_host.assign(bases, bases + n);
    for (char &c : ctx->ref_host)
        if (c >= 'a' && c <= 'z') c = (char)(c - 32);
    if (ctx->d_ref) cudaFree(ctx->d_ref);
    ctx->d_ref = nullptr;
    // padded to whole 16-byte words (plus one) so the walk can read the
    // reference in 16-byte windows
    const size_t padded = ((size_t)n + 15) / 16 * 16 + 16;
    RV_CUDA(cudaMalloc((void **)&ctx->d_ref, padded));
    RV_CUDA(cudaMemset(ctx->d_ref, 0, padded));
    RV_CUDA(cudaMemcpy(ctx->d_ref, ctx->ref_host.data(), (size_t)n, cudaMemcpyHostToDevice));
    ctx->ref_len = (int32_t)n;
    return RV_OK;
}

namespace {

// rv_submit_batch in two steps, so that a tumor/normal pair prepares both
// samples before either's bulk upload is queued (one host-to-device copy
// engine serves both: a sample's preparation would otherwise wait behind
// the other's bases and qualities).  submit_prepare: the arrays the
// preparation reads, its kernels (spans, classes, region bounds, read
// lists, tiles) and the context's tables; submit_upload: the rest of the
// batch, and the preparation's results.
// The device read buffers sized for batch b.
rv_status grow_reads(rv_ctx *ctx, const rv_read_batch *b) {
    const int64_t n = b->n_reads;
    size_t cr = ctx->cap_reads, cr2 = cr, cr3 = cr, cr4 = cr, cr5 = cr, cr6 = cr, cr7 = cr, cr8 = cr, cr9 = cr;
    rv_status st;
    size_t need = (size_t)std::max<int64_t>(n, 1);
    if ((st = grow(ctx, ctx->d_pos, cr, need)) || (st = grow(ctx, ctx->d_mpos, cr2, need)) ||
        (st = grow(ctx, ctx->d_nm, cr3, need)) || (st = grow(ctx, ctx->d_lq, cr4, need)) ||
        (st = grow(ctx, ctx->d_flag, cr5, need)) || (st = grow(ctx, ctx->d_ncig, cr6, need)) ||
        (st = grow(ctx, ctx->d_mapq, cr7, need)) || (st = grow(ctx, ctx->d_cigoff, cr8, need)) ||
        (st = grow(ctx, ctx->d_boff, cr9, need)))
        return st;
    ctx->cap_reads = cr;
    size_t cc = ctx->cap_cigar;
    if ((st = grow(ctx, ctx->d_cigar, cc, (size_t)std::max<int64_t>(b->n_cigar_words, 1)))) return st;
    ctx->cap_cigar = cc;
    size_t cb = ctx->cap_bases, cb2 = cb;
    if ((st = grow(ctx, ctx->d_qual, cb, (size_t)std::max<int64_t>(b->n_bases, 32) + 64)) ||
        (st = grow(ctx, ctx->d_seq, cb2, (size_t)std::max<int64_t>(b->n_bases, 32) / 2 + 64)))
        return st;
    ctx->cap_bases = cb;
    return RV_OK;
}

// The arrays of batch b that the preparation reads, or the rest of it, on stream s.
rv_status copy_reads(rv_ctx *ctx, const rv_read_batch *b, cudaStream_t s, bool prep_part) {
    const int64_t n = b->n_reads;
    if (n <= 0) return RV_OK;
    if (prep_part) {
        RV_CUDA(cudaMemcpyAsync(ctx->d_pos, b->pos, n * 4, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_lq, b->l_qseq, n * 4, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_ncig, b->n_cigar, n * 2, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_cigoff, b->cig_off, n * 4, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_boff, b->base_off, n * 8, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_cigar, b->cigar, b->n_cigar_words * 4, cudaMemcpyHostToDevice, s));
    } else {
        // bases and qualities may already be on the device (a batch of a BAM
        // decoded there by rv_bam_read_gpu): the copy direction follows the pointers
        RV_CUDA(cudaMemcpyAsync(ctx->d_mpos, b->mpos, n * 4, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_nm, b->nm, n * 4, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_flag, b->flag, n * 2, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_mapq, b->mapq, n, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_seq, b->seq, (size_t)(b->n_bases + 1) / 2, cudaMemcpyDefault, s));
        RV_CUDA(cudaMemcpyAsync(ctx->d_qual, b->qual, (size_t)b->n_bases, cudaMemcpyDefault, s));
    }
    return RV_OK;
}

// Queues the whole of batch b into the context's read buffers on its copy
// stream, behind the context's last pileup chain (ev[1]): the read arrays
// are not read again after that chain (the realigner, the scoring and the
// formatting of the batch in flight use the maps, and the host arrays), so
// the next batch's upload overlaps them.  The next rv_submit_batch of b on
// this context waits for it instead of copying.
rv_status early_upload(rv_ctx *ctx, const rv_read_batch *b) {
    if (!b || b->n_reads < 0 || b->n_cigar_words < 0 || b->n_bases < 0) return RV_OK;
    rv_status st = grow_reads(ctx, b);
    if (st) return st;
    RV_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev[1], 0));
    if ((st = copy_reads(ctx, b, ctx->copy_stream, true)) || (st = copy_reads(ctx, b, ctx->copy_stream, false)))
        return st;
    RV_CUDA(cudaEventRecord(ctx->ev_up, ctx->copy_stream));
    ctx->early_batch = b;
    return RV_OK;
}

rv_status submit_prepare(rv_ctx *ctx, const rv_read_batch *b, const rv_region *regs, int n_regions,
                         cudaStream_t s) {
    if (!ctx || !b || (!regs && n_regions > 0) || n_regions < 0) return RV_ERR_ARG;
    if (!ctx->d_ref) { ctx->err = "reference not uploaded"; return RV_ERR_STATE; }
    RV_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = b->n_reads;
    if (n < 0 || b->n_cigar_words < 0 || b->n_bases < 0) return RV_ERR_ARG;
    ctx->stage = 0;
    PhaseTimer tm("submit");
    ctx->n_reads = n;
    ctx->n_cigar_words = b->n_cigar_words;
    ctx->n_bases = b->n_bases;
    rv_status st;
    ctx->batch_early = ctx->early_batch == b;
    ctx->early_batch = nullptr;
    if ((st = grow_reads(ctx, b))) return st;
    size_t need = (size_t)std::max<int64_t>(n, 1);
    size_t cp = ctx->cap_prep, cp2 = cp, cp3 = cp;
    if ((st = grow(ctx, ctx->d_span_lo, cp, need)) || (st = grow(ctx, ctx->d_span_hi, cp2, need)) ||
        (st = grow(ctx, ctx->d_cost, cp3, need)))
        return st;
    ctx->cap_prep = std::min(cp, std::min(cp2, cp3));
    ctx->io_h2d = n * (4 + 4 + 4 + 4 + 2 + 2 + 1 + 4 + 8) + b->n_cigar_words * 4;
    {
        cudaPointerAttributes pa;
        const bool dev_bases = n > 0 && cudaPointerGetAttributes(&pa, b->qual) == cudaSuccess &&
                               pa.type == cudaMemoryTypeDevice;
        cudaGetLastError();
        if (!dev_bases) ctx->io_h2d += (b->n_bases + 1) / 2 + b->n_bases;
    }
    ctx->io_d2h = 0;
    // the arrays the batch's preparation reads go up first (the rest is
    // queued behind the preparation's kernels), unless the whole batch was
    // queued early on the copy stream
    if (ctx->batch_early) RV_CUDA(cudaStreamWaitEvent(s, ctx->ev_up, 0));
    else if ((st = copy_reads(ctx, b, s, true))) return st;
    // the batch's longest reference span and read (the region records'
    // bounds) on host threads, and each read's CIGAR inside the batch's
    // words; every other per-read step is the device's
    int max_span = 1, max_lq = 1;
    {
        const int64_t nch = chunks_for(n, 1 << 16);
        std::vector<int> ms((size_t)nch, 1), ml((size_t)nch, 1);
        std::vector<uint8_t> bad((size_t)nch, 0);
        parallel_chunks(n, 1 << 16, [&](int64_t k, int64_t a, int64_t e) {
            int msp = 1, mlq = 1;
            uint8_t bd = 0;
            for (int64_t i = a; i < e; i++) {
                const int nc = b->n_cigar[i];
                if ((int64_t)b->cig_off[i] + nc > b->n_cigar_words) {
                    bd = 1;
                    continue;
                }
                const uint32_t *c = b->cigar + b->cig_off[i];
                int sp = 0;
                for (int q = 0; q < nc; q++) {
                    const uint32_t o = c[q] & 15u;
                    if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) sp += (int)(c[q] >> 4);
                }
                msp = std::max(msp, sp);
                mlq = std::max(mlq, (int)b->l_qseq[i]);
            }
            ms[k] = msp;
            ml[k] = mlq;
            bad[k] = bd;
        });
        bool cig_bad = false;
        for (int64_t k = 0; k < nch; k++) {
            max_span = std::max(max_span, ms[k]);
            max_lq = std::max(max_lq, ml[k]);
            cig_bad |= bad[k] != 0;
        }
        if (cig_bad) { ctx->err = "a read's CIGAR lies outside the batch's CIGAR words"; return RV_ERR_ARG; }
    }
    // per read on the device: its span, walk-cost class and the record
    // checks (read back with the tile count before the pileup)
    RV_CUDA(cudaMemsetAsync(ctx->d_prep, 0, PREP_WORDS * 4, s));
    {
        ReadPrepIn in;
        in.n = n;
        in.pos = ctx->d_pos;
        in.l_qseq = ctx->d_lq;
        in.n_cigar = ctx->d_ncig;
        in.cig_off = ctx->d_cigoff;
        in.cigar = ctx->d_cigar;
        in.base_off = ctx->d_boff;
        in.n_cigar_words = b->n_cigar_words;
        in.n_bases = b->n_bases;
        in.widen = ctx->params.local_realign != 0;
        ReadPrepOut out;
        out.span_lo = ctx->d_span_lo;
        out.span_hi = ctx->d_span_hi;
        out.cost = ctx->d_cost;
        out.words = ctx->d_prep;
        // every buffer the kernel touches exists and holds the batch
        if (n > 0 && (!in.pos || !in.l_qseq || !in.n_cigar || !in.cig_off || !in.cigar || !in.base_off ||
                      !out.span_lo || !out.span_hi || !out.cost || !out.words || ctx->cap_prep < (size_t)n ||
                      ctx->cap_reads < (size_t)n || ctx->cap_cigar < (size_t)b->n_cigar_words)) {
            ctx->err = "batch preparation buffers missing";
            return RV_ERR_STATE;
        }
        launch_read_prep(in, out, ctx->sm_count, s);
        RV_CUDA(cudaGetLastError());
    }
    ctx->max_span = max_span;
    ctx->max_lq = max_lq;
    tm.lap("read prep");
    // -k 1: the realigner reads the batch's alignments again from the
    // caller's arrays (noPassingReads)
    ctx->hb_n = ctx->params.local_realign ? n : 0;
    ctx->hb_pos = b->pos;
    ctx->hb_flag = b->flag;
    ctx->hb_ncig = b->n_cigar;
    ctx->hb_cigoff = b->cig_off;
    ctx->hb_cigar = b->cigar;
    const int pad = max_span + max_lq + 4;
    const rv_params &P = ctx->params;
    ctx->regions.clear();
    ctx->n_tiles = 0;
    ctx->score_base.clear();
    std::vector<int64_t> list_begin;  // per region: its first entry in the tile read list
    int64_t list_total = 0;
    int64_t cell_base = 0, score = 0;
    for (int r = 0; r < n_regions; r++) {
        Region R;
        memset(&R, 0, sizeof R);
        R.start = regs[r].start;
        R.end = regs[r].end;
        if (R.start < 1 || R.end < R.start) { ctx->err = "bad region"; return RV_ERR_ARG; }
        int ext = P.ref_extension, x = P.extend_nt;
        R.ws = R.start - x - ext < 1 ? 1 : R.start - x - ext;
        int seq_end = R.end + x + ext > ctx->ref_len ? ctx->ref_len : R.end + x + ext;
        R.we = seq_end - 17;  // CONF_SEED_1
        R.clo = std::max(1, R.start - pad);
        R.chi = R.end + pad;
        // align the cell base so that a region's kflags words are not shared
        cell_base = (cell_base + 3) & ~3LL;
        R.cell_base = cell_base;
        cell_base += (R.chi - R.clo + 1);
        // reads overlapping [start-1, end): pos < end and pos + span > start-1
        int lo_pos = R.start - 1 - max_span;
        R.r0 = std::lower_bound(b->pos, b->pos + n, lo_pos) - b->pos;
        R.r1 = std::lower_bound(b->pos, b->pos + n, R.end) - b->pos;
        ctx->regions.push_back(R);
        list_begin.push_back(list_total);
        list_total += R.r1 - R.r0;
        ctx->score_base.push_back(score);
        score += R.end - R.start + 1;
    }
    list_begin.push_back(list_total);
    if (n > (int64_t)UINT32_MAX) { ctx->err = "more than 2^32 reads in one batch"; return RV_ERR_ARG; }
    ctx->n_tile_reads = (size_t)list_total;
    size_t &tile_bound = ctx->tile_bound;
    ctx->n_score = score;
    ctx->n_cells = cell_base + 4;
    // -t: RecordPreprocessor::next_record's duplicate filter
    // (src/recordPreprocessor.cpp:152-176), in each region's read order
    ctx->use_skip = false;
    if (P.dedup && n > 0) {
        std::vector<uint8_t> skip((size_t)n, 0), seen((size_t)n, 0);
        for (const Region &R : ctx->regions) {
            std::set<std::string> dups;
            int first_match = 0;
            for (int64_t r = R.r0; r < R.r1; r++) {
                const uint32_t *c = b->cigar + b->cig_off[r];
                int span = 0;
                for (int k = 0; k < b->n_cigar[r]; k++) {
                    int o = c[k] & 15;
                    if (o == 0 || o == 2 || o == 3 || o == 7 || o == 8) span += (int)(c[k] >> 4);
                }
                int endpos = ((b->flag[r] & 4) || span == 0) ? b->pos[r] + 1 : b->pos[r] + span;
                if (endpos <= R.start - 1 || b->pos[r] >= R.end) continue;
                if ((b->flag[r] & P.samfilter) || (int)b->mapq[r] < P.min_mapq || b->l_qseq[r] == 1) continue;
                const int a = b->pos[r] + 1, m = b->mpos[r] + 1;
                if (a != first_match) dups.clear();
                std::string key;
                if (m < 10) {
                    key = std::to_string(a) + ((b->flag[r] & 1) ? "-=-" : "-*-") + std::to_string(m);
                } else if ((b->flag[r] & 1) && (b->flag[r] & 4)) {
                    key = std::to_string(a) + "-";
                    for (int k = 0; k < b->n_cigar[r]; k++) key += std::to_string(c[k] >> 4) + "MIDNSHP=XB"[c[k] & 15];
                } else {
                    continue;
                }
                uint8_t d = dups.count(key) ? 1 : 0;
                if (!d) {
                    dups.insert(key);
                    first_match = a;
                }
                if (seen[r] && skip[r] != d) {
                    ctx->err = "-t: a read is a duplicate in one region and not in an overlapping one";
                    return RV_ERR_UNSUPPORTED;
                }
                seen[r] = 1;
                skip[r] = d;
            }
        }
        size_t cs = ctx->cap_skip;
        if ((st = grow(ctx, ctx->d_skip, cs, (size_t)n))) return st;
        ctx->cap_skip = cs;
        RV_CUDA(cudaMemcpyAsync(ctx->d_skip, skip.data(), (size_t)n, cudaMemcpyHostToDevice, s));
        RV_CUDA(cudaStreamSynchronize(s));
        ctx->io_h2d += n;
        ctx->use_skip = true;
    }
    // region records, score bases and list starts through the context's
    // pinned staging; then per region on the device: its bounds, read list
    // (reads grouped by walk-cost class: one M op, soft clips around one M
    // op, the rest; file order within each, so a tile holds reads of about
    // equal walk cost and its threads reach the tile's end together) and
    // tiles over that list, sized so a tile's window fits kTileW positions,
    // each tile's window starting at the lowest span start of its non-edge
    // reads
    {
        size_t creg = ctx->cap_regions, creg2 = ctx->cap_regions, creg3 = ctx->cap_regions, creg4 = ctx->cap_regions;
        const size_t nr1 = ctx->regions.size() + 1;
        if ((st = grow(ctx, ctx->d_regions, creg, nr1)) || (st = grow(ctx, ctx->d_score_base, creg2, nr1)) ||
            (st = grow(ctx, ctx->d_list_begin, creg3, nr1)) || (st = grow(ctx, ctx->d_rtiles, creg4, nr1)))
            return st;
        ctx->cap_regions = std::min(std::min(creg, creg2), std::min(creg3, creg4));
        // tiles: at most one per 32 reads of each class segment, plus one per segment
        tile_bound = (size_t)list_total / 32 + 3 * ctx->regions.size() + 1;
        size_t ct = ctx->cap_tiles, cl = ctx->cap_tile_reads;
        if ((st = grow(ctx, ctx->d_tiles, ct, tile_bound)) ||
            (st = grow(ctx, ctx->d_tile_reads, cl, (size_t)list_total + 1)))
            return st;
        ctx->cap_tiles = ct;
        ctx->cap_tile_reads = cl;
        auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
        const size_t b_reg = up16(ctx->regions.size() * sizeof(Region)), b_sb = up16(ctx->score_base.size() * 8);
        const size_t b_lb = up16(list_begin.size() * 8);
        if ((st = ensure_pinned(ctx, (void **)&ctx->h_meta, ctx->cap_meta, b_reg + b_sb + b_lb + 16))) return st;
        char *h = ctx->h_meta;
        if (!ctx->regions.empty()) {
            memcpy(h, ctx->regions.data(), ctx->regions.size() * sizeof(Region));
            memcpy(h + b_reg, ctx->score_base.data(), ctx->score_base.size() * 8);
            memcpy(h + b_reg + b_sb, list_begin.data(), list_begin.size() * 8);
            RV_CUDA(cudaMemcpyAsync(ctx->d_regions, h, ctx->regions.size() * sizeof(Region), cudaMemcpyHostToDevice, s));
            RV_CUDA(cudaMemcpyAsync(ctx->d_score_base, h + b_reg, ctx->score_base.size() * 8, cudaMemcpyHostToDevice,
                                    s));
            RV_CUDA(cudaMemcpyAsync(ctx->d_list_begin, h + b_reg + b_sb, list_begin.size() * 8,
                                    cudaMemcpyHostToDevice, s));
            if (!ctx->d_regions || !ctx->d_rtiles || !ctx->d_list_begin || !ctx->d_tiles || !ctx->d_tile_reads ||
                !ctx->d_span_lo || !ctx->d_span_hi || !ctx->d_cost || !ctx->d_prep || !ctx->d_pos) {
                ctx->err = "batch preparation buffers missing";
                return RV_ERR_STATE;
            }
            RegionPrepArgs ra;
            ra.regions = ctx->d_regions;
            ra.span_lo = ctx->d_span_lo;
            ra.span_hi = ctx->d_span_hi;
            ra.pos = ctx->d_pos;
            ra.cost = ctx->d_cost;
            ra.max_span = max_span;
            ra.max_lq = max_lq;
            ra.rtiles = ctx->d_rtiles;
            ra.words = ctx->d_prep;
            launch_region_prep(ra, (int)ctx->regions.size(), s);
            RegionFillArgs fa;
            fa.regions = ctx->d_regions;
            fa.rtiles = ctx->d_rtiles;
            fa.list_begin = ctx->d_list_begin;
            fa.span_lo = ctx->d_span_lo;
            fa.span_hi = ctx->d_span_hi;
            fa.cost = ctx->d_cost;
            fa.list = ctx->d_tile_reads;
            fa.tiles = ctx->d_tiles;
            launch_region_fill(fa, (int)ctx->regions.size(), s);
            RV_CUDA(cudaGetLastError());
        }
        RV_CUDA(cudaMemcpyAsync(ctx->h_prep, ctx->d_prep, PREP_WORDS * 4, cudaMemcpyDeviceToHost, s));
        RV_CUDA(cudaEventRecord(ctx->ev[10], s));
    }
    tm.lap("regions+tiles");
    // cells: 7 x 4 words + first (4 words) per position, plus cov, kflags, head
    size_t need_cells = (size_t)ctx->n_cells;
    if (need_cells > ctx->cap_cells || !ctx->d_cellmem) {
        if (ctx->d_cellmem) cudaFree(ctx->d_cellmem);
        if (ctx->d_head) cudaFree(ctx->d_head);
        ctx->d_cellmem = nullptr;
        ctx->d_head = nullptr;
        size_t cap = need_cells + need_cells / 4 + 1024;
        cap = (cap + 63) & ~(size_t)63;
        RV_CUDA(cudaMalloc(&ctx->d_cellmem, cap * (8 * 16 + 4 + 1)));
        RV_CUDA(cudaMalloc((void **)&ctx->d_head, cap * 8));
        ctx->cap_cells = cap;
    }
    {
        size_t cap = ctx->cap_cells;
        char *m = (char *)ctx->d_cellmem;
        Cells &C = ctx->cells;
        C.fwd = (uint32_t *)m; m += cap * 16;
        C.rev = (uint32_t *)m; m += cap * 16;
        C.hi = (uint32_t *)m; m += cap * 16;
        C.tp = (uint32_t *)m; m += cap * 16;
        C.q = (uint32_t *)m; m += cap * 16;
        C.mq = (uint32_t *)m; m += cap * 16;
        C.nm = (int32_t *)m; m += cap * 16;
        C.first = (uint32_t *)m; m += cap * 16;
        C.cov = (uint32_t *)m; m += cap * 4;
        C.kflags = (uint8_t *)m;
        C.n_cells = ctx->n_cells;
    }
    tm.lap("cells");
    // hash table / arena / deferred / order-fix list sized from the batch (or
    // the capacities rv_set_capacities forced for this batch); every table
    // grows when a pileup overflows it (pileup_finish runs the pileup again)
    {
        const double est = ctx->keys_per_read > 0 ? 2.5 * ctx->keys_per_read * (double)n : (double)n;
        unsigned long long want = next_pow2(std::max<unsigned long long>(1ULL << 16, (unsigned long long)est));
        if (ctx->force_hash) want = next_pow2(ctx->force_hash);
        if (want > ctx->hash_cap || !ctx->d_slots || (ctx->force_hash && want != ctx->hash_cap))
            if ((st = alloc_hash(ctx, want))) return st;
        unsigned long long want_arena = std::max<unsigned long long>(1ULL << 20, (unsigned long long)n * 16);
        if (ctx->force_arena) want_arena = ctx->force_arena;
        if (want_arena > ctx->arena_cap || !ctx->d_arena || (ctx->force_arena && want_arena != ctx->arena_cap))
            if ((st = alloc_arena(ctx, want_arena))) return st;
        unsigned int want_def = (unsigned int)std::min<int64_t>(INT32_MAX, n / 8 + 4096);
        if (ctx->force_deferred) want_def = ctx->force_deferred;
        if (want_def > ctx->deferred_cap || !ctx->d_deferred || (ctx->force_deferred && want_def != ctx->deferred_cap))
            if ((st = alloc_deferred(ctx, want_def))) return st;
        unsigned int want_fix = (unsigned int)std::min<int64_t>(INT32_MAX, n / 64 + 4096);
        if (ctx->force_fix) want_fix = ctx->force_fix;
        if (want_fix > ctx->ofix_cap || !ctx->d_ofix || (ctx->force_fix && want_fix != ctx->ofix_cap))
            if ((st = alloc_fix(ctx, want_fix))) return st;
        ctx->force_hash = ctx->force_arena = 0;
        ctx->force_deferred = ctx->force_fix = 0;
    }
    tm.lap("tables");
    unsigned int want_wide = (unsigned int)std::min<int64_t>(INT32_MAX / 2, score / 8 + 4096);
    if (want_wide > ctx->wide_cap || !ctx->d_wide) {
        if (ctx->d_wide) cudaFree(ctx->d_wide);
        ctx->d_wide = nullptr;
        ctx->wide_cap = 0;
        RV_CUDA(cudaMalloc((void **)&ctx->d_wide, 2 * (size_t)want_wide * sizeof(WidePos)));
        ctx->wide_cap = want_wide;
        // the two lists' scratch offsets (k_wide_offsets)
        if (ctx->d_wide_off) cudaFree(ctx->d_wide_off);
        ctx->d_wide_off = nullptr;
        ctx->cap_wide_off = 0;
        RV_CUDA(cudaMalloc((void **)&ctx->d_wide_off, 2 * ((size_t)want_wide + 1) * sizeof(int64_t)));
        ctx->cap_wide_off = 2 * ((size_t)want_wide + 1);
    }
    // candidates: a few per candidate position; pileup mode scores every position
    const int64_t cand_est = ctx->dp.do_pileup ? 2 * score + 65536 : score / 4 + 1024;
    unsigned int want_cand = (unsigned int)std::min<int64_t>(INT32_MAX, std::max<int64_t>(1 << 16, cand_est));
    if (want_cand > ctx->cand_cap || !ctx->d_cand) {
        if (ctx->d_cand) cudaFree(ctx->d_cand);
        ctx->d_cand = nullptr;
        RV_CUDA(cudaMalloc((void **)&ctx->d_cand, (size_t)want_cand * sizeof(CandVar)));
        ctx->cand_cap = want_cand;
    }
    tm.lap("wide+candidates");
    return RV_OK;
}

rv_status submit_upload(rv_ctx *ctx, const rv_read_batch *b, cudaStream_t s) {
    const int64_t n = b->n_reads;
    // the rest of the batch (the bases and qualities are most of it) after
    // the preparation's kernels
    if (!ctx->batch_early) {
        rv_status st = copy_reads(ctx, b, s, false);
        if (st) return st;
    }
    ctx->prep_pending = true;
    ctx->stage = 1;
    return RV_OK;
}

}  // namespace

// The batch preparation's results, queued by rv_submit_batch and waited for
// here, before the first kernel that needs them (the pileup): the device's
// record checks and the tile count.
rv_status prep_finish(rv_ctx *ctx) {
    if (!ctx->prep_pending) return RV_OK;
    ctx->prep_pending = false;
    RV_CUDA(cudaEventSynchronize(ctx->ev[10]));
    const unsigned int *w = ctx->h_prep;
    rv_status st = RV_OK;
    if (w[PREP_MISALIGNED] & 1u) { ctx->err = "base_off must be a multiple of 32"; st = RV_ERR_ARG; }
    else if (w[PREP_MISALIGNED] & 2u) { ctx->err = "a read's CIGAR lies outside the batch's CIGAR words"; st = RV_ERR_ARG; }
    else if (w[PREP_MISALIGNED] & 4u) { ctx->err = "a read's bases lie outside the batch's bases"; st = RV_ERR_ARG; }
    else if ((int)w[PREP_MAX_SPAN] > ctx->max_span || (int)w[PREP_MAX_LQ] > ctx->max_lq) {
        ctx->err = "the device's read spans disagree with the host's";
        st = RV_ERR_UNSUPPORTED;
    } else if (w[PREP_SPAN_BAD]) {
        ctx->err = "read span outside the region's cell range";
        st = RV_ERR_UNSUPPORTED;
    }
    if (!st) {
        ctx->n_tiles = ctx->regions.empty() ? 0 : (int64_t)w[PREP_N_TILES];
        if ((size_t)ctx->n_tiles > ctx->tile_bound) { ctx->err = "tile count above its bound"; st = RV_ERR_UNSUPPORTED; }
    }
    if (st) ctx->stage = 0;
    return st;
}

namespace {

// Both samples of a pair: both preparations, then both uploads.
rv_status submit_pair(rv_ctx *tumor, rv_ctx *normal, const rv_read_batch *bt, const rv_read_batch *bn,
                      const rv_region *regs, int n_regions) {
    rv_status s = submit_prepare(tumor, bt, regs, n_regions, tumor->stream);
    if (!s && (s = submit_prepare(normal, bn, regs, n_regions, normal->stream))) tumor->err = normal->err;
    if (!s) s = submit_upload(tumor, bt, tumor->stream);
    if (!s && (s = submit_upload(normal, bn, normal->stream))) tumor->err = normal->err;
    return s;
}

}  // namespace

rv_status rv_submit_batch(rv_ctx *ctx, const rv_read_batch *b, const rv_region *regs, int n_regions,
                          void *stream) {
    if (!ctx || !b) return RV_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    rv_status st = submit_prepare(ctx, b, regs, n_regions, s);
    if (st) return st;
    return submit_upload(ctx, b, s);
}

namespace {

// The memsets and kernels of one pileup, queued on s; `marks` records the
// per-stage events (left out when the chain is captured into a graph).
rv_status queue_pileup_chain(rv_ctx *ctx, cudaStream_t s, int resident, int variant, bool marks) {
    size_t cap = ctx->cap_cells;
    RV_CUDA(cudaMemsetAsync(ctx->d_cellmem, 0, cap * (8 * 16 + 4 + 1), s));
    RV_CUDA(cudaMemsetAsync(ctx->d_head, 0xFF, cap * 8, s));
    // the slots the previous run claimed (its used-slot list, whose length is
    // still in the counters), or the whole table when it was just allocated
    if (ctx->slots_fresh) launch_init_slots(ctx->d_slots, ctx->hash_cap, s);
    else launch_clear_used(ctx->d_slots, ctx->d_used, ctx->d_counters + CNT_USED, ctx->hash_cap, s);
    ctx->slots_fresh = false;
    RV_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 64 * sizeof(unsigned int), s));
    RV_CUDA(cudaMemsetAsync(ctx->d_arena, 0, 16, s));
    DevState st = ctx->state();
    if (marks) RV_CUDA(cudaEventRecord(ctx->ev[4], s));
    launch_region_reset(st, s);
    launch_edge_detect(st, ctx->dp, s);
    if (marks) RV_CUDA(cudaEventRecord(ctx->ev[5], s));
    RV_CUDA(launch_pileup(st, ctx->dp, resident, s, variant, ctx->low_priority));
    if (marks) RV_CUDA(cudaEventRecord(ctx->ev[6], s));
    launch_serial(st, ctx->dp, s);
    if (marks) RV_CUDA(cudaEventRecord(ctx->ev[7], s));
    launch_resolve(st, ctx->dp, s);
    launch_fix_order(st, ctx->dp, s);
    launch_link(st, s);
    launch_collisions(st, s);
    RV_CUDA(cudaGetLastError());
    return RV_OK;
}

// The same chain through the context's executable graph: captured from s,
// applied to the graph of the previous batch by cudaGraphExecUpdate (kernel
// arguments, grids and memset sizes may change between batches), instantiated
// again when the update is refused, then launched on s.
rv_status launch_pileup_graph(rv_ctx *ctx, cudaStream_t s, int resident, int variant) {
    cudaGraph_t g = nullptr;
    RV_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    rv_status st = queue_pileup_chain(ctx, s, resident, variant, false);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != RV_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        ctx->err = std::string("pileup graph capture: ") + cudaGetErrorString(e);
        return RV_ERR_CUDA;
    }
    if (ctx->pileup_exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(ctx->pileup_exec, g, &info) != cudaSuccess) {
            (void)cudaGetLastError();  // a refused update is not an error: instantiate anew
            cudaGraphExecDestroy(ctx->pileup_exec);
            ctx->pileup_exec = nullptr;
        }
    }
    if (!ctx->pileup_exec) {
        e = cudaGraphInstantiate(&ctx->pileup_exec, g, 0);
        if (e == cudaSuccess) ctx->graph_instantiations++;
        else ctx->pileup_exec = nullptr;
    }
    cudaGraphDestroy(g);
    RV_CUDA(e);
    RV_CUDA(cudaGraphLaunch(ctx->pileup_exec, s));
    ctx->graph_launches++;
    return RV_OK;
}

// Queues the pileup kernels of the submitted batch on stream s without
// waiting for them; pileup_finish waits and reads the device error word.
rv_status pileup_launch(rv_ctx *ctx, cudaStream_t s) {
    if (ctx->stage < 1) { ctx->err = "rv_pileup before rv_submit_batch"; return RV_ERR_STATE; }
    RV_CUDA(cudaSetDevice(ctx->device));
    rv_status ps = prep_finish(ctx);
    if (ps) return ps;
    // autotuner: unless RV_PILEUP_VARIANT pins one, the first batch of the
    // context runs the whole pileup chain once with every tile-kernel variant
    // (register budget x warp aggregation), timing the tile kernel of each;
    // that batch and the later ones use the fastest
    int nvar = pileup_variants();
    int variant;
    const char *pin = getenv("RV_PILEUP_VARIANT");
    const bool pinned = pin && *pin;
    // blocks of the variant resident at once (sets the tile kernel's per-block quota)
    auto resident_of = [&](int v) {
        const int per_sm = std::max(1, pileup_blocks_per_sm(v));
        return (int)std::max<int64_t>(1, std::min<int64_t>(ctx->n_tiles, (int64_t)per_sm * ctx->sm_count));
    };
    if (pinned) {
        variant = std::max(0, std::min(nvar - 1, atoi(pin)));
    } else {
        if (ctx->variant_runs < nvar && ctx->n_tiles > 0) {
            for (int v = 0; v < nvar; v++) {
                rv_status ts = queue_pileup_chain(ctx, s, resident_of(v), v, true);
                if (ts != RV_OK) return ts;
                RV_CUDA(cudaStreamSynchronize(s));
                float m = 0;
                cudaEventElapsedTime(&m, ctx->ev[5], ctx->ev[6]);
                ctx->variant_ms[v] = m;
            }
            ctx->variant_runs = nvar;
        }
        variant = 0;
        for (int v = 1; v < nvar; v++)
            if (ctx->variant_ms[v] < ctx->variant_ms[variant]) variant = v;
    }
    ctx->variant = variant;
    const int resident = resident_of(variant);
    // the legacy default stream cannot be captured
    const bool graphed = ctx->use_graph && s != nullptr;
    RV_CUDA(cudaEventRecord(ctx->ev[0], s));
    rv_status qs = graphed ? launch_pileup_graph(ctx, s, resident, variant)
                           : queue_pileup_chain(ctx, s, resident, variant, true);
    if (qs != RV_OK) return qs;
    RV_CUDA(cudaEventRecord(ctx->ev[1], s));
    ctx->pileup_graphed = graphed;
    ctx->kernels = 9;  // init_slots, region_reset, edge_detect, pileup_tiles, serial, resolve, fix_order, link, collisions
    ctx->pileup_pin = pinned;
    ctx->mirror_pending = false;
    ctx->stage = 1;  // launched, not finished
    ctx->pileup_pending = true;
    return RV_OK;
}

// Waits for the pileup queued by pileup_launch; timings, autotuner, errors.
// A table that overflowed (hash slots, key arena, deferred subtractions,
// order-dependent entries: the kernels set an error bit and drop the
// observation) is grown to what the run needed and the pileup runs again,
// up to kRetries times; the realigner mirror queued behind the failed run is
// queued again behind the new one.
rv_status pileup_finish(rv_ctx *ctx, cudaStream_t s) {
    if (!ctx->pileup_pending) { ctx->err = "no pileup in flight"; return RV_ERR_STATE; }
    ctx->pileup_pending = false;
    RV_CUDA(cudaSetDevice(ctx->device));
    constexpr int kRetries = 3;
    constexpr unsigned int kCapBits = ERR_HASH_FULL | ERR_ARENA_FULL | ERR_DEFER_FULL | ERR_FIX_FULL;
    unsigned int cnt[16];
    bool retried = false;
    for (int attempt = 0;; attempt++) {
        RV_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters, sizeof cnt, cudaMemcpyDeviceToHost, s));
        RV_CUDA(cudaStreamSynchronize(s));
        const unsigned int cap = cnt[CNT_ERR] & kCapBits;
        if (!cap || attempt >= kRetries) break;
        rv_status st;
        if (cap & ERR_HASH_FULL) {
            // at least one slot per read (the automatic size before any keys
            // were counted), at least four times the table that overflowed
            const unsigned long long want = std::max<unsigned long long>(
                ctx->hash_cap * 4, next_pow2(std::max<unsigned long long>(1ULL << 16, (unsigned long long)ctx->n_reads)));
            if ((st = alloc_hash(ctx, want))) return st;
        }
        if (cap & ERR_ARENA_FULL) {
            unsigned long long need;
            memcpy(&need, cnt + 8, sizeof need);  // arena_used counts every key, also those that did not fit
            need = std::max<unsigned long long>(need, ctx->arena_cap);
            if ((st = alloc_arena(ctx, need + need / 2 + (1ULL << 20)))) return st;
        }
        if (cap & ERR_DEFER_FULL) {
            const unsigned long long need = std::max<unsigned long long>(cnt[CNT_DEFER], ctx->deferred_cap);
            if ((st = alloc_deferred(ctx, (unsigned int)std::min<unsigned long long>(INT32_MAX, need + need / 2 + 4096))))
                return st;
        }
        if (cap & ERR_FIX_FULL) {
            const unsigned long long need = std::max<unsigned long long>(cnt[CNT_FIX], ctx->ofix_cap);
            if ((st = alloc_fix(ctx, (unsigned int)std::min<unsigned long long>(INT32_MAX, need + need / 2 + 4096))))
                return st;
        }
        const bool mirror = ctx->mirror_pending;
        if ((st = pileup_launch(ctx, s))) return st;
        ctx->pileup_pending = false;
        if (mirror && (st = mirror_launch(ctx, nullptr))) return st;
        ctx->capacity_retries++;
        retried = true;
    }
    const unsigned int err = cnt[CNT_ERR];
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    ctx->pileup_ms = ms;
    if (ctx->pileup_graphed) {
        // no per-stage events inside the graph: only the whole chain is timed
        for (int k = 0; k < 5; k++) ctx->stage_ms[k] = 0;
    } else {
        const int marks[5] = {0, 4, 5, 6, 7};
        for (int k = 0; k < 4; k++) {
            float m = 0;
            cudaEventElapsedTime(&m, ctx->ev[marks[k]], ctx->ev[marks[k + 1]]);
            ctx->stage_ms[k] = m;
        }
        cudaEventElapsedTime(&ms, ctx->ev[7], ctx->ev[1]);
        ctx->stage_ms[4] = ms;
    }
    (void)retried;
    if (err) {
        char buf[160];
        snprintf(buf, sizeof buf, "pileup device error bits 0x%x", err);
        ctx->err = buf;
        if (err & kCapBits) return RV_ERR_CAPACITY;
        if (err & ERR_COLLISION) return RV_ERR_COLLISION;
        return RV_ERR_UNSUPPORTED;
    }
    if (ctx->n_reads > 0)
        ctx->keys_per_read = std::max(ctx->keys_per_read, (double)cnt[CNT_USED] / (double)ctx->n_reads);
    ctx->stage = 2;
    return RV_OK;
}

}  // namespace

rv_status rv_pileup(rv_ctx *ctx, void *stream) {
    if (!ctx) return RV_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    rv_status st = pileup_launch(ctx, s);
    if (st) return st;
    return pileup_finish(ctx, s);
}

rv_status rv_realign(rv_ctx *ctx, void *stream) {
    if (!ctx) return RV_ERR_ARG;
    if (ctx->stage < 2) { ctx->err = "rv_realign before rv_pileup"; return RV_ERR_STATE; }
    if (ctx->stage >= 3) { ctx->err = "rv_realign called twice on one batch"; return RV_ERR_STATE; }
    (void)stream;
    RV_CUDA(cudaSetDevice(ctx->device));
    rv_status st = ctx->params.local_realign ? host_realign_full(ctx) : host_realign_mnp(ctx);
    if (st) return st;
    ctx->stage = 3;
    return RV_OK;
}

// The score stage in two steps, so that the two samples of a pair queue
// their kernels together and share one wait (while another batch's tile
// kernel holds the SMs, a wait lasts until one of its chunks ends).
// score_a queues everything: counters, the insertion adjustments and their
// wide pass, the score kernel and its wide pass, and the counter words'
// copy to the context's pinned words.
static rv_status score_a(rv_ctx *ctx, cudaStream_t s, const DevParams &dp) {
    if (ctx->stage < 2) { ctx->err = "rv_score before rv_pileup"; return RV_ERR_STATE; }
    if (ctx->stage >= 4) { ctx->err = "this batch was already scored (submit it again)"; return RV_ERR_STATE; }
    RV_CUDA(cudaSetDevice(ctx->device));
    DevState st = ctx->state();
    RV_CUDA(cudaEventRecord(ctx->ev[2], s));
    RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_CAND, 0, 4, s));
    RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_WIDE_INS, 0, 4, s));
    RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_WIDE_SCORE, 0, 4, s));
    launch_ins_adjust(st, s);
    // positions with more insertion keys than the kernel's arrays: their
    // adjustments land before any position is scored
    queue_wide(ctx, 0, dp, s);
    RV_CUDA(cudaEventRecord(ctx->ev[8], s));
    launch_score(st, dp, s);
    queue_wide(ctx, 1, dp, s);
    RV_CUDA(cudaGetLastError());
    RV_CUDA(cudaEventRecord(ctx->ev[3], s));
    RV_CUDA(cudaMemcpyAsync(ctx->h_cnt, ctx->d_counters, kHdrWords * 4, cudaMemcpyDeviceToHost, s));
    ctx->kernels += 2;
    return RV_OK;
}

// score_c, after score_a's copy has landed: what overflowed (the candidate
// buffer, the wide scratch) is grown and scored again, then the error bits
// and the candidates to the host.
static rv_status score_c(rv_ctx *ctx, cudaStream_t s, const DevParams &dp) {
    unsigned int hdr[kHdrWords];
    std::memcpy(hdr, ctx->h_cnt, sizeof hdr);
    for (int attempt = 0; attempt < 3 && (hdr[CNT_ERR] & kScoreRetryBits); attempt++) {
        rv_status g;
        if ((hdr[CNT_ERR] & ERR_CAND_FULL) && (g = grow_cand(ctx, hdr[CNT_CAND]))) return g;
        if ((hdr[CNT_ERR] & (ERR_WIDE_INS_SCRATCH | ERR_WIDE_SCORE_SCRATCH)) && (g = grow_wide_scratch(ctx, s)))
            return g;
        DevState st = ctx->state();
        // the insertion pass that did nothing runs now (its offsets stand);
        // the score kernel only reads the maps, so it runs again whole
        if (hdr[CNT_ERR] & ERR_WIDE_INS_SCRATCH)
            launch_ins_adjust_wide(st, wide_off(ctx, 0), ctx->d_wide_scratch, wide_entries(ctx), s);
        RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_CAND, 0, 4, s));
        RV_CUDA(cudaMemsetAsync(ctx->d_counters + CNT_WIDE_SCORE, 0, 4, s));
        launch_clear_err_bits(st, ~kScoreRetryBits, s);
        launch_score(st, dp, s);
        queue_wide(ctx, 1, dp, s);
        RV_CUDA(cudaGetLastError());
        RV_CUDA(cudaEventRecord(ctx->ev[3], s));
        RV_CUDA(cudaMemcpyAsync(hdr, ctx->d_counters, sizeof hdr, cudaMemcpyDeviceToHost, s));
        RV_CUDA(cudaStreamSynchronize(s));
        ctx->kernels += 3;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
    ctx->score_ms = ms;
    cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[8]);
    ctx->stage_ms[5] = ms;
    cudaEventElapsedTime(&ms, ctx->ev[8], ctx->ev[3]);
    ctx->stage_ms[6] = ms;
    const unsigned int n = hdr[CNT_CAND];
    rv_status e = score_errors(ctx, hdr, n);
    if (e) return e;
    // (copies on the context's stream: a legacy-stream copy was measured to
    // wait for another batch's pileup queued on the other streams)
    ctx->h_cand.resize(n);
    if (n)
        RV_CUDA(cudaMemcpyAsync(ctx->h_cand.data(), ctx->d_cand, (size_t)n * sizeof(CandVar), cudaMemcpyDeviceToHost,
                                s));
    unsigned long long used = 0;
    RV_CUDA(cudaMemcpyAsync(&used, ctx->d_counters + 8, 8, cudaMemcpyDeviceToHost, s));
    RV_CUDA(cudaStreamSynchronize(s));
    used = std::min<unsigned long long>(used, ctx->arena_cap);
    ctx->h_arena.resize(used);
    if (used) RV_CUDA(cudaMemcpyAsync(ctx->h_arena.data(), ctx->d_arena, used, cudaMemcpyDeviceToHost, s));
    RV_CUDA(cudaStreamSynchronize(s));
    ctx->io_d2h += (int64_t)sizeof hdr + (int64_t)n * (int64_t)sizeof(CandVar) + 8 + (int64_t)used;
    ctx->stage = 4;
    return RV_OK;
}

static rv_status score_impl(rv_ctx *ctx, void *stream, const DevParams &dp) {
    if (!ctx) return RV_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    rv_status st;
    if ((st = score_a(ctx, s, dp))) return st;
    RV_CUDA(cudaStreamSynchronize(s));
    return score_c(ctx, s, dp);
}

rv_status rv_score(rv_ctx *ctx, void *stream) {
    if (!ctx) return RV_ERR_ARG;
    ctx->dp.dataset_min = 0;
    return score_impl(ctx, stream, ctx->dp);
}

rv_status rv_score_candidates(rv_ctx *ctx, int min_count) {
    if (!ctx || min_count < 1) return RV_ERR_ARG;
    if (ctx->params.somatic) { ctx->err = "rv_score_candidates scores one sample (somatic = 0)"; return RV_ERR_ARG; }
    ctx->dp.dataset_min = min_count;
    // every covered position may keep all its alleles
    const unsigned int want = (unsigned int)std::min<int64_t>(INT32_MAX, ctx->n_score * 6 + 1024);
    if (want > ctx->cand_cap) {
        if (ctx->d_cand) cudaFree(ctx->d_cand);
        ctx->d_cand = nullptr;
        RV_CUDA(cudaMalloc((void **)&ctx->d_cand, (size_t)want * sizeof(CandVar)));
        ctx->cand_cap = want;
    }
    rv_status s = score_impl(ctx, nullptr, ctx->dp);
    return s;
}

rv_status rv_candidates(rv_ctx *ctx, float *features, rv_candidate *cands, int64_t cap, int64_t *n) {
    if (!ctx || !n) return RV_ERR_ARG;
    if (ctx->stage < 4) { ctx->err = "rv_candidates before a scoring call"; return RV_ERR_STATE; }
    int64_t nv = 0;
    for (const CandVar &c : ctx->h_cand) nv += c.kind == 1;
    *n = nv;
    if (!features && !cands) return RV_OK;
    if (cap < nv) { ctx->err = "rv_candidates: buffers too small"; return RV_ERR_CAPACITY; }
    RV_CUDA(cudaSetDevice(ctx->device));
    const int64_t all = (int64_t)ctx->h_cand.size();
    std::vector<float> f((size_t)std::max<int64_t>(all, 1) * RV_FEATURES);
    if (features && all > 0) {
        float *df = nullptr;
        RV_CUDA(cudaMalloc((void **)&df, (size_t)all * RV_FEATURES * sizeof(float)));
        DevState st = ctx->state();
        launch_features(st, ctx->dp, ctx->d_cand, all, df, ctx->stream);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(f.data(), df, (size_t)all * RV_FEATURES * sizeof(float),
                                                  cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        cudaFree(df);
        if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return RV_ERR_CUDA; }
        ctx->kernels += 1;
    }
    std::vector<uint8_t> emitted((size_t)std::max<int64_t>(all, 1), 0);
    if (cands) {
        std::string keep = ctx->text;
        rv_status s = host_format_records(ctx, "", "", emitted.data());
        ctx->text.swap(keep);
        if (s) return s;
    }
    int64_t j = 0;
    for (int64_t i = 0; i < all; i++) {
        const CandVar &c = ctx->h_cand[i];
        if (c.kind != 1) continue;
        if (features) memcpy(features + j * RV_FEATURES, f.data() + i * RV_FEATURES, RV_FEATURES * sizeof(float));
        if (cands) {
            rv_candidate &o = cands[j];
            memset(&o, 0, sizeof o);
            o.region = c.region;
            o.position = c.pos;
            o.hard_pass = emitted[i];
            if (c.key_len < 0) {
                o.key_len = 1;
                o.key[0] = "ACGT"[c.key_off & 3];
            } else {
                o.key_len = c.key_len;
                memcpy(o.key, ctx->h_arena.data() + c.key_off, std::min<int>(c.key_len, (int)sizeof o.key - 1));
            }
        }
        j++;
    }
    return RV_OK;
}

rv_status rv_format_records(rv_ctx *ctx, const char *sample, const char *gene, const char **text,
                            size_t *text_len, int64_t *n_records) {
    if (!ctx) return RV_ERR_ARG;
    if (ctx->stage < 4) { ctx->err = "rv_format_records before rv_score"; return RV_ERR_STATE; }
    rv_status st = host_format_records(ctx, sample ? sample : "", gene ? gene : ctx->chr.c_str(), nullptr);
    if (st) return st;
    if (text) *text = ctx->text.c_str();
    if (text_len) *text_len = ctx->text.size();
    if (n_records) *n_records = ctx->n_records;
    return RV_OK;
}

rv_status rv_fetch_records(rv_ctx *ctx, rv_site_record *out, size_t cap, size_t *n) {
    if (!ctx || !n) return RV_ERR_ARG;
    *n = ctx->h_records.size();
    if (out) memcpy(out, ctx->h_records.data(), std::min(cap, ctx->h_records.size()) * sizeof(rv_site_record));
    return RV_OK;
}

rv_status rv_call_regions(rv_ctx *ctx, const rv_read_batch *reads, const rv_region *regions, int n_regions,
                          const char *sample, const char *gene, const char **text, size_t *text_len,
                          int64_t *n_records) {
    rv_status s;
    if ((s = rv_submit_batch(ctx, reads, regions, n_regions, nullptr))) return s;
    if ((s = rv_pileup(ctx, nullptr))) return s;
    if ((s = rv_realign(ctx, nullptr))) return s;
    if ((s = rv_score(ctx, nullptr))) return s;
    return rv_format_records(ctx, sample, gene, text, text_len, n_records);
}

rv_status rv_score_pair(rv_ctx *tumor, rv_ctx *normal) {
    if (!tumor || !normal || tumor == normal) return RV_ERR_ARG;
    if (!tumor->params.somatic || !normal->params.somatic) {
        tumor->err = "rv_score_pair needs two contexts created with somatic = 1";
        return RV_ERR_ARG;
    }
    if (!same_regions(tumor, normal) || tumor->device != normal->device) {
        tumor->err = "rv_score_pair: the two samples must share the contig, the region list and the device";
        return RV_ERR_ARG;
    }
    rv_status s;
    PhaseTimer tm("score_pair");
    // each step is queued for both samples before either is waited for
    rv_ctx *both[2] = {tumor, normal};
    auto each = [&](const std::function<rv_status(rv_ctx *)> &f) -> rv_status {
        for (rv_ctx *c : both) {
            rv_status r = f(c);
            if (r) {
                if (c != tumor) tumor->err = c->err;
                return r;
            }
        }
        return (rv_status)RV_OK;
    };
    auto wait = [&](rv_ctx *c) -> rv_status {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { c->err = std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e); return RV_ERR_CUDA; }
        return (rv_status)RV_OK;
    };
    tumor->dp.dataset_min = normal->dp.dataset_min = 0;
    if ((s = each([](rv_ctx *c) { return score_a(c, c->stream, c->dp); }))) return s;
    tm.lap("queue");
    if ((s = wait(tumor))) return s;
    tm.lap("wait_tumor");
    if ((s = wait(normal))) { tumor->err = normal->err; return s; }
    tm.lap("wait_normal");
    if ((s = each([](rv_ctx *c) { return score_c(c, c->stream, c->dp); }))) return s;
    tm.lap("collect");
    // every position where one sample has a candidate is needed in both
    std::vector<int2> pt = positions_of(tumor), pn = positions_of(normal);
    tm.lap("positions");
    const std::vector<int2> lt = missing(pn, pt), ln = missing(pt, pn);
    if ((s = score_list_a(tumor, lt))) return s;
    if ((s = score_list_a(normal, ln))) { tumor->err = normal->err; return s; }
    if ((s = score_list_b(tumor, lt))) return s;
    if ((s = score_list_b(normal, ln))) { tumor->err = normal->err; return s; }
    tm.lap("score_list");
    return RV_OK;
}

namespace {

// Queues both samples' pileups (and, with -k 1, their realigner mirrors)
// without waiting.  The tumor's mirror kernels go before the normal's
// pileup, so the tumor's realigner can start as soon as they end; the
// mirror's copies then overlap the normal's kernels.  On an error nothing
// stays in flight.
rv_status pair_launch(rv_ctx *tumor, rv_ctx *normal, cudaEvent_t after = nullptr) {
    rv_status s;
    // `after`: the pileups queue behind that event (another pair's pileup),
    // so the two pairs' tile kernels do not share the SMs
    if (after) {
        cudaError_t e = cudaStreamWaitEvent(tumor->stream, after, 0);
        if (e != cudaSuccess) {
            tumor->err = std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e);
            return RV_ERR_CUDA;
        }
    }
    if ((s = pileup_launch(tumor, tumor->stream))) return s;
    if (tumor->params.local_realign) {
        if ((s = mirror_launch(tumor, tumor->ev[11]))) {
            pileup_finish(tumor, tumor->stream);
            return s;
        }
        cudaError_t e = cudaStreamWaitEvent(normal->stream, tumor->ev[11], 0);
        if (e != cudaSuccess) {
            tumor->err = std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e);
            pileup_finish(tumor, tumor->stream);
            return RV_ERR_CUDA;
        }
    }
    if ((s = pileup_launch(normal, normal->stream))) {
        tumor->err = normal->err;
        pileup_finish(tumor, tumor->stream);
        return s;
    }
    // the normal's mirror queues behind its pileup and runs while the host
    // realigns the tumor
    if (normal->params.local_realign && (s = mirror_launch(normal, nullptr))) {
        tumor->err = normal->err;
        pileup_finish(tumor, tumor->stream);
        pileup_finish(normal, normal->stream);
        return s;
    }
    return RV_OK;
}

// Waits for the tumor's pileup and realigns it on the host (while the
// normal's kernels run), then the normal's.  `between` runs after the
// tumor's pileup finished and before its realigner (the stream uses it to
// queue the next batch's pileups behind this one's, and the upload of the
// tumor's batch after next); `after_normal` after the normal's pileup
// finished (the upload of the normal's batch after next).
rv_status pair_finish(rv_ctx *tumor, rv_ctx *normal, const std::function<rv_status()> &between,
                      const std::function<rv_status()> &after_normal = nullptr) {
    rv_status st = pileup_finish(tumor, tumor->stream);
    if (st) {
        pileup_finish(normal, normal->stream);
        return st;
    }
    if ((st = between())) {
        pileup_finish(normal, normal->stream);
        return st;
    }
    if ((st = rv_realign(tumor, nullptr))) {
        pileup_finish(normal, normal->stream);
        return st;
    }
    if ((st = pileup_finish(normal, normal->stream))) { tumor->err = normal->err; return st; }
    if (after_normal && (st = after_normal())) return st;
    if ((st = rv_realign(normal, nullptr))) { tumor->err = normal->err; return st; }
    return RV_OK;
}

}  // namespace

rv_status rv_pileup_realign_pair(rv_ctx *tumor, rv_ctx *normal) {
    if (!tumor || !normal || tumor == normal) return RV_ERR_ARG;
    // both samples' kernels are queued first (one stream each); the tumor's
    // host realigner then runs while the normal's pileup is on the device
    rv_status s = pair_launch(tumor, normal);
    if (s) return s;
    return pair_finish(tumor, normal, [] { return (rv_status)RV_OK; });
}

rv_status rv_call_somatic_stream(rv_ctx *tumor0, rv_ctx *normal0, rv_ctx *tumor1, rv_ctx *normal1,
                                 const rv_somatic_job *jobs, int64_t n_jobs, rv_somatic_sink sink, void *user) {
    rv_ctx *T[2] = {tumor0, tumor1}, *N[2] = {normal0, normal1};
    if (!tumor0 || !normal0 || !tumor1 || !normal1 || (!jobs && n_jobs > 0) || n_jobs < 0) return RV_ERR_ARG;
    rv_ctx *all[4] = {tumor0, normal0, tumor1, normal1};
    for (int a = 0; a < 4; a++)
        for (int b = a + 1; b < 4; b++)
            if (all[a] == all[b]) { tumor0->err = "rv_call_somatic_stream needs four distinct contexts"; return RV_ERR_ARG; }
    struct Fmt {
        std::thread th;
        rv_status st = RV_OK;
        bool active = false;
    } fmt[2];
    auto join_all = [&] {
        for (auto &f : fmt)
            if (f.active) { f.th.join(); f.active = false; }
    };
    auto finish = [&](int pi, int64_t k) -> rv_status {
        if (!fmt[pi].active) return RV_OK;
        fmt[pi].th.join();
        fmt[pi].active = false;
        if (fmt[pi].st) return fmt[pi].st;
        if (sink) sink(user, k, T[pi]->text.c_str(), T[pi]->text.size(), T[pi]->n_records);
        return RV_OK;
    };
    // a job without batches reuses the batch already on its pair's devices
    auto resident = [&](int pi) -> rv_status {
        if (T[pi]->stage < 1 || N[pi]->stage < 1) {
            T[pi]->err = "rv_call_somatic_stream: a job without batches needs a batch submitted on its pair";
            return RV_ERR_STATE;
        }
        return RV_OK;
    };
    auto submit = [&](int pi, int64_t k) -> rv_status {
        const rv_somatic_job &j = jobs[k];
        if (!j.tumor && !j.normal) return resident(pi);
        // both samples prepared before either's bulk upload
        return (j.tumor && j.normal) ? submit_pair(T[pi], N[pi], j.tumor, j.normal, j.regions, j.n_regions)
                                     : (rv_status)RV_ERR_ARG;
    };
    rv_status s = RV_OK;
    int bad = 0;  // the pair whose context holds the error message
    // jobs 0 and 1 are uploaded here; job k + 2 by the host thread that
    // formats job k, on the same pair, right after it.  Job k + 1's pileups
    // are queued as soon as job k's tumor pileup has finished (and job
    // k - 1's formatting, which uploads job k + 1, has joined), so the device
    // piles up the next batch while the host realigns this one.
    if (n_jobs > 0) s = submit(0, 0);
    if (!s && n_jobs > 1) {
        bad = 1;
        s = submit(1, 1);
    }
    if (!s && n_jobs > 0) {
        bad = 0;
        s = pair_launch(T[0], N[0]);
    }
    bool next_in_flight = false;  // job k + 1's pileups are queued
    PhaseTimer tm("stream");
    for (int64_t k = 0; k < n_jobs && !s; k++) {
        const int pi = (int)(k & 1);
        bad = pi;
        next_in_flight = false;
        // device stages of job k on pair pi: its pileups were queued earlier;
        // once the tumor's has finished, the host thread that formatted job
        // k - 1 (and uploaded job k + 1) is joined and job k + 1's pileups
        // are queued on the other pair
        auto between = [&]() -> rv_status {
            tm.lap("pileup_wait");
            rv_status f = finish(pi ^ 1, k - 1);
            if (f) {
                bad = pi ^ 1;
                return f;
            }
            tm.lap("wait_format");
            if (k + 1 < n_jobs) {
                // behind this job's normal pileup (its end event, ev[1])
                rv_status l = pair_launch(T[pi ^ 1], N[pi ^ 1], N[pi]->ev[1]);
                if (l) {
                    bad = pi ^ 1;
                    return l;
                }
                next_in_flight = true;
            }
            // job k + 2 runs on this pair: its tumor reads go up now (the
            // tumor's pileup chain is done with the read buffers)
            if (k + 2 < n_jobs && jobs[k + 2].tumor && jobs[k + 2].normal) {
                rv_status u = early_upload(T[pi], jobs[k + 2].tumor);
                if (u) return u;
            }
            return (rv_status)RV_OK;
        };
        auto after_normal = [&]() -> rv_status {
            if (k + 2 < n_jobs && jobs[k + 2].tumor && jobs[k + 2].normal) {
                rv_status u = early_upload(N[pi], jobs[k + 2].normal);
                if (u) {
                    T[pi]->err = N[pi]->err;
                    return u;
                }
            }
            return (rv_status)RV_OK;
        };
        if ((s = pair_finish(T[pi], N[pi], between, after_normal))) break;
        tm.lap("realign");
        if ((s = rv_score_pair(T[pi], N[pi]))) break;
        tm.lap("score");
        fmt[pi].active = true;
        const rv_somatic_job *j = &jobs[k];
        rv_ctx *t = T[pi], *n = N[pi];
        rv_status *out = &fmt[pi].st;
        const rv_somatic_job *next = k + 2 < n_jobs ? &jobs[k + 2] : nullptr;
        fmt[pi].th = std::thread([t, n, j, next, out] {
            rv_status st = rv_format_somatic(t, n, j->sample, j->gene, nullptr, nullptr, nullptr);
            // the records stay in t->text until this pair is formatted again
            if (!st && next && (next->tumor || next->normal)) {
                st = (next->tumor && next->normal)
                         ? submit_pair(t, n, next->tumor, next->normal, next->regions, next->n_regions)
                         : (rv_status)RV_ERR_ARG;
            }
            *out = st;
        });
    }
    // a failure leaves no pileup of the next job in flight
    if (s && next_in_flight) {
        const int pn = bad ^ 1;
        for (rv_ctx *c : {T[pn], N[pn]})
            if (c->pileup_pending) pileup_finish(c, c->stream);
    }
    if (!s && n_jobs > 0) {
        bad = (int)((n_jobs - 1) & 1);
        s = finish(bad, n_jobs - 1);
    }
    join_all();
    // an upload queued for a job that did not run stays unused
    for (rv_ctx *c : all) c->early_batch = nullptr;
    if (s && bad != 0) T[0]->err = T[bad]->err;
    return s;
}

rv_status rv_format_somatic(rv_ctx *tumor, rv_ctx *normal, const char *sample, const char *gene, const char **text,
                            size_t *text_len, int64_t *n_records) {
    if (!tumor || !normal) return RV_ERR_ARG;
    if (tumor->stage < 4 || normal->stage < 4) {
        tumor->err = "rv_format_somatic before rv_score_pair";
        return RV_ERR_STATE;
    }
    rv_status st = host_format_somatic(tumor, normal, sample ? sample : "", gene ? gene : tumor->chr.c_str());
    if (st) return st;
    if (text) *text = tumor->text.c_str();
    if (text_len) *text_len = tumor->text.size();
    if (n_records) *n_records = tumor->n_records;
    return RV_OK;
}

rv_status rv_call_somatic(rv_ctx *tumor, rv_ctx *normal, const rv_read_batch *tumor_reads,
                          const rv_read_batch *normal_reads, const rv_region *regions, int n_regions,
                          const char *sample, const char *gene, const char **text, size_t *text_len,
                          int64_t *n_records) {
    if (!tumor || !normal) return RV_ERR_ARG;
    rv_status s;
    if (!tumor_reads || !normal_reads) return RV_ERR_ARG;
    if ((s = submit_pair(tumor, normal, tumor_reads, normal_reads, regions, n_regions))) return s;
    if ((s = rv_pileup_realign_pair(tumor, normal))) return s;
    if ((s = rv_score_pair(tumor, normal))) return s;
    return rv_format_somatic(tumor, normal, sample, gene, text, text_len, n_records);
}

rv_status rv_export_maps(rv_ctx *ctx, int region, const char *stages, const char **text, size_t *text_len) {
    if (!ctx || region < 0 || region >= (int)ctx->regions.size()) return RV_ERR_ARG;
    if (ctx->stage < 2) { ctx->err = "rv_export_maps before rv_pileup"; return RV_ERR_STATE; }
    RV_CUDA(cudaSetDevice(ctx->device));
    rv_status st = host_export_maps(ctx, region, stages ? stages : "P");
    if (st) return st;
    if (text) *text = ctx->dump.c_str();
    if (text_len) *text_len = ctx->dump.size();
    return RV_OK;
}

rv_status rv_last_timings(const rv_ctx *ctx, double *pileup_ms, double *score_ms, double *total_ms,
                          int64_t *kernels) {
    if (!ctx) return RV_ERR_ARG;
    if (pileup_ms) *pileup_ms = ctx->pileup_ms;
    if (score_ms) *score_ms = ctx->score_ms;
    if (total_ms) *total_ms = ctx->pileup_ms + ctx->score_ms;
    if (kernels) *kernels = ctx->kernels;
    return RV_OK;
}

rv_status rv_io_bytes(const rv_ctx *ctx, int64_t *h2d, int64_t *d2h) {
    if (!ctx) return RV_ERR_ARG;
    if (h2d) *h2d = ctx->io_h2d;
    if (d2h) *d2h = ctx->io_d2h;
    return RV_OK;
}

rv_status rv_stage_times(const rv_ctx *ctx, double *ms, int n) {
    if (!ctx || !ms || n < 0) return RV_ERR_ARG;
    for (int i = 0; i < n && i < 8; i++) ms[i] = ctx->stage_ms[i];
    if (n > 7) ms[7] = ctx->variant;
    return RV_OK;
}

rv_status rv_set_pileup_graph(rv_ctx *ctx, int enable) {
    if (!ctx) return RV_ERR_ARG;
    if (ctx->pileup_pending) { ctx->err = "rv_set_pileup_graph while a pileup is in flight"; return RV_ERR_STATE; }
    ctx->use_graph = enable != 0;
    return RV_OK;
}

rv_status rv_set_capacities(rv_ctx *ctx, size_t hash_slots, size_t arena_bytes, size_t deferred, size_t order_fix) {
    if (!ctx) return RV_ERR_ARG;
    if (ctx->pileup_pending) { ctx->err = "rv_set_capacities while a pileup is in flight"; return RV_ERR_STATE; }
    if (deferred > (size_t)INT32_MAX || order_fix > (size_t)INT32_MAX || hash_slots > (1ULL << 32)) {
        ctx->err = "rv_set_capacities: capacity out of range";
        return RV_ERR_ARG;
    }
    ctx->force_hash = hash_slots;
    ctx->force_arena = arena_bytes;
    ctx->force_deferred = (unsigned int)deferred;
    ctx->force_fix = (unsigned int)order_fix;
    return RV_OK;
}

rv_status rv_capacity_stats(const rv_ctx *ctx, int64_t *retries, int64_t *hash_slots, int64_t *arena_bytes) {
    if (!ctx) return RV_ERR_ARG;
    if (retries) *retries = ctx->capacity_retries;
    if (hash_slots) *hash_slots = (int64_t)ctx->hash_cap;
    if (arena_bytes) *arena_bytes = (int64_t)ctx->arena_cap;
    return RV_OK;
}

rv_status rv_pileup_graph_stats(const rv_ctx *ctx, int64_t *launches, int64_t *instantiations) {
    if (!ctx) return RV_ERR_ARG;
    if (launches) *launches = ctx->graph_launches;
    if (instantiations) *instantiations = ctx->graph_instantiations;
    return RV_OK;
}

rv_status rv_fisher_batch(rv_ctx *ctx, const int32_t *tables, int64_t n, double *two_sided, double *ratio) {
    if (!ctx || n < 0 || (n > 0 && (!tables || !two_sided || !ratio))) return RV_ERR_ARG;
    if (n == 0) return RV_OK;
    RV_CUDA(cudaSetDevice(ctx->device));
    int32_t *dt = nullptr;
    double *dp = nullptr;
    RV_CUDA(cudaMalloc((void **)&dt, (size_t)n * 16));
    cudaError_t e = cudaMalloc((void **)&dp, (size_t)n * 16);
    if (e != cudaSuccess) { cudaFree(dt); ctx->err = cudaGetErrorString(e); return RV_ERR_CUDA; }
    e = cudaMemcpy(dt, tables, (size_t)n * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_fisher(dt, n, dp, dp + n, ctx->stream, ctx->d_logfact);
        e = cudaStreamSynchronize(ctx->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpy(two_sided, dp, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ratio, dp + n, (size_t)n * 8, cudaMemcpyDeviceToHost);
    cudaFree(dt);
    cudaFree(dp);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return RV_ERR_CUDA; }
    return RV_OK;
}

}  // extern "C"
