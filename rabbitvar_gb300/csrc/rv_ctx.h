// Host-side context of librvgpu (not part of the public ABI).
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "rv_internal.h"

namespace rv {

// kernel launchers (rv_pileup.cu, rv_score.cu)
void launch_init_slots(Slot *slots, unsigned long long n, cudaStream_t s);
void launch_clear_used(Slot *slots, const uint32_t *used, const unsigned int *n_used, unsigned long long cap,
                       cudaStream_t s);
void launch_region_reset(const DevState &st, cudaStream_t s);
cudaError_t launch_pileup(const DevState &st, const DevParams &P, int resident_blocks, cudaStream_t s, int variant,
                          int priority);
int tile_quota(int64_t n_tiles, int resident_blocks);
void launch_read_prep(const ReadPrepIn &in, const ReadPrepOut &out, int sm_count, cudaStream_t s);
void launch_region_prep(const RegionPrepArgs &a, int n_regions, cudaStream_t s);
void launch_region_fill(const RegionFillArgs &a, int n_regions, cudaStream_t s);
int pileup_variants();
void launch_serial(const DevState &st, const DevParams &P, cudaStream_t s);
void launch_edge_detect(const DevState &st, const DevParams &P, cudaStream_t s);
void launch_resolve(const DevState &st, const DevParams &P, cudaStream_t s);
void launch_fix_order(const DevState &st, const DevParams &P, cudaStream_t s);
int pileup_blocks_per_sm(int variant);
size_t pileup_smem_bytes();
void launch_link(const DevState &st, cudaStream_t s);
void launch_collisions(const DevState &st, cudaStream_t s);
void launch_ins_adjust(const DevState &st, cudaStream_t s);
void launch_score(const DevState &st, const DevParams &P, cudaStream_t s);
void launch_clear_err_bits(const DevState &st, unsigned int keep, cudaStream_t s);
size_t wide_entry_bytes();
void launch_wide_offsets(const DevState &st, int list, int64_t *off, cudaStream_t s);
void launch_ins_adjust_wide(const DevState &st, const int64_t *off, void *scratch, int64_t entries, cudaStream_t s);
void launch_score_wide(const DevState &st, const DevParams &P, const int64_t *off, void *scratch, int64_t entries,
                       cudaStream_t s);
void launch_fisher(const int32_t *tab, int64_t n, double *p2, double *ratio, cudaStream_t s,
                   const double *lf = nullptr);
void launch_fill_logfact(double *lf, cudaStream_t s);
void launch_features(const DevState &st, const DevParams &P, const CandVar *cand, int64_t n, float *out,
                     cudaStream_t s);
void launch_score_list(const DevState &st, const DevParams &P, const int2 *list, int n, cudaStream_t s);
void launch_compact_slots(const DevState &st, uint32_t *out, unsigned int *n_out, cudaStream_t s);
void launch_gather_slots(const Slot *slots, const uint32_t *idx, int64_t n, Slot *out, cudaStream_t s);

// one cell (position) as seen by the host realigner
struct CellView {
    uint32_t fwd[4], rev[4], hi[4], tp[4], q[4], mq[4];
    int32_t nm[4];
    uint32_t first[4];
    uint32_t cov;
    uint32_t kflags;
};
void launch_select_mnv(const DevState &st, uint32_t *out, unsigned int *n_out, cudaStream_t s);
void launch_gather_lists(const DevState &st, const int64_t *cells, int64_t n, uint32_t *out, unsigned int *n_out,
                         unsigned int cap, cudaStream_t s);
void launch_gather_cells(const DevState &st, const int64_t *cells, int64_t n, CellView *out, cudaStream_t s);

// patch written back by the host realigner
struct Patch {
    // 0 overwrite a slot's statistics (adjustMNP: integer sums)
    // 1 erase a slot (flags |= SF_ERASED | flags_or)
    // 2 erase a single-base cell key
    // 3 add coverage
    // 4 set a slot's realigned statistics (SF_OVR)
    // 5 find or create the slot (region, pos, kind, key bytes) and set them
    // 6 remove a position's cell keys from the map
    int32_t type;
    int32_t base;
    int64_t target;     // slot index or cell index
    int32_t fwd, rev, hi, lo, extracnt, flags_or;
    long long tp_sum, mq_sum, nm_sum;
    double q_sum;
    int32_t cov_add, cnt;
    double tp, mq, nm;                  // types 4 and 5
    int32_t region, pos, kind, klen;    // type 5
    int64_t key_off;                    // type 5: key bytes in the patch key buffer
};
void launch_apply_patches(const DevState &st, const Patch *p, int64_t n, const uint8_t *keys, cudaStream_t s);
void launch_find35(const int32_t *pairs, int64_t n, const char *strs, int32_t *res, cudaStream_t s);
// flattened per-cell key lists (-k 1 realigner mirror): 5 launches, then 1
void launch_list_offsets(const DevState &st, uint32_t *off, uint32_t *bsum, cudaStream_t s);
void launch_list_fill(const DevState &st, const uint32_t *off, Slot *out, uint32_t *out_idx, cudaStream_t s);
void launch_clip_consensus(const DevState &st, const uint32_t *off, const Slot *list, uint32_t *meta, uint8_t *cons,
                           cudaStream_t s);

// Host phase timer: with RV_TRACE set in the environment, each lap prints
// "<scope> <phase> <ms>" to stderr (diagnostics only; no effect on results).
struct PhaseTimer {
    const char *scope;
    bool on;
    std::chrono::steady_clock::time_point t;
    explicit PhaseTimer(const char *s) : scope(s), on(getenv("RV_TRACE") != nullptr), t(std::chrono::steady_clock::now()) {}
    void lap(const char *phase) {
        if (!on) return;
        auto n = std::chrono::steady_clock::now();
        fprintf(stderr, "trace %s %s %.3f\n", scope, phase, std::chrono::duration<double, std::milli>(n - t).count());
        t = n;
    }
};

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
};

}  // namespace rv

struct rv_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    rv_params params;
    rv::DevParams dp;
    std::string err;
    size_t budget = 0;
    int sm_count = 0;

    // reference contig
    std::string chr;
    std::string ref_host;   // uppercase
    char *d_ref = nullptr;
    int32_t ref_len = 0;

    // batch (device copies)
    int64_t n_reads = 0, n_cigar_words = 0, n_bases = 0;
    size_t cap_reads = 0, cap_cigar = 0, cap_bases = 0;
    int32_t *d_pos = nullptr, *d_mpos = nullptr, *d_nm = nullptr, *d_lq = nullptr;
    uint16_t *d_flag = nullptr, *d_ncig = nullptr;
    uint8_t *d_mapq = nullptr;
    uint32_t *d_cigoff = nullptr, *d_cigar = nullptr;
    uint64_t *d_boff = nullptr;
    uint8_t *d_seq = nullptr, *d_qual = nullptr;
    uint8_t *d_skip = nullptr;  // -t duplicate flags
    size_t cap_skip = 0;
    bool use_skip = false;
    // -k 1: the submitted batch's host arrays, read again by the realigner
    // (noPassingReads); the caller keeps them until rv_realign returns
    const int32_t *hb_pos = nullptr;
    const uint16_t *hb_flag = nullptr, *hb_ncig = nullptr;
    const uint32_t *hb_cigoff = nullptr, *hb_cigar = nullptr;
    int64_t hb_n = 0;

    // regions / tiles
    std::vector<rv::Region> regions;
    int64_t n_tiles = 0;
    size_t tile_bound = 0;    // tiles the device list holds (the preparation's bound)
    // pinned host staging of the region records, score bases and list
    // starts, so their copies queue without waiting behind other uploads
    char *h_meta = nullptr;
    size_t cap_meta = 0;
    size_t n_tile_reads = 0;
    // batch preparation on the device: per read its span and walk-cost
    // class; per region its list start and tile segments
    int32_t *d_span_lo = nullptr, *d_span_hi = nullptr;
    uint8_t *d_cost = nullptr;
    size_t cap_prep = 0;
    int64_t *d_list_begin = nullptr;
    rv::RegionTiles *d_rtiles = nullptr;
    // a stream of batches uploads the next batch's reads on the copy stream
    // as soon as the last pileup chain no longer reads them (early_upload)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_up = nullptr;                 // that upload's end
    const rv_read_batch *early_batch = nullptr;  // the batch it carries
    bool batch_early = false;                    // the submitted batch came that way
    int *d_prep = nullptr;                // the preparation's result words (PREP_*)
    unsigned int *h_prep = nullptr;       // their pinned host copy
    bool prep_pending = false;            // results queued, not yet read (read before the pileup)
    int max_span = 1;                     // the batch's longest reference span (host scan)
    std::vector<int64_t> score_base;
    rv::Region *d_regions = nullptr;
    rv::Tile *d_tiles = nullptr;
    uint32_t *d_tile_reads = nullptr;
    size_t cap_tile_reads = 0;
    int64_t *d_score_base = nullptr;
    size_t cap_regions = 0, cap_tiles = 0;
    int64_t n_score = 0;

    // cells
    int64_t n_cells = 0;
    size_t cap_cells = 0;
    void *d_cellmem = nullptr;
    rv::Cells cells{};
    uint32_t *d_head = nullptr;

    // hash
    unsigned long long hash_cap = 0;
    rv::Slot *d_slots = nullptr;
    uint32_t *d_used = nullptr;       // used-slot list (hash_cap entries)
    bool slots_fresh = true;          // the table needs a whole-table reset (just allocated)
    double keys_per_read = 0;         // largest keys / reads seen (sizes the next table)
    // capacities forced by rv_set_capacities for the next batch (0 = automatic)
    unsigned long long force_hash = 0, force_arena = 0;
    unsigned int force_deferred = 0, force_fix = 0;
    int64_t capacity_retries = 0;     // pileups run again after a table grew
    uint8_t *d_arena = nullptr;
    unsigned long long arena_cap = 0;

    // deferred, candidates
    rv::Deferred *d_deferred = nullptr;
    unsigned int deferred_cap = 0;
    rv::CandVar *d_cand = nullptr;
    unsigned int cand_cap = 0;
    // map entries whose pstd/qstd are replayed in read order
    rv::OrderFix *d_ofix = nullptr;
    unsigned int ofix_cap = 0;
    // positions with more alleles than the scoring kernels' per-thread arrays:
    // two lists (insertion adjustment, scoring) of wide_cap entries, their
    // scratch offsets and the scratch itself (grown on demand)
    rv::WidePos *d_wide = nullptr;
    unsigned int wide_cap = 0;
    int64_t *d_wide_off = nullptr;
    size_t cap_wide_off = 0;
    void *d_wide_scratch = nullptr;
    size_t cap_wide_scratch = 0;
    int32_t max_lq = 0;   // longest read of the batch

    // small counters (64 words): n_deferred, n_used, err, n_cand, aux, n_ofix, n_wide_ins,
    // arena_used (64-bit, words 8-9), n_wide_score, tile counter (word 32)
    unsigned int *d_counters = nullptr;
    unsigned int *h_cnt = nullptr;  // pinned host copy of the counter words (asynchronous reads)

    // scratch for the realigner boundary (grown on demand, owned by the context)
    uint32_t *d_tmp_idx = nullptr;
    size_t cap_tmp_idx = 0;
    rv::Slot *d_tmp_slots = nullptr;
    size_t cap_tmp_slots = 0;
    int64_t *d_tmp_cells = nullptr;
    size_t cap_tmp_cells = 0;
    void *d_tmp_views = nullptr;
    size_t cap_tmp_views = 0;
    unsigned int *d_tmp_n = nullptr;
    // -k 1 realigner mirror: flattened key lists on the device, pinned host copies
    uint32_t *d_list_off = nullptr, *d_list_bsum = nullptr, *d_list_idx = nullptr;
    size_t cap_list_off = 0, cap_list_bsum = 0, cap_list_idx = 0;
    rv::Slot *d_list_slots = nullptr;
    size_t cap_list_slots = 0;
    uint32_t *d_cons_meta = nullptr;  // soft-clip consensus per listed aggregate
    size_t cap_cons_meta = 0;
    uint8_t *d_cons = nullptr;
    size_t cap_cons = 0;
    void *h_mirror = nullptr;  // pinned: cells, list offsets
    size_t cap_mirror = 0;
    void *h_mirror_slots = nullptr;  // pinned: listed keys, slot indices
    size_t cap_mirror_slots = 0;
    bool mirror_pending = false;     // mirror_launch queued, not yet consumed
    void *d_f35 = nullptr;           // realigner: clip pairs, their strings and find35 results
    size_t cap_f35 = 0;
    rv::Patch *d_patches = nullptr;
    size_t cap_patches = 0;
    uint8_t *d_patch_keys = nullptr;
    size_t cap_patch_keys = 0;
    // somatic mode: positions to score without screens; Fisher tables and results
    double *d_logfact = nullptr;  // log(k!) table for the Fisher tests
    int2 *d_list = nullptr;
    size_t cap_list = 0;
    int32_t *d_ftab = nullptr;
    size_t cap_ftab = 0;  // tables
    void *h_fstage = nullptr;  // pinned staging of the Fisher tables and p-values
    size_t cap_fstage = 0;

    // host mirrors
    std::vector<rv::CandVar> h_cand;
    std::vector<uint8_t> h_arena;
    std::vector<rv_site_record> h_records;
    std::string text;
    std::string dump;
    int64_t n_records = 0;

    // stage
    int stage = 0;  // 0 none, 1 submitted, 2 piled up, 3 realigned, 4 scored
    cudaEvent_t ev[12] = {};
    cudaEvent_t ev_block = nullptr;  // blocking-sync event (waits off the critical path)
    double pileup_ms = 0, score_ms = 0, total_ms = 0;
    double stage_ms[8] = {};
    // pileup kernel autotuning: variant in use, per-variant best time seen
    int variant = -1;
    double variant_ms[8] = {};
    int variant_runs = 0;
    int low_priority = 0;    // the device's lowest stream priority (the tile kernel's)
    bool pileup_pin = false;       // RV_PILEUP_VARIANT pinned the variant of the pileup in flight
    bool pileup_pending = false;   // pileup queued, not yet finished
    // pileup chain as a CUDA graph (rv_set_pileup_graph): each batch's chain
    // is captured and applied to one executable graph with cudaGraphExecUpdate
    // (instantiated again only when the update is refused)
    bool use_graph = false;
    bool pileup_graphed = false;   // the pileup in flight was launched as a graph
    cudaGraphExec_t pileup_exec = nullptr;
    int64_t graph_launches = 0, graph_instantiations = 0;
    int64_t kernels = 0;
    // bytes moved host<->device since the last rv_submit_batch
    int64_t io_h2d = 0, io_d2h = 0;

    rv::DevState state() const;
};

namespace rv {
// two-sided Fisher p-values of n (a, b, c, d) tables on the context's device
rv_status device_fisher(rv_ctx *ctx, const int32_t *tables, int64_t n, double *p2);
rv_status host_format_somatic(rv_ctx *tumor, rv_ctx *normal, const char *sample, const char *gene);
// -k 1 realigner: queue the mirror's device work (record `after_kernels` once its kernels are queued)
rv_status mirror_launch(rv_ctx *ctx, cudaEvent_t after_kernels);
}  // namespace rv
