// Internal declarations shared by the device kernels and the host side of
// librvgpu.  Not part of the public C ABI (include/rvgpu.h).
#pragma once
#include <cstddef>
#include <cstdint>

#include "rvgpu.h"

namespace rv {

// Hard limits of this build.
constexpr int kMaxKey = 640;        // longest allele key a walk may build
constexpr int kTileW = 640;         // positions per shared-memory tile window
constexpr int kPileupThreads = 256; // threads per pileup block (one read per thread at a time)
constexpr int kTileReads = 256;     // reads per tile at most (bounds the packed shared-memory counters)

// Allele-key kinds stored in the device hash table (the maps of
// include/scopedata/VariationData.h:14-56).
enum KeyKind : uint16_t {
    KIND_NONINS = 0,   // nonInsertionVariants, string keys (MNV, deletion, complex, non-ACGT bases)
    KIND_INS = 1,      // insertionVariants
    KIND_SC5 = 2,      // softClips5End aggregate Variation
    KIND_SC3 = 3,      // softClips3End aggregate Variation
    KIND_SC5_SEQ = 4,  // softClips5End seq[idx][ch] (key = idx, ch)
    KIND_SC3_SEQ = 5,
    KIND_SPLICE = 6,   // spliceCount (key "a-b")
};

// Entry flags
enum : uint32_t {
    SF_PDIFF = 1u,      // two pstd-relevant observations with different read positions
    SF_QDIFF = 2u,      // ... with different mean qualities
    SF_ZERO = 4u,       // an observation with read position 0 or quality 0: pstd/qstd depend on
                        // the order of observations and are replayed in read order (k_fix_order)
    SF_ERASED = 8u,     // removed by the realigner
    SF_FIRST = 16u,     // first_tp / first_q hold a value
    SF_FORCE_STD = 32u, // pstd and qstd forced true (adjCnt)
    SF_OVR = 64u,       // statistics set by the -k 1 realigner: the allele count is
                        // in first_tp, tp_sum/mq_sum/nm_sum hold double bits, and
                        // pstd/qstd are exactly SF_PDIFF/SF_QDIFF
    SF_NOMAP = 128u,    // the realigner removed the position's map entry
};

// One allele key of the device hash table.
struct alignas(16) Slot {
    unsigned long long fp;   // fingerprint of (region, kind, pos, key); 0 = empty
    unsigned long long h2x;  // XOR of a second hash over all inserters (collision check)
    int32_t region, pos;
    uint16_t kind, klen;
    uint32_t koff;           // key bytes in the arena
    int32_t fwd, rev, hi, lo, obs, extracnt;
    long long tp_sum, mq_sum, nm_sum;
    double q_sum;
    unsigned long long first_q;  // double bits of the first pstd-relevant quality
    int32_t first_tp;
    uint32_t flags;
    uint32_t min_stamp;      // first read (batch index) that created the key
    uint32_t next;           // next slot at the same position (per-position list), ~0u = end
};

// Per-region record on the device.
struct Region {
    int32_t start, end;      // region, 1-based inclusive
    int32_t ws, we;          // reference window [ws, we] (RecordPreprocessor::makeReference)
    int32_t clo, chi;        // cell range (positions with a cell)
    int64_t cell_base;       // index of position clo in the cell arrays
    int64_t r0, r1;          // candidate read range in the batch
    int32_t span_lo, span_hi; // min/max position any read of the region may touch
    int32_t serial;          // 1: reads can reach past the window (edge reads); with edge_hit set,
                             // the region is processed by the in-order exact walker
    int32_t max_read_len;    // maxReadLength of the region
    int32_t err;             // error bits
    int32_t edge_hit;        // an edge read would insert a position past the window
    int32_t reach;           // max over the region's reads of (span end - 1-based start)
    int32_t pad;
};

struct Tile {
    int32_t region;
    int32_t wlo;             // first position of the tile's shared-memory window (host-computed)
    int64_t r0, r1;          // entries [r0, r1) of the tile read list (DevState::tile_reads)
};

// A read is an edge read of a region when its span reaches within this many
// positions of the reference window's end.
constexpr int kEdgeMargin = 8;

// Batch preparation on the device (rv_prep.cu): result words
// (PREP_MISALIGNED bits: 1 base_off not a multiple of 32, 2 CIGAR outside the
// batch's words, 4 bases outside the batch's bases)
enum { PREP_MAX_SPAN = 0, PREP_MAX_LQ = 1, PREP_MISALIGNED = 2, PREP_SPAN_BAD = 3, PREP_N_TILES = 4, PREP_WORDS = 8 };

struct ReadPrepIn {
    int64_t n;
    const int32_t *pos, *l_qseq;
    const uint16_t *n_cigar;
    const uint32_t *cig_off, *cigar;
    const uint64_t *base_off;
    int64_t n_cigar_words, n_bases;  // bounds of every read's CIGAR and bases (checked)
    int widen;               // -k 1: edge insertions widen the span
};
struct ReadPrepOut {
    int32_t *span_lo, *span_hi;
    uint8_t *cost;           // walk-cost class: 0 one M op, 1 soft clips around one M op, 2 other
    int *words;
};
// Per region: its read list's class segments and their tiles.
struct RegionTiles {
    long long start[3], count[3];  // list segment of each class (relative to the region's list start)
    long long per[3];              // reads per tile of each class
    int tile0[3];                  // first tile of each class (relative to base)
    int n_tiles, base;             // tiles of the region; its first tile in the batch's list
};
struct RegionPrepArgs {
    Region *regions;
    const int32_t *span_lo, *span_hi, *pos;
    const uint8_t *cost;
    int max_span, max_lq;
    RegionTiles *rtiles;
    int *words;
};
struct RegionFillArgs {
    const Region *regions;
    const RegionTiles *rtiles;
    const int64_t *list_begin;
    const int32_t *span_lo, *span_hi;
    const uint8_t *cost;
    uint32_t *list;
    Tile *tiles;
};

// Device copy of rv_params plus derived values.
struct DevParams {
    double goodq, freq, qratio, mapq_filter, lofreq, bias;
    int32_t vext, mismatch, local_realign, minr, read_pos_filter, min_mapq, min_bias_reads, samfilter;
    int32_t trim_bases_after, minmatch, dedup, unique_fwd, unique_first, do_pileup, fisher, move_indels_3;
    int32_t svminlen, somatic;
    int32_t dataset_min;  // > 0: candidate-set scoring (every allele seen this many times)
    int32_t goodq_i;      // ceil(goodq): for an integer quality q, q >= goodq exactly when q >= goodq_i
};

// Cell arrays: one cell per (position, base A/C/G/T); index = 4 * cell + b.
struct Cells {
    uint32_t *fwd, *rev, *hi, *tp, *q, *mq;
    int32_t *nm;
    uint32_t *first;     // packed first (tp, q) of pstd-relevant observations | flag bits
    uint32_t *cov;       // per position: refCoverage
    uint8_t *kflags;     // per position: bit b = key b exists, bit 4+b = key b erased
    int64_t n_cells;     // positions
};

struct Batch {
    int64_t n_reads;
    const int32_t *pos, *mpos, *nm, *l_qseq;
    const uint16_t *flag, *n_cigar;
    const uint8_t *mapq;
    const uint32_t *cig_off, *cigar;
    const uint64_t *base_off;
    const uint8_t *seq, *qual;
    const uint8_t *skip;    // -t: 1 = duplicate read (null when -t is off)
    int32_t max_lq;         // longest read of the batch (bounds how far left of its
                            // position a read can reach)
};

struct Hash {
    Slot *slots;
    unsigned long long mask;   // capacity - 1 (power of two)
    uint8_t *arena;
    unsigned long long arena_cap;
    unsigned long long *arena_used;
    unsigned int *n_used;      // slots claimed so far
    uint32_t *used;            // their indexes, in claim order (mask + 1 entries):
                               // scans and the next reset visit only these
};

#ifdef __CUDACC__
// Number of valid entries of the used-slot list.
__device__ __forceinline__ unsigned long long used_count(const Hash &H) {
    const unsigned long long n = *H.n_used;
    return n <= H.mask ? n : H.mask + 1ULL;
}

// Claims the next entry of the used-slot list for slot i.
__device__ __forceinline__ void note_used(const Hash &H, unsigned long long i) {
    const unsigned int k = atomicAdd(H.n_used, 1u);
    if ((unsigned long long)k <= H.mask) H.used[k] = (uint32_t)i;
}
#endif

// Deferred subtraction of a reference-base observation after an insertion
// (src/parseCigar.cpp:1471-1490): applied only if the key existed when the
// insertion was seen, which a later kernel decides.
struct Deferred {
    int32_t region, pos;
    int64_t read;            // batch index of the read that saw the insertion
    int32_t ci;              // CIGAR op index of the insertion
    int32_t base;            // 0..3
    int32_t dir, tp, q, mapq, nm;
    int32_t pad;
};

// A map entry whose pstd/qstd the pileup cannot settle without the order of
// its observations: the reference sets the flag when an observation differs
// from the previous one and the previous one is nonzero
// (src/parseCigar.cpp:902-914, 1446-1457), so an observation with read
// position 0 or quality 0 (or a value outside the packed cell range) makes
// the result order-dependent.  k_fix_order replays such entries in read order.
struct OrderFix {
    int32_t region, pos;
    int32_t base;            // 0..3: the A/C/G/T cell key; -1: a hash slot
    int32_t pad;
    int64_t index;           // cell word (4 * cell + base) or slot index
};

// A position whose alleles do not fit the per-thread arrays of the scoring
// kernels (kMaxVars): scored again by the wide kernels with `need` entries
// of global scratch.
struct WidePos {
    int32_t region, pos;
    int32_t need;            // alleles (and insertion keys) at the position
    int32_t forced;          // scored without screens (somatic list)
};

// Error word bits (per context)
enum : uint32_t {
    ERR_HASH_FULL = 1u,
    ERR_ARENA_FULL = 2u,
    ERR_KEY_TOO_LONG = 4u,
    ERR_DEFER_FULL = 8u,
    ERR_CELL_RANGE = 16u,
    ERR_UNSUPPORTED = 32u,
    ERR_PROBE_LIMIT = 64u,
    ERR_COLLISION = 128u,
    ERR_FIX_FULL = 256u,     // more order-dependent entries than the OrderFix list holds
    ERR_CAND_FULL = 512u,    // more scored alleles than the candidate buffer holds
    ERR_WIDE_FULL = 1024u,   // more wide positions than the WidePos lists hold
    ERR_WIDE_INS_SCRATCH = 2048u,    // the wide insertion pass needs more scratch (it did nothing)
    ERR_WIDE_SCORE_SCRATCH = 4096u,  // the wide score pass needs more scratch (it did nothing)
};

// One scored allele at a candidate position, handed to the host for the
// string part of collectReferenceVariants and the record text.
struct CandVar {
    int32_t region, pos;
    int32_t kind;            // 0 reference allele, 1 variant allele
    int32_t rank;            // order after the CMP_VARI sort (src/ToVarsBuilder.cpp:20-26)
    int32_t key_off, key_len;  // key bytes in the arena; key_len < 0: single base, key_off = 0..3
    int32_t pc, fwd, rev, hicnt, hicov, tpc, rfc, rrc;
    int32_t bias, ref_bias, pstd, qstd, pass, nvars;
    double freq, pmean, qual, mq, qratio, hifreq, extrafreq, nm;
    double fisher_p, fisher_ratio;
};

struct DevState {
    Batch batch;
    Region *regions;
    int32_t n_regions;
    Tile *tiles;
    int32_t n_tiles;
    const uint32_t *tile_reads;  // per region, its reads grouped by CIGAR shape (one M op; clips around one M op; other)
    unsigned int *tile_counter;
    Cells cells;
    Hash hash;
    Deferred *deferred;
    unsigned int *n_deferred;
    unsigned int deferred_cap;
    const char *ref;        // whole contig, uppercase, 0-based
    int32_t ref_len;
    unsigned int *err;
    uint32_t *head;          // per cell: first NONINS/INS hash slot at that position
    uint32_t *head_sc;       // per cell: first soft-clip slot at that position
    int64_t *score_base;     // per region: first scoring thread (prefix sum of region lengths)
    int64_t n_score;
    CandVar *cand;
    unsigned int *n_cand;
    unsigned int cand_cap;
    const double *logfact;   // log(k!) for k < kLogFact (Fisher tests)
    OrderFix *ofix;          // entries k_fix_order replays
    unsigned int *n_ofix;
    unsigned int ofix_cap;
    WidePos *wide_ins;       // positions k_ins_adjust left to the wide pass
    WidePos *wide_score;     // positions the score kernels left to the wide pass
    unsigned int *n_wide_ins, *n_wide_score;
    unsigned int wide_cap;
};

constexpr int kLogFact = 1 << 16;

}  // namespace rv
