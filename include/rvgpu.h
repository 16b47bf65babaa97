/* rvgpu.h -- C ABI of the GB300 pileup-and-scoring library.
 *
 * Replaces the per-region stage sequence RabbitVar runs in one_region_run
 * (src/modes/simpleMode.cpp:18-64):
 *     RecordPreprocessor(region, conf, bamReaders)       src/recordPreprocessor.cpp:10-32
 *     CigarParser::process(Scope<InitialData>)           src/parseCigar.cpp:410-440
 *     VariationRealigner::process(Scope<VariationData>)  src/VariationRealigner.cpp:135-161
 *     ToVarsBuilder::process(Scope<RealignedVariationData>) src/ToVarsBuilder.cpp:97-205
 *     SimpleMode::output / print_output_variant_simple   src/modes/simpleMode.cpp:66-208
 * for a whole batch of regions at once.  All entry points are extern "C",
 * take plain pointers and sizes, return rv_status (0 = OK, negative = error)
 * and never exit the process.  One context per host thread; calls on one
 * context are not thread-safe.  The context owns all device memory; the
 * caller owns every host buffer it passes in.
 */
#ifndef RVGPU_H
#define RVGPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef int rv_status;
enum {
    RV_OK = 0,
    RV_ERR_ARG = -1,         /* bad argument or size */
    RV_ERR_CUDA = -2,        /* a CUDA runtime call failed (rv_last_error has the text) */
    RV_ERR_CAPACITY = -3,    /* a device table overflowed; retry with a larger budget */
    RV_ERR_TIMEOUT = -4,     /* a bounded device wait gave up */
    RV_ERR_UNSUPPORTED = -5, /* input uses a feature this build does not handle */
    RV_ERR_STATE = -6,       /* call out of order (e.g. score before pileup) */
    RV_ERR_COLLISION = -7,   /* allele-key fingerprint collision detected */
    RV_ERR_FORMAT = -8       /* malformed BAM/BGZF input */
};

typedef struct rv_ctx rv_ctx;

/* Mirrors the Configuration fields the path reads (include/Configuration.h:98-401).
 * rv_default_params fills the reference's defaults. */
typedef struct {
    double goodq;          /* -q  22.5 */
    int32_t vext;          /* -X  2 */
    int32_t mismatch;      /* -m  8 */
    int32_t local_realign; /* -k  1: the CIGAR rewrite runs in rv_pileup; rv_realign runs adjustMNP
                              and the indel passes (realignIndels) over the device maps */
    double freq;           /* -f  0.01 */
    int32_t minr;          /* -r  2 */
    int32_t read_pos_filter; /* -P 5 */
    double qratio;         /* -o  1.5 */
    double mapq_filter;    /* -O  0 */
    int32_t min_mapq;      /* -Q  0 */
    double lofreq;         /* -V  0.05 */
    double bias;           /* 0.05 */
    int32_t min_bias_reads; /* -B 2 */
    int32_t samfilter;     /* -F  0x504 */
    int32_t ref_extension; /* -Y  1200 */
    int32_t extend_nt;     /* -x  0 */
    int32_t trim_bases_after; /* -T 0 */
    int32_t minmatch;      /* -M  0 */
    int32_t dedup;         /* -t */
    int32_t unique_fwd;    /* -u */
    int32_t unique_first;  /* --UN */
    int32_t do_pileup;     /* -p: every covered position printed (simple mode; no effect in somatic mode) */
    int32_t fisher;        /* --fisher */
    int32_t move_indels_3; /* -3 */
    int32_t svminlen;      /* 1000 */
    int32_t somatic;       /* a second BAM is configured (conf->bam.hasBam2()): the context is
                              one sample of a tumor/normal pair, see rv_score_pair */
} rv_params;

/* Reads of one contig in coordinate (file) order, structure of arrays.
 * seq is BAM-packed (4-bit codes, high nibble first) at byte base_off[i]/2;
 * qual holds one Phred byte per base at base_off[i]; base_off[i] must be a
 * multiple of 32 (so every read's bases start 16-byte aligned).
 * nm[i] is the NM tag or INT32_MIN when the record has none. */
typedef struct {
    int64_t n_reads;
    const int32_t *pos;      /* 0-based leftmost (BAM POS) */
    const uint16_t *flag;
    const uint8_t *mapq;
    const int32_t *mpos;     /* 0-based mate position */
    const int32_t *nm;
    const uint16_t *n_cigar;
    const uint32_t *cig_off; /* index of the first CIGAR word */
    const uint32_t *cigar;   /* BAM CIGAR words (len << 4 | op) */
    int64_t n_cigar_words;
    const int32_t *l_qseq;
    const uint64_t *base_off;
    const uint8_t *seq;      /* n_bases / 2 bytes */
    const uint8_t *qual;     /* n_bases bytes */
    int64_t n_bases;
} rv_read_batch;

/* One region [start, end] (1-based inclusive, as Region in include/Region.h). */
typedef struct {
    int32_t start;
    int32_t end;
} rv_region;

/* Per emitted record, the numeric part; the allele strings and flanks are in
 * the text produced by rv_format_records. */
typedef struct {
    int32_t region;
    int32_t position;
    int32_t start, end;
    int32_t total_cov, var_cov, ref_fwd, ref_rev, alt_fwd, alt_rev;
    double freq, pmean, qual, mapq, qratio, hifreq, extrafreq, msi, nm;
    int32_t pstd, qstd, shift3, msint, hicnt, hicov;
    double fisher_p, fisher_ratio;
} rv_site_record;

void rv_default_params(rv_params *p);

/* device: CUDA ordinal; hbm_budget: bytes of device memory the context may
 * hold (0 = up to 90% of free memory). */
rv_status rv_create(rv_ctx **out, const rv_params *p, int device, size_t hbm_budget);
void rv_destroy(rv_ctx *ctx);
const char *rv_last_error(const rv_ctx *ctx);

/* Replaces RecordPreprocessor::makeReference (src/recordPreprocessor.cpp:41-78):
 * uploads a whole contig (ASCII bases, any case); each region's window is
 * derived from it exactly as the reference does. */
rv_status rv_upload_reference(rv_ctx *ctx, const char *chr, const char *bases, int64_t n);

/* Replaces the record iterator (sam_itr_querys + next_record,
 * src/recordPreprocessor.cpp:101-180) for a batch of regions: queues the
 * copy of the host batch to the device on `stream` (cudaStream_t, NULL =
 * default) and the batch's preparation there (read spans, region bounds,
 * the tiles of the pileup), without waiting for either; the host arrays
 * must stay unchanged until the following rv_pileup has returned.  A CIGAR
 * outside the batch's words is refused here; the device's record checks
 * (base_off a multiple of 32, bases inside the batch's bases) are reported
 * by that rv_pileup.
 * With local realignment (-k 1) rv_realign reads the batch's host arrays
 * pos, flag, n_cigar, cig_off and cigar again (the reference's realigner
 * re-reads the records of a region): they must stay valid and unchanged
 * until rv_realign of this batch returns. */
rv_status rv_submit_batch(rv_ctx *ctx, const rv_read_batch *reads, const rv_region *regions, int n_regions,
                          void *stream);

/* Replaces CigarParser::process (src/parseCigar.cpp:410-974): record filters,
 * CIGAR walk and allele-count maps for every region of the batch. */
rv_status rv_pileup(rv_ctx *ctx, void *stream);

/* Replaces VariationRealigner::process (src/VariationRealigner.cpp:135-161):
 * host realigner over the device-built maps.  -k 0: adjustMNP (:334-465),
 * reading only the MNP keys and their neighbours from the device.  -k 1:
 * adjustMNP and realignIndels (:467-1360) per region (regions in parallel)
 * over a mirror of the maps filled from the device around every candidate;
 * noPassingReads reads the batch's alignment spans kept on the host.  The
 * changes are written back to the device maps (realigned statistics, erased
 * and new keys, coverage).  Once per batch (RV_ERR_STATE on a second call). */
rv_status rv_realign(rv_ctx *ctx, void *stream);

/* Replaces ToVarsBuilder::process (src/ToVarsBuilder.cpp:97-205), the hard
 * filter (Variant::isGoodVar, include/Variant.h:197-248) and the --fisher
 * test: per-site statistics and candidate selection on the device. */
rv_status rv_score(rv_ctx *ctx, void *stream);

/* Replaces SimpleMode::output (src/modes/simpleMode.cpp:144-208): builds the
 * tab-delimited records (allele strings, MSI, flanks on the host) into a
 * context-owned buffer valid until the next call on ctx.  `sample` is the -N
 * name, `gene` the region label (the contig name for -R). */
rv_status rv_format_records(rv_ctx *ctx, const char *sample, const char *gene, const char **text,
                            size_t *text_len, int64_t *n_records);

/* Copies up to `cap` numeric records; *n receives the total available. */
rv_status rv_fetch_records(rv_ctx *ctx, rv_site_record *out, size_t cap, size_t *n);

/* Convenience: submit + pileup + realign + score + format in one call. */
rv_status rv_call_regions(rv_ctx *ctx, const rv_read_batch *reads, const rv_region *regions, int n_regions,
                          const char *sample, const char *gene, const char **text, size_t *text_len,
                          int64_t *n_records);

/* Pileup-boundary map export for parity checks and for host consumers of the
 * maps (the realigner's input, VariationData in
 * include/scopedata/VariationData.h:14-56): writes a text dump of region
 * `region` in the same line format as the oracle dump (P* lines).  Valid
 * until the next call on ctx. */
/* Somatic mode: the tumor/normal pair of `-b 'T.bam|N.bam'` (SomaticMode::process,
 * src/modes/somaticMode.cpp:83-127 one_region_run_somt, :311-353 output).  `tumor`
 * and `normal` are two contexts created with params.somatic = 1, given the same
 * contig (rv_upload_reference) and the same region list (rv_submit_batch with each
 * sample's reads), and each taken through rv_pileup and rv_realign.
 *
 * rv_score_pair replaces the two ToVarsBuilder::process calls: it scores both
 * samples and then, in each sample, the positions where only the other one has a
 * candidate, so every position that can produce a record is complete in both.
 * rv_format_somatic replaces SomaticMode::output + print_output_variant_simple
 * (:151-309): the labels StrongSomatic, LikelySomatic, Germline, AFDiff,
 * LikelyLOH, StrongLOH, SampleSpecific and the 63-column records (64 fields with
 * the trailing tab; 55 without --fisher), the three Fisher tests of each record
 * run on the device.  As in the reference, positions come from the tumor only.
 * The text belongs to `tumor` until its next call.  rv_call_somatic runs the
 * whole sequence. */
rv_status rv_score_pair(rv_ctx *tumor, rv_ctx *normal);

/* rv_pileup then rv_realign on both samples of a pair, overlapped: both
 * samples' pileup kernels are queued first (each context has its own
 * stream) and the tumor's host realigner runs while the normal's pileup is
 * on the device.  Same results and errors as the four calls in sequence. */
rv_status rv_pileup_realign_pair(rv_ctx *tumor, rv_ctx *normal);
rv_status rv_format_somatic(rv_ctx *tumor, rv_ctx *normal, const char *sample, const char *gene,
                            const char **text, size_t *text_len, int64_t *n_records);
rv_status rv_call_somatic(rv_ctx *tumor, rv_ctx *normal, const rv_read_batch *tumor_reads,
                          const rv_read_batch *normal_reads, const rv_region *regions, int n_regions,
                          const char *sample, const char *gene, const char **text, size_t *text_len,
                          int64_t *n_records);

/* A sequence of somatic batches (the contigs of a pair of BAM files, or
 * chunks of a BED file): the two samples' reads of one region list.  A job
 * whose tumor and normal batches are both NULL runs again on the batch its
 * context pair already holds (regions as submitted then). */
typedef struct {
    const rv_read_batch *tumor, *normal;
    const rv_region *regions;
    int n_regions;
    const char *sample, *gene;
} rv_somatic_job;

/* Receives each job's records, in job order, on the calling thread; the text
 * is valid during the call. */
typedef void (*rv_somatic_sink)(void *user, int64_t job, const char *text, size_t text_len, int64_t n_records);

/* rv_call_somatic over n_jobs jobs with two context pairs (tumor0/normal0 take
 * the even jobs, tumor1/normal1 the odd ones): while one pair's batch is piled
 * up, realigned and scored, a host thread formats the other pair's records and
 * uploads that pair's next batch.  The records are those of n_jobs rv_call_somatic calls (the
 * reference's per-region loop over a BED file, SomaticMode::process,
 * src/modes/somaticMode.cpp:736-990, emits them in the same order). */
rv_status rv_call_somatic_stream(rv_ctx *tumor0, rv_ctx *normal0, rv_ctx *tumor1, rv_ctx *normal1,
                                 const rv_somatic_job *jobs, int64_t n_jobs, rv_somatic_sink sink, void *user);

/* Candidate set of the learned filter (include/rvgpu_mlp.h); no counterpart in
 * the reference.  rv_score_candidates replaces rv_score after rv_realign: every
 * position with a non-reference allele seen at least `min_count` times keeps all
 * its alleles (the -f gate and the isGoodVar pre-screen are not applied).
 * rv_candidates then returns, for every candidate allele (reference alleles
 * excluded) in one order, RV_FEATURES floats (features[n][RV_FEATURES], computed
 * on the device from the allele's site statistics, its key and the reference
 * around it) and an rv_candidate with its position, key and whether simple mode
 * (rv_format_records, i.e. the hard filter) emits it.  With both pointers NULL
 * only *n is set. */
#define RV_FEATURES 40
typedef struct {
    int32_t region, position;  /* region index, 1-based position */
    int32_t hard_pass;         /* 1: emitted by the hard filter */
    int32_t key_len;           /* length of the allele key */
    char key[48];              /* allele key, truncated to 47 bytes, NUL-terminated */
} rv_candidate;
rv_status rv_score_candidates(rv_ctx *ctx, int min_count);
rv_status rv_candidates(rv_ctx *ctx, float *features, rv_candidate *cands, int64_t cap, int64_t *n);

rv_status rv_export_maps(rv_ctx *ctx, int region, const char *stages, const char **text, size_t *text_len);

/* Timing of the last rv_pileup/rv_score call (device time, ms, CUDA events on
 * the launch stream) and the number of device kernels those calls launched. */
rv_status rv_last_timings(const rv_ctx *ctx, double *pileup_ms, double *score_ms, double *total_ms,
                          int64_t *kernels);

/* Device time (ms, CUDA events on the launch stream) of the last rv_pileup /
 * rv_score calls by stage:
 * stages: [0] cell/table reset, [1] region spans, [2] pileup tiles,
 * [3] in-order edge walk, [4] deferred subtraction + list linking +
 * collision check, [5] insertion coverage adjustment, [6] site scoring;
 * [7] the pileup kernel variant the autotuner used (not a time).
 * Stages [0]-[4] read 0 after a pileup launched as a graph. */
rv_status rv_stage_times(const rv_ctx *ctx, double *ms, int n);

/* Batched-region form of CigarParser::process (src/parseCigar.cpp:410-440)
 * under a CUDA graph: with enable != 0, rv_pileup captures its chain of
 * memsets and kernels (table resets, edge detection, the tile kernel fed
 * from the device tile queue, in-order edge walk, deferred
 * subtraction, list linking, collision check) into a graph and launches that,
 * once the autotuner has settled on a kernel variant.  Each batch's chain is
 * applied to the previous executable graph with cudaGraphExecUpdate; a new
 * one is instantiated only when the update is refused.  The stream must not
 * be the legacy default stream (NULL selects the context's own stream).
 * Results are the same as without the graph. */
rv_status rv_set_pileup_graph(rv_ctx *ctx, int enable);

/* Graph launches and graph instantiations of rv_pileup since rv_create. */
rv_status rv_pileup_graph_stats(const rv_ctx *ctx, int64_t *launches, int64_t *instantiations);

/* Capacities of the context's device tables for the next rv_submit_batch
 * (0 keeps the automatic size): hash slots of string-keyed alleles (rounded
 * up to a power of two), bytes of allele-key text, deferred reference-base
 * subtractions after insertions, and map entries whose pstd/qstd are replayed
 * in read order.  A table that overflows during rv_pileup grows to what the
 * run needed and the pileup runs again (at most three times, then
 * RV_ERR_CAPACITY), so these set where growth starts.  No counterpart in
 * the reference, whose maps grow on the host heap (include/VariationUtils.h:
 * 148-195); the automatic sizes follow the keys per read seen so far. */
rv_status rv_set_capacities(rv_ctx *ctx, size_t hash_slots, size_t arena_bytes, size_t deferred,
                            size_t order_fix);

/* Pileups run again after a table grew (since rv_create), and the current
 * hash-slot and key-arena capacities. */
rv_status rv_capacity_stats(const rv_ctx *ctx, int64_t *retries, int64_t *hash_slots, int64_t *arena_bytes);

/* Bytes copied host->device by the last rv_submit_batch and device->host
 * by the calls since then (realigner boundary, scored candidates). */
rv_status rv_io_bytes(const rv_ctx *ctx, int64_t *h2d, int64_t *d2h);

/* Fisher exact test on the device for n tables (a,b,c,d) stored as 4*n int32;
 * writes two-sided p and the simple-mode ratio. Replaces the kt_fisher_exact
 * call sites (src/modes/simpleMode.cpp:96-108). */
rv_status rv_fisher_batch(rv_ctx *ctx, const int32_t *tables, int64_t n, double *two_sided, double *ratio);

/* Allocation-free variant of rv_fisher_batch for callers that cannot call
 * cudaMalloc: processes whose device memory belongs to another allocator (a
 * framework's caching pool) or to a fixed budget, and plugin hosts that
 * forbid a library from allocating behind their back.  It has no
 * counterpart in the reference (which calls htslib's kt_fisher_exact on the
 * host per record); it runs the same two-sided test as rv_fisher_batch.
 *
 * d_tables (4*n int32: a b c d per table), d_two_sided and d_ratio (n
 * doubles each) are device buffers the caller owns; `stream` is a
 * cudaStream_t (NULL = legacy default stream) on the current device.  The
 * only other memory used is a file-scope device array: a log-factorial table
 * for totals a+b+c+d up to 262143 (2 MB), held on every GPU that loads the
 * library until the process exits.  A table with a negative count or a
 * larger total is rejected with RV_ERR_ARG and a message in errbuf (when
 * errbuf_len > 0); nothing is written to the outputs then.
 * The first call on each device looks up the device address of that array
 * (cudaGetSymbolAddress, with the device current).  Every call shares the
 * array and re-clears the words that must start at zero; calls whose work
 * overlaps on the GPU (two streams, two host threads on one device) race on
 * it and must be serialised by the caller.  The call reads the largest
 * table total back to the host and synchronises `stream` (a host wait)
 * before it launches the test kernels. */
rv_status rv_fisher_batch_static(const int32_t *d_tables, int64_t n, double *d_two_sided, double *d_ratio,
                                 void *stream, char *errbuf, size_t errbuf_len);

#ifdef __cplusplus
}
#endif
#endif
