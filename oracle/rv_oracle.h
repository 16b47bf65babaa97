/* Oracle test infrastructure -- not part of the product.
 *
 * CPU restatement of RabbitVar's per-region pileup and scoring path
 * (record filters, CIGAR walk, local-realigner MNP adjustment, per-site
 * statistics, hard filter, Fisher test, simple-mode record formatting).
 * Each function in rv_oracle.cpp cites the reference file:line it restates.
 * It is pinned against the reference itself (oracle/_ref, built from the
 * unmodified sources by oracle/Makefile) by the CPU tests, and is then the
 * checker for the GPU library.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it. */
#ifndef RV_ORACLE_H
#define RV_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Reads of one contig in file (coordinate) order; the same structure of
 * arrays the GPU library consumes.  seq4 holds one BAM 4-bit code per base
 * (unpacked), qual one Phred value per base, both at base_off[i]. */
typedef struct {
    int64_t n;
    const int32_t *pos;     /* 0-based */
    const uint16_t *flag;
    const uint8_t *mapq;
    const int32_t *mpos;    /* 0-based */
    const int32_t *nm;      /* NM tag, INT32_MIN when absent */
    const uint16_t *n_cigar;
    const uint32_t *cig_off;
    const uint32_t *cigar;
    const int32_t *l_qseq;
    const uint64_t *base_off;
    const uint8_t *seq4;
    const uint8_t *qual;
} rvo_reads;

typedef struct {
    double goodq;          /* -q, 22.5 */
    int vext;              /* -X, 2 */
    int mismatch;          /* -m, 8 */
    int local_realign;     /* -k, 1 */
    double freq;           /* -f, 0.01 */
    int minr;              /* -r, 2 */
    int read_pos_filter;   /* -P, 5 */
    double qratio;         /* -o, 1.5 */
    double mapq_filter;    /* -O, 0 */
    int min_mapq;          /* -Q, 0 */
    double lofreq;         /* -V, 0.05 */
    double bias;           /* 0.05 */
    int min_bias_reads;    /* -B, 2 */
    int samfilter;         /* -F, 0x504 */
    int ref_extension;     /* -Y, 1200 */
    int extend_nt;         /* -x, 0 */
    int trim_bases_after;  /* -T, 0 */
    int minmatch;          /* -M, 0 */
    int dedup;             /* -t */
    int unique_fwd;        /* -u */
    int unique_first;      /* --UN */
    int do_pileup;         /* -p */
    int fisher;            /* --fisher */
    int move_indels_3;     /* -3 */
    int svminlen;          /* 1000 */
} rvo_params;

void rvo_default_params(rvo_params *p);

/* Runs the region [start, end] (1-based, inclusive) of contig `chr`
 * (`ref` holds the whole contig, 0-based, `contig_len` bytes).
 * `stages` selects dump sections: P (pileup maps), R (after realigner),
 * V (per-site variants), O (output records).  The text is malloc'd into
 * *out (free with rvo_free).  Returns 0 on success. */
int rvo_run_region(const rvo_reads *reads, const char *ref, int contig_len,
                   const char *chr, int start, int end, const char *sample,
                   const rvo_params *p, const char *stages, char **out, size_t *out_len);

/* Same pipeline over many regions with OpenMP (one region per task, as the
 * reference's BED mode does); only the output records are produced.
 * Returns the number of records written into *out. */
long rvo_run_regions(const rvo_reads *reads, const char *ref, int contig_len, const char *chr,
                     const int32_t *starts, const int32_t *ends, int n_regions,
                     const char *sample, const rvo_params *p, int threads,
                     char **out, size_t *out_len);

/* Somatic mode (a tumor/normal pair, `-b 'T.bam|N.bam'`): both samples run
 * the per-region pipeline on the same reference window; the tumor's
 * positions are classified against the normal's variants and written as
 * 63-column records (64 with the trailing tab).  Stage V dumps the per-site
 * variants of both samples (VT / VN lines). */
int rvo_run_somatic(const rvo_reads *tumor, const rvo_reads *normal, const char *ref, int contig_len,
                    const char *chr, int start, int end, const char *sample,
                    const rvo_params *p, const char *stages, char **out, size_t *out_len);

long rvo_run_somatic_regions(const rvo_reads *tumor, const rvo_reads *normal, const char *ref,
                             int contig_len, const char *chr, const int32_t *starts,
                             const int32_t *ends, int n_regions, const char *sample,
                             const rvo_params *p, int threads, char **out, size_t *out_len);

void rvo_free(char *p);

double rvo_fisher(int n11, int n12, int n21, int n22, double *left, double *right, double *two);

#ifdef __cplusplus
}
#endif
#endif
