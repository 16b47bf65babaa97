/* rvgpu_io.h -- host input helpers of librvgpu (C ABI).
 *
 * Replace the htslib calls RabbitVar makes to obtain records and reference
 * bases (RecordPreprocessor, src/recordPreprocessor.cpp:10-78): BGZF/BAM
 * decode into pinned structure-of-arrays read batches, FASTA loading, and
 * pinned host allocations for callers that build batches themselves.
 */
#ifndef RVGPU_IO_H
#define RVGPU_IO_H
#include "rvgpu.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct rv_bam rv_bam;

/* Inflates a whole BGZF-compressed BAM file (members decoded on `threads`
 * host threads, 0 = all cores) and indexes its records.  Replaces sam_open +
 * sam_hdr_read + the record iterator (src/recordPreprocessor.cpp:10-32). */
rv_status rv_bam_read(const char *path, int threads, rv_bam **out);

/* rv_bam_read on a BGZF/BAM file already in memory (n bytes at bgzf). */
rv_status rv_bam_read_mem(const uint8_t *bgzf, size_t n, int threads, rv_bam **out);

/* Reference sequences named in the BAM header (bam_hdr_t target_name/len). */
rv_status rv_bam_contigs(const rv_bam *bam, int *n, const char *const **names, const int32_t **lens);

/* Structure-of-arrays batch of every record on contig `tid`, in file order,
 * in pinned host memory owned by `bam` (valid until rv_bam_free). */
rv_status rv_bam_batch(rv_bam *bam, int tid, rv_read_batch *out);

/* BGZF/BAM decode on the GPU `device`: `bgzf` (n bytes of host memory,
 * pinned for a fast upload) is a whole BAM file.  Each BGZF member is inflated
 * by one device thread; record starts are found per member on the device and
 * checked as one chain from the header's end; fixed fields and the NM tag are
 * read per record on the device.  Same records, fields and layout as
 * rv_bam_read; replaces htslib's BGZF reader and record iterator
 * (src/recordPreprocessor.cpp:10-32,101-180).  RV_ERR_FORMAT on malformed
 * input (the device decoder bounds every access and reports instead). */
rv_status rv_bam_read_gpu(const uint8_t *bgzf, size_t n, int device, rv_bam **out);

/* Decodes another BGZF/BAM file into a handle from rv_bam_read_gpu, reusing
 * its device and pinned buffers (they only grow); batches taken from the
 * handle before are invalid afterwards. */
rv_status rv_bam_reread_gpu(rv_bam *bam, const uint8_t *bgzf, size_t n);

/* For a BAM from rv_bam_read_gpu, rv_bam_batch leaves `seq` and `qual` in
 * device memory of that GPU (rv_submit_batch copies them device to device)
 * and the other arrays in pinned host memory; rv_bam_batch_host returns every
 * array in pinned host memory.  For a BAM from rv_bam_read both are the same. */
rv_status rv_bam_batch_host(rv_bam *bam, int tid, rv_read_batch *out);

void rv_bam_free(rv_bam *bam);

/* Reads sequence `name` (NULL = first) of a FASTA file; *seq is malloc'd,
 * free it with rv_free.  Replaces fai_load/fai_fetch
 * (src/recordPreprocessor.cpp:56-72). */
rv_status rv_fasta_read(const char *path, const char *name, char **seq, int64_t *len);
void rv_free(void *p);

/* Pinned (page-locked) host memory for batch buffers the caller fills. */
void *rv_alloc_pinned(size_t bytes);
void rv_free_pinned(void *p);

#ifdef __cplusplus
}
#endif
#endif
