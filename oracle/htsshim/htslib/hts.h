/* Oracle test infrastructure: project-written subset of the public htslib
 * API used by RabbitVar (file handles, index and region iterators).
 * Semantics follow the htslib documentation; the implementation in
 * hts_shim.cpp is written from the SAM/BAM v1 and BGZF specifications. */
#ifndef RV_SHIM_HTS_H
#define RV_SHIM_HTS_H
#include <stdint.h>
#include <stddef.h>

typedef int64_t hts_pos_t;

struct rvshim_file;   /* opaque: a BAM file whose records are held in memory */
struct rvshim_index;
struct rvshim_iter;
typedef struct rvshim_file samFile;
typedef struct rvshim_file htsFile;
typedef struct rvshim_index hts_idx_t;
typedef struct rvshim_iter hts_itr_t;

void hts_idx_destroy(hts_idx_t *idx);
void hts_itr_destroy(hts_itr_t *iter);
#endif
