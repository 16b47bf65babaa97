/* Oracle test infrastructure: project-written subset of the htslib FASTA
 * index API (fai_load / fai_fetch), following the .fai format
 * (name, length, offset, bases per line, bytes per line). */
#ifndef RV_SHIM_FAIDX_H
#define RV_SHIM_FAIDX_H
#include "hts.h"
struct rvshim_fai;
typedef struct rvshim_fai faidx_t;
faidx_t *fai_load(const char *fn);
void fai_destroy(faidx_t *fai);
/* region "name:beg-end" (1-based, inclusive); returns malloc'd upper/lower
 * case bases as stored, length in *len; beyond the contig end is clipped. */
char *fai_fetch(const faidx_t *fai, const char *reg, int *len);
#endif
