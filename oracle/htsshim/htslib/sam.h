/* Oracle test infrastructure: project-written subset of the public htslib
 * SAM/BAM API used by RabbitVar.  Record layout follows the BAM v1
 * specification (section 4.2): the variable-length block of a record is
 * read name (NUL-terminated, padded with extra NULs so the CIGAR starts on
 * a 4-byte boundary), CIGAR (uint32 per op: len<<4|op), 4-bit packed
 * sequence, Phred qualities, then optional tags. */
#ifndef RV_SHIM_SAM_H
#define RV_SHIM_SAM_H
#include "hts.h"

/* CIGAR operation codes (BAM spec 4.2: "MIDNSHP=X" -> 0..8) */
enum {
    BAM_CMATCH = 0, BAM_CINS = 1, BAM_CDEL = 2, BAM_CREF_SKIP = 3,
    BAM_CSOFT_CLIP = 4, BAM_CHARD_CLIP = 5, BAM_CPAD = 6, BAM_CEQUAL = 7,
    BAM_CDIFF = 8, BAM_CBACK = 9
};
#define BAM_CIGAR_SHIFT 4
#define BAM_CIGAR_MASK  0xf

/* FLAG bits (SAM spec 1.4) */
#define BAM_FPAIRED        0x1
#define BAM_FPROPER_PAIR   0x2
#define BAM_FUNMAP         0x4
#define BAM_FMUNMAP        0x8
#define BAM_FREVERSE       0x10
#define BAM_FMREVERSE      0x20
#define BAM_FREAD1         0x40
#define BAM_FREAD2         0x80
#define BAM_FSECONDARY     0x100
#define BAM_FQCFAIL        0x200
#define BAM_FDUP           0x400
#define BAM_FSUPPLEMENTARY 0x800

typedef struct {
    hts_pos_t pos;      /* 0-based leftmost position */
    int32_t tid;
    uint16_t bin;
    uint8_t qual;       /* MAPQ */
    uint8_t l_extranul; /* NULs added after the read name for alignment */
    uint16_t flag;
    uint16_t l_qname;   /* name length including NULs and padding */
    uint32_t n_cigar;
    int32_t l_qseq;
    int32_t mtid;
    hts_pos_t mpos;
    hts_pos_t isize;
} bam1_core_t;

typedef struct {
    bam1_core_t core;
    uint64_t id;
    uint8_t *data;
    int l_data;
    uint32_t m_data;
} bam1_t;

typedef struct {
    int32_t n_targets;
    uint32_t *target_len;
    char **target_name;
} bam_hdr_t;
typedef bam_hdr_t sam_hdr_t;

/* 4-bit base code -> character (BAM spec 4.2, field seq) */
extern const char seq_nt16_str[];

static inline uint32_t *bam_get_cigar(const bam1_t *b) {
    return (uint32_t *)(b->data + b->core.l_qname);
}
static inline uint8_t *bam_get_seq(const bam1_t *b) {
    return b->data + b->core.l_qname + 4u * b->core.n_cigar;
}
static inline uint8_t *bam_get_qual(const bam1_t *b) {
    return bam_get_seq(b) + ((b->core.l_qseq + 1) >> 1);
}
static inline uint8_t *bam_get_aux(const bam1_t *b) {
    return bam_get_qual(b) + b->core.l_qseq;
}
static inline int bam_seqi(const uint8_t *s, int i) {
    return (i & 1) ? (s[i >> 1] & 0xf) : (s[i >> 1] >> 4);
}
static inline int bam_is_rev(const bam1_t *b) { return (b->core.flag & BAM_FREVERSE) != 0; }
static inline int bam_cigar_op(uint32_t c) { return (int)(c & BAM_CIGAR_MASK); }
static inline uint32_t bam_cigar_oplen(uint32_t c) { return c >> BAM_CIGAR_SHIFT; }
static inline char bam_cigar_opchr(uint32_t c) {
    static const char ops[] = "MIDNSHP=XB??????";
    return ops[c & BAM_CIGAR_MASK];
}
/* bit 0: consumes query; bit 1: consumes reference (SAM spec 1.4, CIGAR table) */
static inline int bam_cigar_type(int op) {
    switch (op) {
    case BAM_CMATCH: case BAM_CEQUAL: case BAM_CDIFF: return 3;
    case BAM_CINS: case BAM_CSOFT_CLIP: return 1;
    case BAM_CDEL: case BAM_CREF_SKIP: return 2;
    default: return 0;
    }
}

samFile *sam_open(const char *fn, const char *mode);
int sam_close(samFile *fp);
bam_hdr_t *sam_hdr_read(samFile *fp);
void bam_hdr_destroy(bam_hdr_t *h);
hts_idx_t *sam_index_load(samFile *fp, const char *fn);
hts_itr_t *sam_itr_querys(const hts_idx_t *idx, bam_hdr_t *hdr, const char *region);
int sam_itr_next(samFile *fp, hts_itr_t *iter, bam1_t *b);
bam1_t *bam_init1(void);
void bam_destroy1(bam1_t *b);
hts_pos_t bam_endpos(const bam1_t *b);
uint8_t *bam_aux_get(const bam1_t *b, const char tag[2]);
int64_t bam_aux2i(const uint8_t *s);
char *bam_aux2Z(const uint8_t *s);
#endif
