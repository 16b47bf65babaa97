/* Oracle test infrastructure.
 *
 * FP64 restatement of the two-sided Fisher exact test on a 2x2 table, the
 * computation RabbitVar obtains from htslib's kt_fisher_exact at
 * src/modes/simpleMode.cpp:96-108 and src/modes/somaticMode.cpp:130-149.
 * htslib is absent here, so parity with htslib's own p-values is unpinned;
 * this restatement is written from the hypergeometric definition and is
 * cross-checked against scipy.stats.fisher_exact in the CPU tests.
 *
 *   P(X = x) = C(r1, x) C(n - r1, c1 - x) / C(n, c1),  r1 = n11 + n12,
 *   c1 = n11 + n21, n = n11 + n12 + n21 + n22, x in [max(0, r1 + c1 - n),
 *   min(r1, c1)].
 *   left  = P(X <= n11), right = P(X >= n11),
 *   two   = sum of P(X = x) over x with P(X = x) <= P(X = n11) (1 + 1e-7).
 * The relative slack 1e-7 treats numerically tied tables as tied. */
#ifndef RV_FISHER_ORACLE_H
#define RV_FISHER_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif
double rv_oracle_fisher(int n11, int n12, int n21, int n22,
                        double *left, double *right, double *two);
#ifdef __cplusplus
}
#endif
#endif
