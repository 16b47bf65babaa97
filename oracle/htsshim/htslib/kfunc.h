/* Oracle test infrastructure: project restatement of the htslib Fisher
 * exact test entry point (two-sided, left and right tails of the
 * hypergeometric distribution of the 2x2 table). */
#ifndef RV_SHIM_KFUNC_H
#define RV_SHIM_KFUNC_H
double kt_fisher_exact(int n11, int n12, int n21, int n22,
                       double *left, double *right, double *two);
#endif
