/* Oracle test infrastructure: see fisher_oracle.h. */
#include "fisher_oracle.h"
#include <math.h>

static double log_choose(int n, int k) {
    return lgamma((double)n + 1.0) - lgamma((double)k + 1.0) - lgamma((double)(n - k) + 1.0);
}

double rv_oracle_fisher(int n11, int n12, int n21, int n22,
                        double *left, double *right, double *two) {
    int r1 = n11 + n12, c1 = n11 + n21, n = n11 + n12 + n21 + n22;
    int lo = r1 + c1 - n > 0 ? r1 + c1 - n : 0;
    int hi = r1 < c1 ? r1 : c1;
    if (n11 < 0 || n12 < 0 || n21 < 0 || n22 < 0 || lo >= hi) {
        *left = *right = *two = 1.0;
        return 1.0;
    }
    double base = log_choose(n, c1);
    double lp_obs = log_choose(r1, n11) + log_choose(n - r1, c1 - n11) - base;
    double p_obs = exp(lp_obs);
    double thr = p_obs * (1.0 + 1e-7);
    double sl = 0.0, sr = 0.0, st = 0.0;
    for (int x = lo; x <= hi; ++x) {
        double p = exp(log_choose(r1, x) + log_choose(n - r1, c1 - x) - base);
        if (x <= n11) sl += p;
        if (x >= n11) sr += p;
        if (p <= thr) st += p;
    }
    *left = sl > 1.0 ? 1.0 : sl;
    *right = sr > 1.0 ? 1.0 : sr;
    *two = st > 1.0 ? 1.0 : st;
    return p_obs;
}
