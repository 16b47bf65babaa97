// Allocation-free Fisher exact tests.
//
// Some callers of this library cannot call cudaMalloc: host processes whose
// device memory is owned by another allocator (a framework's caching pool)
// or that run under a fixed device-memory budget, and plugin hosts that
// forbid a library from allocating behind their back.  rv_fisher_batch_static
// serves them: the caller passes device buffers for the tables and the
// results, and the only extra memory the kernels use is a file-scope
// __device__ array (the log-factorial table below), reserved on every GPU
// that loads the library for as long as the process runs.
//
// The call scans the tables on the device, reads the largest total back to
// the host and waits for `stream` (cudaStreamSynchronize) before it launches
// the test kernels.
//
// The two-sided test is the same computation as rv_fisher_batch (the
// hypergeometric definition, relative tie slack 1e-7); here the log
// factorials come from the scratch table instead of per-term lgamma calls.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "rvgpu.h"

namespace {

// Largest a+b+c+d a table may have (the scratch table holds log(k!) for
// k = 0..kMaxTotal): 2 MB of device memory.
constexpr int kMaxTotal = (1 << 18) - 1;
constexpr int kMaxDevices = 64;

// scratch: log-factorial table and two words (largest total, invalid-table flag)
static __device__ __align__(256) double g_logfact[kMaxTotal + 1];
static __device__ __align__(256) unsigned int g_words[2];

double *g_lf_ptr[kMaxDevices];
unsigned int *g_words_ptr[kMaxDevices];
bool g_ready[kMaxDevices];
std::mutex g_mu;

__global__ void k_scan_totals(const int32_t *tab, int64_t n, unsigned int *words) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        long long a = tab[4 * i], b = tab[4 * i + 1], c = tab[4 * i + 2], d = tab[4 * i + 3];
        long long t = a + b + c + d;
        if (a < 0 || b < 0 || c < 0 || d < 0 || t > kMaxTotal) {
            atomicOr(&words[1], 1u);
            continue;
        }
        atomicMax(&words[0], (unsigned int)t);
    }
}

// log(k!) for k = 0..top (top <= kMaxTotal, checked by the host)
__global__ void k_fill_logfact(double *lf, unsigned int top) {
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k <= top; k += gridDim.x * blockDim.x)
        lf[k] = lgamma((double)k + 1.0);
}

__device__ __forceinline__ double log_choose_t(const double *lf, int n, int k) { return lf[n] - lf[k] - lf[n - k]; }

// `top`: the largest total this call filled the table for.  A table outside
// [0, top] (possible only if another call changed the tables or the scratch
// words in between, which the caller must not allow) gets NaN instead of an
// index past the filled part of the table.
__global__ void k_fisher_table(const int32_t *tab, int64_t n, const double *lf, unsigned int top, double *p2,
                               double *ratio) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int n11 = tab[4 * i], n12 = tab[4 * i + 1], n21 = tab[4 * i + 2], n22 = tab[4 * i + 3];
        const long long total = (long long)n11 + n12 + n21 + n22;
        if (n11 < 0 || n12 < 0 || n21 < 0 || n22 < 0 || total > (long long)top) {
            p2[i] = __longlong_as_double(0x7FF8000000000000LL);
            ratio[i] = __longlong_as_double(0x7FF8000000000000LL);
            continue;
        }
        int r1 = n11 + n12, c1 = n11 + n21, nn = (int)total;
        int lo = r1 + c1 - nn > 0 ? r1 + c1 - nn : 0;
        int hi = r1 < c1 ? r1 : c1;
        double two = 1.0;
        if (!(n11 < 0 || n12 < 0 || n21 < 0 || n22 < 0 || lo >= hi)) {
            double base = log_choose_t(lf, nn, c1);
            double p_obs = exp(log_choose_t(lf, r1, n11) + log_choose_t(lf, nn - r1, c1 - n11) - base);
            double thr = p_obs * (1.0 + 1e-7);
            double s = 0.0;
            for (int x = lo; x <= hi; ++x) {
                double p = exp(log_choose_t(lf, r1, x) + log_choose_t(lf, nn - r1, c1 - x) - base);
                if (p <= thr) s += p;
            }
            two = s > 1.0 ? 1.0 : s;
        }
        p2[i] = two;
        double ad = (double)n11 * n22, bc = (double)n12 * n21;
        ratio[i] = (bc != 0 && ad != 0) ? (ad > bc ? ad / bc : bc / ad) : 0.0;
    }
}

void put_err(char *buf, size_t len, const char *msg) {
    if (buf && len) {
        strncpy(buf, msg, len - 1);
        buf[len - 1] = 0;
    }
}

}  // namespace

extern "C" rv_status rv_fisher_batch_static(const int32_t *d_tables, int64_t n, double *d_two_sided, double *d_ratio,
                                            void *stream, char *errbuf, size_t errbuf_len) {
    if (n < 0 || (n > 0 && (!d_tables || !d_two_sided || !d_ratio))) {
        put_err(errbuf, errbuf_len, "rv_fisher_batch_static: null buffer or negative count");
        return RV_ERR_ARG;
    }
    if (n == 0) return RV_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        put_err(errbuf, errbuf_len, e != cudaSuccess ? cudaGetErrorString(e) : "device ordinal out of range");
        return RV_ERR_CUDA;
    }
    // set-up, once per device with that device current: the device addresses
    // of the scratch symbols (the host-side names are not device addresses)
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_ready[dev]) {
            void *a = nullptr, *b = nullptr;
            e = cudaGetSymbolAddress(&a, g_logfact);
            if (e == cudaSuccess) e = cudaGetSymbolAddress(&b, g_words);
            if (e != cudaSuccess) {
                put_err(errbuf, errbuf_len, cudaGetErrorString(e));
                return RV_ERR_CUDA;
            }
            g_lf_ptr[dev] = (double *)a;
            g_words_ptr[dev] = (unsigned int *)b;
            g_ready[dev] = true;
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *lf = g_lf_ptr[dev];
    unsigned int *words = g_words_ptr[dev];
    // the two scratch words keep the previous call's values: clear them
    e = cudaMemsetAsync(words, 0, 2 * sizeof(unsigned int), s);
    int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    if (e == cudaSuccess) {
        k_scan_totals<<<grid, 256, 0, s>>>(d_tables, n, words);
        e = cudaGetLastError();
    }
    unsigned int host_words[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_words, words, sizeof host_words, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        put_err(errbuf, errbuf_len, cudaGetErrorString(e));
        return RV_ERR_CUDA;
    }
    if (host_words[1]) {
        char msg[160];
        snprintf(msg, sizeof msg,
                 "rv_fisher_batch_static: a table has a negative count or a total above %d (the scratch limit)",
                 kMaxTotal);
        put_err(errbuf, errbuf_len, msg);
        return RV_ERR_ARG;
    }
    const unsigned int top = host_words[0];  // <= kMaxTotal: larger totals set the invalid word
    k_fill_logfact<<<(int)((top + 256) / 256 < 1024 ? (top + 256) / 256 : 1024), 256, 0, s>>>(lf, top);
    k_fisher_table<<<grid, 128, 0, s>>>(d_tables, n, lf, top, d_two_sided, d_ratio);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        put_err(errbuf, errbuf_len, cudaGetErrorString(e));
        return RV_ERR_CUDA;
    }
    return RV_OK;
}
