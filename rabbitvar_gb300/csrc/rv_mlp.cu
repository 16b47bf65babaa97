// Learned candidate filter: an MLP 40 -> 128 -> 128 -> 128 -> 1 (GELU, erf
// form) over the per-candidate feature vector, trained and run with
// hand-written tcgen05 kernels: BF16 operands staged in shared memory, FP32
// accumulators in tensor memory (TMEM), one elected thread issuing the MMAs.
//
// Every matrix product is C[M x N] = A[M x K] * B[N x K]^T with both operands
// K-major (K contiguous), M tiles of 128 rows, N = 64 or 128, K in chunks of
// 64.  Forward layers, the hidden-gradient products and the weight-gradient
// products (K = batch, split across CTAs) differ only in their epilogues.
// One training step is a fixed sequence of launches (gather, 3 forward
// GEMMs, the output layer with loss, 3 weight-gradient GEMMs, 2
// hidden-gradient GEMMs, Adam) captured once in a CUDA graph.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "rvgpu_mlp.h"

namespace {

constexpr int H = 128;       // hidden width
constexpr int KIN = 64;      // first-layer input width (40 features, zero padded)
constexpr int NF = RV_MLP_FEATURES;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * KIN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + H,
              N_PARAM = OFF_B4 + 1;
static_assert(N_PARAM == RV_MLP_PARAMS, "parameter layout");

constexpr int kTileM = 128, kChunkK = 64;
constexpr uint32_t kTmemCols = 256;
// 2 CTAs per SM at most (dynamic shared memory), so the 512 TMEM columns of
// an SM always cover both allocations
constexpr int kGemmSmem = 96 * 1024;

typedef __nv_bfloat16 bf16;

enum { EPI_FWD = 0, EPI_DH = 1, EPI_DW = 2 };

struct Epi {
    const float *bias;    // EPI_FWD: bias[n]
    float *z;             // EPI_FWD: pre-activation out [m][H]; EPI_DH: pre-activation of the layer below (in)
    bf16 *h;              // EPI_FWD: GELU out [m][H]; EPI_DH: dz out [m][H]
    bf16 *ht;             // transposed copy [n][ldt]
    int ldt;
    float *db;            // EPI_DH: column sums of dz (bias gradient of the layer below)
    float *dw;            // EPI_DW: fp32 accumulation target [m][N]
    unsigned int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of
// 8 rows x 16 bytes; `lbo` = byte distance of core matrices along K, `sbo`
// = along M/N.  Version field 1 (bits 46-47) for this architecture.
__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// Waits for phase `parity` of an mbarrier, at most ~1 s; false on timeout.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > 4000000000LL) return false;
    }
}

// Copies rows [r0, r0 + R) x columns [k0, k0 + 64) of a K-major BF16 matrix
// into shared memory in the core-matrix layout of make_desc(.., 128, 1024):
// element (r, k) at (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
template <int R>
__device__ __forceinline__ void stage_tile(unsigned char *dst, const bf16 *src, int ld, int r0, int k0) {
    for (int i = threadIdx.x; i < R * 8; i += blockDim.x) {
        int r = i >> 3, j = i & 7;
        uint4 v = *reinterpret_cast<const uint4 *>(src + (size_t)(r0 + r) * ld + k0 + 8 * j);
        *reinterpret_cast<uint4 *>(dst + (r >> 3) * 1024 + j * 128 + (r & 7) * 16) = v;
    }
}

// C tile = A[m0.., k-range] * B[0..N, k-range]^T, accumulated in TMEM, then the epilogue.
// grid.x: M tiles; grid.y: K splits of `kper` columns each.  The operands of
// 64-column chunks are staged in two shared-memory buffers: while the tensor
// core multiplies chunk i out of one, the threads stage chunk i + 1 into the
// other (after the MMAs of chunk i - 1, which read it, have completed: each
// buffer's commits arrive on its own mbarrier).
template <int N, int EPI>
__global__ void __launch_bounds__(128, 1) k_umma(const bf16 *A, int lda, const bf16 *B, int ldb, int kper, Epi e) {
    extern __shared__ __align__(1024) unsigned char smem[];
    constexpr int kStage = 16384 + N * kChunkK * 2;  // one buffer: A 128 x 64, B N x 64 (bf16)
    static_assert(2 * kStage <= kGemmSmem, "two staging buffers");
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t s_tmem;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTileM;
    const int kb = blockIdx.y * kper;
    const int nk = (kper + kChunkK - 1) / kChunkK;
    const uint32_t bar0 = smem_u32(&bar[0]);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (nk > 0) {
        stage_tile<kTileM>(smem, A, lda, m0, kb);
        stage_tile<N>(smem + 16384, B, ldb, 0, kb);
    }
    // generic-proxy shared-memory writes -> visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = make_idesc(kTileM, N);
    bool ok = true;
    int committed = -1;  // last chunk whose MMAs were committed
    for (int it = 0; it < nk; ++it) {
        const int buf = it & 1;
        unsigned char *sa = smem + buf * kStage;
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(sa), b0 = a0 + 16384;
#pragma unroll
            for (int kk = 0; kk < kChunkK / 16; kk++) {
                uint64_t ad = make_desc(a0 + kk * 256, 128, 1024);
                uint64_t bd = make_desc(b0 + kk * 256, 128, 1024);
                uint32_t acc = (it > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             bar0 + 8 * buf)
                         : "memory");
        }
        committed = it;
        if (it + 1 < nk) {
            // the other buffer was read by chunk it - 1: wait for its MMAs
            // (the (it - 1) / 2-th phase of that buffer's barrier)
            bool done = true;
            if (it >= 1) done = mbar_wait(bar0 + 8 * (buf ^ 1), (uint32_t)(((it - 1) >> 1) & 1));
            if (!__syncthreads_and(done)) {
                ok = false;
                break;
            }
            unsigned char *na = smem + (buf ^ 1) * kStage;
            stage_tile<kTileM>(na, A, lda, m0, kb + (it + 1) * kChunkK);
            stage_tile<N>(na + 16384, B, ldb, 0, kb + (it + 1) * kChunkK);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
        }
    }
    // the last commit tracks every MMA issued before it; after a timeout the
    // MMAs already committed are waited for (bounded) before TMEM is freed
    if (committed >= 0) {
        const bool done = mbar_wait(bar0 + 8 * (committed & 1), (uint32_t)((committed >> 1) & 1));
        if (!__syncthreads_and(done)) ok = false;
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicOr(e.err, 1u);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int m = m0 + warp * 32 + lane;  // TMEM lane = row of the tile
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t v[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int n = c0 + j;
                const float acc = __uint_as_float(v[j]);
                if (EPI == EPI_FWD) {
                    const float z = acc + e.bias[n];
                    e.z[(size_t)m * H + n] = z;
                    const bf16 hv = __float2bfloat16_rn(gelu(z));
                    e.h[(size_t)m * H + n] = hv;
                    e.ht[(size_t)n * e.ldt + m] = hv;
                } else if (EPI == EPI_DH) {
                    const bf16 dz = __float2bfloat16_rn(acc * gelu_grad(e.z[(size_t)m * H + n]));
                    e.h[(size_t)m * H + n] = dz;
                    e.ht[(size_t)n * e.ldt + m] = dz;
                    float s = __bfloat162float(dz);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                    if (lane == 0) atomicAdd(&e.db[n], s);
                } else {
                    atomicAdd(&e.dw[(size_t)m * N + n], acc);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// Per-step scalars of a training run, in device memory so that one captured
// step replays for every batch: the batch index within the epoch and the
// Adam step count.
struct StepState {
    int64_t batch;
    int64_t t;
};

// Batch rows -> BF16 layer-1 input (zero padded to 64 columns) and its
// transpose; rows past `n` are zero (their loss weight is zero).  The first
// row is `b0`, or batch * B when `ss` is given.
__global__ void k_gather(const float *feat, const int32_t *idx, int64_t n, int64_t b0, int B, bf16 *h0, bf16 *h0t,
                         float *y_out, const float *y, const StepState *ss) {
    if (ss) b0 = ss->batch * B;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * KIN; i += gridDim.x * blockDim.x) {
        const int r = i / KIN, c = i % KIN;
        const int64_t g = b0 + r;
        float v = 0.f;
        if (g < n && c < NF) v = feat[(size_t)(idx ? idx[g] : g) * NF + c];
        const bf16 hv = __float2bfloat16_rn(v);
        h0[(size_t)r * KIN + c] = hv;
        h0t[(size_t)c * B + r] = hv;
        if (c == 0 && y_out) y_out[r] = g < n ? y[idx ? idx[g] : g] : -1.f;
    }
}

// Output layer (dot with w4) and, when training, the weighted BCE loss, the
// gradient of the last hidden layer (dz3 = dlogit * w4 * GELU'(z3)) and the
// output-layer gradients.  One thread per row.
__global__ void k_head(const bf16 *h3, const float *z3, const float *params, int B, const float *y, float pos_weight,
                       float inv_n, float *logit_out, bf16 *dz3, bf16 *dz3t, float *grad, float *loss,
                       const StepState *ss = nullptr, int64_t n_total = 0) {
    if (ss) inv_n = 1.f / (float)min((int64_t)B, n_total - ss->batch * B);  // rows of this batch
    __shared__ float s_db3[H], s_dw4[H];
    for (int i = threadIdx.x; i < H; i += blockDim.x) { s_db3[i] = 0.f; s_dw4[i] = 0.f; }
    __syncthreads();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const float *w4 = params + OFF_W4;
    float lsum = 0.f, dl = 0.f;
    bool live = false;
    if (m < B) {
        float a = params[OFF_B4];
        for (int nn = 0; nn < H; nn++) a += __bfloat162float(h3[(size_t)m * H + nn]) * w4[nn];
        if (logit_out) logit_out[m] = a;
        if (y && y[m] >= 0.f) {
            live = true;
            const float t = y[m];
            const float w = t > 0.5f ? pos_weight : 1.f;
            const float sp = a > 0.f ? a + log1pf(expf(-a)) : log1pf(expf(a));
            lsum = w * (sp - t * a);
            const float sig = 1.f / (1.f + expf(-a));
            dl = w * (sig - t) * inv_n;
        }
    }
    if (y) {
        if (m < B) {
            for (int nn = 0; nn < H; nn++) {
                const bf16 d = __float2bfloat16_rn(dl * w4[nn] * gelu_grad(z3[(size_t)m * H + nn]));
                dz3[(size_t)m * H + nn] = d;
                dz3t[(size_t)nn * B + m] = d;
                if (live) {
                    atomicAdd(&s_db3[nn], __bfloat162float(d));
                    atomicAdd(&s_dw4[nn], dl * __bfloat162float(h3[(size_t)m * H + nn]));
                }
            }
        }
        float ls = lsum, dsum = dl;
        for (int o = 16; o > 0; o >>= 1) {
            ls += __shfl_xor_sync(0xffffffffu, ls, o);
            dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(loss, ls * inv_n);
            atomicAdd(&grad[OFF_B4], dsum);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < H; i += blockDim.x) {
            atomicAdd(&grad[OFF_B3 + i], s_db3[i]);
            atomicAdd(&grad[OFF_W4 + i], s_dw4[i]);
        }
    }
}

__global__ void k_logistic(const float *logit, int64_t n, float *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = 1.f / (1.f + expf(-logit[i]));
}

// BF16 copies of the weights: W[out][in] (forward) and W^T[in][out] (hidden gradients)
__global__ void k_cast(const float *p, bf16 *w1, bf16 *w2, bf16 *w3, bf16 *w2t, bf16 *w3t) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * H; i += gridDim.x * blockDim.x) {
        const int o = i / H, c = i % H;
        if (i < H * KIN) w1[i] = __float2bfloat16_rn(p[OFF_W1 + i]);
        const bf16 a = __float2bfloat16_rn(p[OFF_W2 + i]), b = __float2bfloat16_rn(p[OFF_W3 + i]);
        w2[i] = a;
        w3[i] = b;
        w2t[(size_t)c * H + o] = a;
        w3t[(size_t)c * H + o] = b;
    }
}

// Adam on the FP32 master parameters; the padded input columns of W1 stay 0.
__global__ void k_adam(float *p, const float *g, float *mo, float *ve, float lr, float b1, float b2, float eps,
                       float c1, float c2, const StepState *ss) {
    if (ss) {  // bias corrections of step t (1-based)
        const double t = (double)(ss->t + 1);
        c1 = (float)(1.0 - pow((double)b1, t));
        c2 = (float)(1.0 - pow((double)b2, t));
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N_PARAM; i += gridDim.x * blockDim.x) {
        if (i < OFF_B1 && (i % KIN) >= NF) continue;
        const float gi = g[i];
        const float m = b1 * mo[i] + (1.f - b1) * gi;
        const float v = b2 * ve[i] + (1.f - b2) * gi * gi;
        mo[i] = m;
        ve[i] = v;
        p[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

__global__ void k_advance(StepState *ss) {
    ss->batch += 1;
    ss->t += 1;
}

}  // namespace

struct rv_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    int B = 0;  // batch rows (multiple of 128)
    float *params = nullptr, *grad = nullptr, *mo = nullptr, *ve = nullptr;
    bf16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr, *w2t = nullptr, *w3t = nullptr;
    bf16 *h0 = nullptr, *h0t = nullptr, *h[3] = {}, *ht[3] = {}, *dz[3] = {}, *dzt[3] = {};
    float *z[3] = {};
    float *y = nullptr, *logit = nullptr, *loss = nullptr;
    unsigned int *err = nullptr;
    float *feat = nullptr, *labels = nullptr;  // device copies of the training set
    int32_t *perm = nullptr;
    int64_t cap_n = 0;
    int64_t steps = 0;
    StepState *ss = nullptr;        // device
    cudaGraphExec_t step_graph = nullptr;
    int64_t graph_n = -1;           // training-set size the graph was captured for
    float graph_lr = 0, graph_pw = 0;
    double step_ms = 0;             // mean time of a training step (last train call)
    std::string msg;
};

namespace {

#define MCUDA(call)                                                           \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) {                                              \
            m->msg = std::string(#call) + ": " + cudaGetErrorString(e_);      \
            return RV_ERR_CUDA;                                               \
        }                                                                     \
    } while (0)

template <int N, int EPI>
cudaError_t gemm(rv_mlp *m, const bf16 *A, int lda, const bf16 *Bm, int ldb, int mtiles, int ksplit, int kper,
                 const Epi &e) {
    k_umma<N, EPI><<<dim3(mtiles, ksplit), 128, kGemmSmem, m->stream>>>(A, lda, Bm, ldb, kper, e);
    return cudaGetLastError();
}

// forward of batch rows already gathered into h0; logits into m->logit
cudaError_t forward(rv_mlp *m, int B) {
    const bf16 *in = m->h0;
    int kin = KIN;
    const bf16 *W[3] = {m->w1, m->w2, m->w3};
    const float *bias[3] = {m->params + OFF_B1, m->params + OFF_B2, m->params + OFF_B3};
    for (int l = 0; l < 3; l++) {
        Epi e{};
        e.bias = bias[l];
        e.z = m->z[l];
        e.h = m->h[l];
        e.ht = m->ht[l];
        e.ldt = B;
        e.err = m->err;
        cudaError_t x = gemm<H, EPI_FWD>(m, in, kin, W[l], kin, B / kTileM, 1, kin, e);
        if (x != cudaSuccess) return x;
        in = m->h[l];
        kin = H;
    }
    return cudaSuccess;
}

// one training step: gather batch `ss->batch` of the shuffled training set,
// forward, backward, Adam; every per-step scalar is read from `ss`, so the
// launch sequence is the same for every step (it is captured once)
cudaError_t train_step(rv_mlp *m, int B, int64_t n, float pos_weight, float lr) {
    k_gather<<<256, 256, 0, m->stream>>>(m->feat, m->perm, n, 0, B, m->h0, m->h0t, m->y, m->labels, m->ss);
    cudaError_t x = forward(m, B);
    if (x != cudaSuccess) return x;
    cudaMemsetAsync(m->grad, 0, N_PARAM * sizeof(float), m->stream);
    k_head<<<B / 128, 128, 0, m->stream>>>(m->h[2], m->z[2], m->params, B, m->y, pos_weight, 1.f, m->logit,
                                           m->dz[2], m->dzt[2], m->grad, m->loss, m->ss, n);
    // weight gradients: dW_l = dz_l^T * h_{l-1}, K = batch, split in chunks of 512 rows
    const int kper = std::min(B, 512), ks = B / kper;
    const bf16 *hprev_t[3] = {m->h0t, m->ht[0], m->ht[1]};
    const int off_w[3] = {OFF_W1, OFF_W2, OFF_W3};
    const int off_b[3] = {OFF_B1, OFF_B2, OFF_B3};
    const bf16 *wt[3] = {nullptr, m->w2t, m->w3t};
    for (int l = 2; l >= 0; l--) {
        Epi e{};
        e.dw = m->grad + off_w[l];
        e.err = m->err;
        if (l == 0) x = gemm<KIN, EPI_DW>(m, m->dzt[0], B, hprev_t[0], B, 1, ks, kper, e);
        else x = gemm<H, EPI_DW>(m, m->dzt[l], B, hprev_t[l], B, 1, ks, kper, e);
        if (x != cudaSuccess) return x;
        if (l == 0) break;
        // dz_{l-1} = (dz_l * W_l) * GELU'(z_{l-1})
        Epi d{};
        d.z = m->z[l - 1];
        d.h = m->dz[l - 1];
        d.ht = m->dzt[l - 1];
        d.ldt = B;
        d.db = m->grad + off_b[l - 1];
        d.err = m->err;
        x = gemm<H, EPI_DH>(m, m->dz[l], H, wt[l], H, B / kTileM, 1, H, d);
        if (x != cudaSuccess) return x;
    }
    const float b1 = 0.9f, b2 = 0.999f;
    k_adam<<<(N_PARAM + 255) / 256, 256, 0, m->stream>>>(m->params, m->grad, m->mo, m->ve, lr, b1, b2, 1e-8f, 1.f,
                                                         1.f, m->ss);
    k_cast<<<64, 256, 0, m->stream>>>(m->params, m->w1, m->w2, m->w3, m->w2t, m->w3t);
    k_advance<<<1, 1, 0, m->stream>>>(m->ss);
    return cudaGetLastError();
}

// the GEMM kernels' shared-memory size is set once, outside any capture
cudaError_t gemm_attrs() {
    cudaError_t x = cudaFuncSetAttribute(k_umma<H, EPI_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    if (x == cudaSuccess)
        x = cudaFuncSetAttribute(k_umma<H, EPI_DH>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    if (x == cudaSuccess)
        x = cudaFuncSetAttribute(k_umma<H, EPI_DW>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    if (x == cudaSuccess)
        x = cudaFuncSetAttribute(k_umma<KIN, EPI_DW>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    return x;
}

rv_status check_err(rv_mlp *m) {
    unsigned int e = 0;
    MCUDA(cudaMemcpyAsync(&e, m->err, 4, cudaMemcpyDeviceToHost, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));
    if (e) {
        m->msg = "tensor-core pipeline wait timed out";
        return RV_ERR_TIMEOUT;
    }
    return RV_OK;
}

rv_status ensure_data(rv_mlp *m, int64_t n) {
    if (n <= m->cap_n && m->feat) return RV_OK;
    cudaFree(m->feat);
    cudaFree(m->labels);
    cudaFree(m->perm);
    m->feat = nullptr;
    m->labels = nullptr;
    m->perm = nullptr;
    MCUDA(cudaMalloc((void **)&m->feat, (size_t)std::max<int64_t>(n, 1) * NF * sizeof(float)));
    MCUDA(cudaMalloc((void **)&m->labels, (size_t)std::max<int64_t>(n, 1) * sizeof(float)));
    MCUDA(cudaMalloc((void **)&m->perm, (size_t)std::max<int64_t>(n, 1) * sizeof(int32_t)));
    m->cap_n = n;
    return RV_OK;
}

}  // namespace

extern "C" {

rv_status rv_mlp_create(rv_mlp **out, int device, int batch, uint64_t seed) {
    if (!out || batch < 128 || batch % 512 != 0 || batch > (1 << 16)) return RV_ERR_ARG;
    rv_mlp *m = new rv_mlp();
    *out = m;
    m->device = device;
    m->B = batch;
    MCUDA(cudaSetDevice(device));
    MCUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    const size_t P = N_PARAM * sizeof(float);
    MCUDA(cudaMalloc((void **)&m->params, P));
    MCUDA(cudaMalloc((void **)&m->grad, P));
    MCUDA(cudaMalloc((void **)&m->mo, P));
    MCUDA(cudaMalloc((void **)&m->ve, P));
    MCUDA(cudaMemset(m->mo, 0, P));
    MCUDA(cudaMemset(m->ve, 0, P));
    MCUDA(cudaMalloc((void **)&m->w1, H * KIN * sizeof(bf16)));
    bf16 **wq[4] = {&m->w2, &m->w3, &m->w2t, &m->w3t};
    for (auto w : wq) MCUDA(cudaMalloc((void **)w, H * H * sizeof(bf16)));
    const size_t B = (size_t)batch;
    MCUDA(cudaMalloc((void **)&m->h0, B * KIN * sizeof(bf16)));
    MCUDA(cudaMalloc((void **)&m->h0t, B * KIN * sizeof(bf16)));
    for (int l = 0; l < 3; l++) {
        MCUDA(cudaMalloc((void **)&m->h[l], B * H * sizeof(bf16)));
        MCUDA(cudaMalloc((void **)&m->ht[l], B * H * sizeof(bf16)));
        MCUDA(cudaMalloc((void **)&m->dz[l], B * H * sizeof(bf16)));
        MCUDA(cudaMalloc((void **)&m->dzt[l], B * H * sizeof(bf16)));
        MCUDA(cudaMalloc((void **)&m->z[l], B * H * sizeof(float)));
    }
    MCUDA(cudaMalloc((void **)&m->y, B * sizeof(float)));
    MCUDA(cudaMalloc((void **)&m->logit, B * sizeof(float)));
    MCUDA(cudaMalloc((void **)&m->loss, sizeof(float)));
    MCUDA(cudaMalloc((void **)&m->err, sizeof(unsigned int)));
    MCUDA(cudaMemset(m->err, 0, sizeof(unsigned int)));
    MCUDA(cudaMalloc((void **)&m->ss, sizeof(StepState)));
    MCUDA(cudaMemset(m->ss, 0, sizeof(StepState)));
    MCUDA(gemm_attrs());
    // He-normal hidden weights, zero biases (host generator, fixed seed)
    std::vector<float> p(N_PARAM, 0.f);
    std::mt19937_64 rng(seed);
    auto normal = [&](double sd) {
        // Box-Muller on 53-bit uniforms: the same numbers on every host
        double u1 = ((rng() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        double u2 = ((rng() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        return (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    };
    for (int o = 0; o < H; o++)
        for (int c = 0; c < NF; c++) p[OFF_W1 + o * KIN + c] = normal(std::sqrt(2.0 / NF));
    for (int i = 0; i < H * H; i++) p[OFF_W2 + i] = normal(std::sqrt(2.0 / H));
    for (int i = 0; i < H * H; i++) p[OFF_W3 + i] = normal(std::sqrt(2.0 / H));
    for (int i = 0; i < H; i++) p[OFF_W4 + i] = normal(std::sqrt(1.0 / H));
    return rv_mlp_set_params(m, p.data());
}

void rv_mlp_destroy(rv_mlp *m) {
    if (!m) return;
    cudaSetDevice(m->device);
    void *ptrs[] = {m->params, m->grad, m->mo, m->ve, m->w1, m->w2, m->w3, m->w2t, m->w3t, m->h0, m->h0t,
                    m->h[0], m->h[1], m->h[2], m->ht[0], m->ht[1], m->ht[2], m->dz[0], m->dz[1], m->dz[2],
                    m->dzt[0], m->dzt[1], m->dzt[2], m->z[0], m->z[1], m->z[2], m->y, m->logit, m->loss,
                    m->err, m->feat, m->labels, m->perm, m->ss};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (m->step_graph) cudaGraphExecDestroy(m->step_graph);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

const char *rv_mlp_last_error(const rv_mlp *m) { return m ? m->msg.c_str() : "null model"; }

rv_status rv_mlp_set_params(rv_mlp *m, const float *params) {
    if (!m || !params) return RV_ERR_ARG;
    MCUDA(cudaSetDevice(m->device));
    std::vector<float> p(params, params + N_PARAM);
    for (int o = 0; o < H; o++)
        for (int c = NF; c < KIN; c++) p[OFF_W1 + o * KIN + c] = 0.f;
    MCUDA(cudaMemcpyAsync(m->params, p.data(), N_PARAM * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    k_cast<<<64, 256, 0, m->stream>>>(m->params, m->w1, m->w2, m->w3, m->w2t, m->w3t);
    MCUDA(cudaGetLastError());
    MCUDA(cudaStreamSynchronize(m->stream));
    return RV_OK;
}

rv_status rv_mlp_get_params(rv_mlp *m, float *params) {
    if (!m || !params) return RV_ERR_ARG;
    MCUDA(cudaSetDevice(m->device));
    MCUDA(cudaMemcpy(params, m->params, N_PARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return RV_OK;
}

rv_status rv_mlp_gradients(rv_mlp *m, const float *features, const float *labels, int64_t n, float pos_weight,
                           float *grad, float *loss) {
    if (!m || !features || !labels || n <= 0 || n > m->B || !grad) return RV_ERR_ARG;
    MCUDA(cudaSetDevice(m->device));
    rv_status s = ensure_data(m, n);
    if (s) return s;
    MCUDA(cudaMemcpyAsync(m->feat, features, (size_t)n * NF * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaMemcpyAsync(m->labels, labels, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
    const int B = m->B;
    k_gather<<<256, 256, 0, m->stream>>>(m->feat, nullptr, n, 0, B, m->h0, m->h0t, m->y, m->labels, nullptr);
    MCUDA(forward(m, B));
    MCUDA(cudaMemsetAsync(m->grad, 0, N_PARAM * sizeof(float), m->stream));
    // the same sequence as a training step, without the optimizer
    k_head<<<B / 128, 128, 0, m->stream>>>(m->h[2], m->z[2], m->params, B, m->y, pos_weight, 1.f / (float)n,
                                           m->logit, m->dz[2], m->dzt[2], m->grad, m->loss);
    const int kper = std::min(B, 512), ks = B / kper;
    const bf16 *hprev_t[3] = {m->h0t, m->ht[0], m->ht[1]};
    const int off_w[3] = {OFF_W1, OFF_W2, OFF_W3};
    const int off_b[3] = {OFF_B1, OFF_B2, OFF_B3};
    const bf16 *wt[3] = {nullptr, m->w2t, m->w3t};
    for (int l = 2; l >= 0; l--) {
        Epi e{};
        e.dw = m->grad + off_w[l];
        e.err = m->err;
        if (l == 0) MCUDA((gemm<KIN, EPI_DW>(m, m->dzt[0], B, hprev_t[0], B, 1, ks, kper, e)));
        else MCUDA((gemm<H, EPI_DW>(m, m->dzt[l], B, hprev_t[l], B, 1, ks, kper, e)));
        if (l == 0) break;
        Epi d{};
        d.z = m->z[l - 1];
        d.h = m->dz[l - 1];
        d.ht = m->dzt[l - 1];
        d.ldt = B;
        d.db = m->grad + off_b[l - 1];
        d.err = m->err;
        MCUDA((gemm<H, EPI_DH>(m, m->dz[l], H, wt[l], H, B / kTileM, 1, H, d)));
    }
    if ((s = check_err(m))) return s;
    MCUDA(cudaMemcpy(grad, m->grad, N_PARAM * sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) MCUDA(cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    return RV_OK;
}

rv_status rv_mlp_train(rv_mlp *m, const float *features, const float *labels, int64_t n, int epochs, float lr,
                       float pos_weight, uint64_t seed, float *epoch_loss) {
    if (!m || !features || !labels || n <= 0 || n > INT32_MAX || epochs <= 0) return RV_ERR_ARG;
    MCUDA(cudaSetDevice(m->device));
    rv_status s = ensure_data(m, n);
    if (s) return s;
    MCUDA(cudaMemcpyAsync(m->feat, features, (size_t)n * NF * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaMemcpyAsync(m->labels, labels, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    const int B = m->B;
    // one step captured as a graph (re-captured when the set size or the
    // hyper-parameters change), replayed once per batch
    if (!m->step_graph || m->graph_n != n || m->graph_lr != lr || m->graph_pw != pos_weight) {
        if (m->step_graph) cudaGraphExecDestroy(m->step_graph);
        m->step_graph = nullptr;
        cudaGraph_t g = nullptr;
        MCUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t x = train_step(m, B, n, pos_weight, lr);
        cudaError_t y = cudaStreamEndCapture(m->stream, &g);
        if (x != cudaSuccess || y != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            m->msg = std::string("step capture: ") + cudaGetErrorString(x != cudaSuccess ? x : y);
            return RV_ERR_CUDA;
        }
        x = cudaGraphInstantiate(&m->step_graph, g, 0);
        cudaGraphDestroy(g);
        if (x != cudaSuccess) { m->msg = cudaGetErrorString(x); return RV_ERR_CUDA; }
        m->graph_n = n;
        m->graph_lr = lr;
        m->graph_pw = pos_weight;
    }
    std::vector<int32_t> perm((size_t)n);
    std::mt19937_64 rng(seed);
    cudaEvent_t e0, e1;
    MCUDA(cudaEventCreate(&e0));
    MCUDA(cudaEventCreate(&e1));
    int64_t total_steps = 0;
    float total_ms = 0;
    for (int ep = 0; ep < epochs; ep++) {
        for (int64_t i = 0; i < n; i++) perm[i] = (int32_t)i;
        for (int64_t i = n - 1; i > 0; i--) std::swap(perm[i], perm[rng() % (uint64_t)(i + 1)]);
        MCUDA(cudaMemcpyAsync(m->perm, perm.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice,
                              m->stream));
        MCUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
        // batch index back to 0; the Adam step count carries on
        MCUDA(cudaMemsetAsync(&m->ss->batch, 0, sizeof(int64_t), m->stream));
        int64_t nb = (n + B - 1) / B;
        MCUDA(cudaEventRecord(e0, m->stream));
        for (int64_t b = 0; b < nb; b++) MCUDA(cudaGraphLaunch(m->step_graph, m->stream));
        MCUDA(cudaEventRecord(e1, m->stream));
        m->steps += nb;
        if ((s = check_err(m))) return s;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
        total_steps += nb;
        float l = 0;
        MCUDA(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
        if (epoch_loss) epoch_loss[ep] = l / (float)nb;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m->step_ms = total_steps ? total_ms / total_steps : 0;
    return RV_OK;
}

rv_status rv_mlp_step_ms(const rv_mlp *m, double *ms) {
    if (!m || !ms) return RV_ERR_ARG;
    *ms = m->step_ms;
    return RV_OK;
}

rv_status rv_mlp_predict(rv_mlp *m, const float *features, int64_t n, float *scores) {
    if (!m || !features || n < 0 || (n > 0 && !scores)) return RV_ERR_ARG;
    if (n == 0) return RV_OK;
    MCUDA(cudaSetDevice(m->device));
    rv_status s = ensure_data(m, n);
    if (s) return s;
    MCUDA(cudaMemcpyAsync(m->feat, features, (size_t)n * NF * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    const int B = m->B;
    std::vector<float> out((size_t)B);
    for (int64_t b0 = 0; b0 < n; b0 += B) {
        const int64_t rows = std::min<int64_t>(B, n - b0);
        k_gather<<<256, 256, 0, m->stream>>>(m->feat, nullptr, n, b0, B, m->h0, m->h0t, nullptr, nullptr, nullptr);
        MCUDA(forward(m, B));
        k_head<<<B / 128, 128, 0, m->stream>>>(m->h[2], m->z[2], m->params, B, nullptr, 1.f, 0.f, m->logit, nullptr,
                                               nullptr, nullptr, nullptr);
        k_logistic<<<(B + 255) / 256, 256, 0, m->stream>>>(m->logit, B, m->logit);
        MCUDA(cudaGetLastError());
        MCUDA(cudaMemcpyAsync(scores + b0, m->logit, (size_t)rows * sizeof(float), cudaMemcpyDeviceToHost,
                              m->stream));
    }
    return check_err(m);
}

}  // extern "C"
