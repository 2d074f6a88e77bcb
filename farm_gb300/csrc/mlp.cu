// Learned scorer: a 520 -> 256 -> 256 -> 1 MLP (GELU; BF16 weights and
// activations on the tensor cores, FP32 accumulate), trained and run on the
// GPU with the hand-written tcgen05 GEMM of tc_gemm.cuh. It replaces the
// reference's "-a" fill-ratio confidence heuristic (query_intersect.cu:100-134):
// pairs it is sure about are decided by it, the rest go to exact refinement.
//
// Features per candidate pair (520, padded to 576 for the GEMM's K tiles):
//  * both polygons' fill classes resampled to 16 x 16 cells over the pair's
//    MBR-intersection window (cell centre -> that polygon's pixel), scaled to
//    [0, 1] and quantised to 4 bits (512 values);
//  * 8 MBR/size features: log MBR areas, window / MBR area ratios, log vertex
//    counts, log pixel counts.
//
// Training: binary cross-entropy on exact-refinement labels, Adam, mini-batches
// of 128-row multiples. Backward GEMMs run on the same kernel with transposed
// bf16 operands (dW = dZ^T x input, dH = dZ x W).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "tc_gemm.cuh"

namespace farm {

constexpr int kIn = 520, kInPad = 576, kHid = 256;

struct Mlp {
    // tensor-core copies (bf16) and FP32 masters
    DevBuf W1, W2, W2T;            // bf16 [256 x 576], [256 x 256], transpose of W2
    DevBuf mW1, mW2, b1, b2, w3;   // fp32 masters; w3 holds 256 weights then b3
    DevBuf adam;                   // fp32 moments for every parameter (m, v)
    uint64_t step = 0;
    float lo = 0.02f, hi = 0.98f;  // abstain band for the learned mode
    float lambda = 0.f;            // cost-aware band: also decide when min(p, 1-p) <= lambda x cost
    bool ready = false;
    // scratch
    DevBuf X, Z1, H1, Z2, H2, logit, dlogit, dZ2, dZ1, T1, T2, T3, gW1, gW2, gb, err;
};

static uint64_t n_params() { return (uint64_t)kHid * kInPad + kHid * kHid + kHid + kHid + kHid + 1; }

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

struct EpiStoreF32 {
    float *C;
    int ldc;
    __device__ void operator()(int row, int col0, const float *v) const {
        float *c = C + (size_t)row * ldc + col0;
#pragma unroll
        for (int i = 0; i < 16; i++) c[i] = v[i];
    }
};

// z = acc + bias; keep z (fp32) and GELU(z) (bf16)
struct EpiBiasGelu {
    const float *bias;
    float *Z;
    __nv_bfloat16 *H;
    int ld;
    __device__ void operator()(int row, int col0, const float *v) const {
#pragma unroll
        for (int i = 0; i < 16; i++) {
            float z = v[i] + bias[col0 + i];
            Z[(size_t)row * ld + col0 + i] = z;
            H[(size_t)row * ld + col0 + i] = __float2bfloat16_rn(gelu(z));
        }
    }
};

// dZ = acc * GELU'(Z) (bf16), bias gradient accumulated per column
struct EpiGeluGrad {
    const float *Z;
    __nv_bfloat16 *dZ;
    float *db;
    int ld;
    __device__ void operator()(int row, int col0, const float *v) const {
#pragma unroll
        for (int i = 0; i < 16; i++) {
            float d = v[i] * gelu_grad(Z[(size_t)row * ld + col0 + i]);
            dZ[(size_t)row * ld + col0 + i] = __float2bfloat16_rn(d);
            atomicAdd(&db[col0 + i], d);
        }
    }
};

template <int BN, typename Epi>
__global__ void __launch_bounds__(tc::kThreads) k_gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B,
                                                       int ldb, int M, int N, int K, int *err, Epi epi) {
    extern __shared__ __align__(1024) unsigned char smem[];
    tc::gemm_tile<BN>(A, lda, B, ldb, M, N, K, blockIdx.x * tc::kBM, blockIdx.y * BN, smem, err, epi);
}

template <int BN, typename Epi>
static int launch_gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                       int *err, Epi epi, cudaStream_t st) {
    constexpr int smem = tc::smem_bytes<BN>();
    static bool attr = false;
    if (!attr) {
        FARM_CUDA(cudaFuncSetAttribute(k_gemm<BN, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    dim3 grid((M + tc::kBM - 1) / tc::kBM, (N + BN - 1) / BN);
    k_gemm<BN, Epi><<<grid, tc::kThreads, smem, st>>>(A, lda, B, ldb, M, N, K, err, epi);
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

// ------------------------------------------------------------ features --

__device__ __forceinline__ float sample_class(const StoreView &sv, const PolyHdr &h, double x, double y, int cc) {
    if (x < h.mbr[0] || x > h.mbr[2] || y < h.mbr[1] || y > h.mbr[3]) return 0.f;
    int px = offset_x(h.mbr, h.step_x, h.dimx, x), py = offset_y(h.mbr, h.step_y, h.dimy, y);
    uint8_t s = sv.status[h.st + (uint32_t)(py * h.dimx + px)];
    // 4-bit quantisation of the fill ratio (w = 4)
    float r = (float)s / (float)(cc - 1);
    return rintf(r * 15.f) / 15.f;
}

// one warp per pair; rows >= n are zero padding
__global__ void k_features(const StoreView sv, const uint32_t *__restrict__ pairs, uint64_t n, uint64_t rows,
                           uint64_t tgt_base, __nv_bfloat16 *__restrict__ X) {
    const int lane = threadIdx.x & 31;
    const int cc = sv.category_count;
    uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = w; r < rows; r += nw) {
        __nv_bfloat16 *x = X + r * kInPad;
        if (r >= n) {
            for (int k = lane; k < kInPad; k += 32) x[k] = __float2bfloat16_rn(0.f);
            continue;
        }
        const PolyHdr &S = sv.hdr[pairs[2 * r]];
        const PolyHdr &T = sv.hdr[tgt_base + pairs[2 * r + 1]];
        double wx0 = fmax(S.mbr[0], T.mbr[0]), wy0 = fmax(S.mbr[1], T.mbr[1]);
        double wx1 = fmin(S.mbr[2], T.mbr[2]), wy1 = fmin(S.mbr[3], T.mbr[3]);
        if (wx1 < wx0) wx1 = wx0;
        if (wy1 < wy0) wy1 = wy0;
        for (int c = lane; c < 256; c += 32) {
            int gx = c & 15, gy = c >> 4;
            double cx = wx0 + (gx + 0.5) * (wx1 - wx0) / 16.0, cy = wy0 + (gy + 0.5) * (wy1 - wy0) / 16.0;
            x[c] = __float2bfloat16_rn(S.err ? 0.f : sample_class(sv, S, cx, cy, cc));
            x[256 + c] = __float2bfloat16_rn(T.err ? 0.f : sample_class(sv, T, cx, cy, cc));
        }
        if (lane < 8) {
            double as = (S.mbr[2] - S.mbr[0]) * (S.mbr[3] - S.mbr[1]);
            double at = (T.mbr[2] - T.mbr[0]) * (T.mbr[3] - T.mbr[1]);
            double aw = (wx1 - wx0) * (wy1 - wy0);
            double f = 0;
            switch (lane) {
                case 0: f = log(as + 1e-12) / 10.0; break;
                case 1: f = log(at + 1e-12) / 10.0; break;
                case 2: f = aw / (as + 1e-30); break;
                case 3: f = aw / (at + 1e-30); break;
                case 4: f = log((double)S.nv) / 10.0; break;
                case 5: f = log((double)T.nv) / 10.0; break;
                case 6: f = log((double)S.P + 1.0) / 10.0; break;
                default: f = log((double)T.P + 1.0) / 10.0; break;
            }
            x[512 + lane] = __float2bfloat16_rn((float)f);
        }
        for (int k = kIn + lane; k < kInPad; k += 32) x[k] = __float2bfloat16_rn(0.f);
    }
}

// ------------------------------------------------- elementwise kernels --

// logit[r] = H2[r] . w3 + b3 (warp per row)
__global__ void k_logit(const __nv_bfloat16 *__restrict__ H2, const float *__restrict__ w3, uint64_t rows,
                        float *__restrict__ logit) {
    const int lane = threadIdx.x & 31;
    uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = w; r < rows; r += nw) {
        float s = 0;
        for (int j = lane; j < kHid; j += 32) s += __bfloat162float(H2[r * kHid + j]) * w3[j];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) logit[r] = s + w3[kHid];
    }
}

// BCE with logits: dlogit = (sigmoid - y) / n; dw3 += dlogit * H2; loss sum.
// Rows >= n (padding) get zero gradient.
__global__ void k_bce(const float *__restrict__ logit, const uint8_t *__restrict__ y, uint64_t n, uint64_t rows,
                      const __nv_bfloat16 *__restrict__ H2, float *__restrict__ dlogit, float *__restrict__ dw3,
                      float *__restrict__ db3, float *__restrict__ loss) {
    const int lane = threadIdx.x & 31;
    uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = w; r < rows; r += nw) {
        float d = 0;
        if (r < n) {
            float z = logit[r], t = (float)y[r];
            float p = 1.f / (1.f + expf(-z));
            d = (p - t) / (float)n;
            if (lane == 0) {
                float l = fmaxf(z, 0.f) - z * t + log1pf(expf(-fabsf(z)));
                atomicAdd(loss, l / (float)n);
                atomicAdd(db3, d);
            }
        }
        if (lane == 0) dlogit[r] = d;
        if (d != 0)
            for (int j = lane; j < kHid; j += 32) atomicAdd(&dw3[j], d * __bfloat162float(H2[r * kHid + j]));
    }
}

// dZ2 = dlogit * w3 * GELU'(Z2) (bf16), db2 column sums
__global__ void k_dz2(const float *__restrict__ dlogit, const float *__restrict__ w3, const float *__restrict__ Z2,
                      uint64_t rows, __nv_bfloat16 *__restrict__ dZ2, float *__restrict__ db2) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < rows * kHid;
         k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t r = k / kHid;
        int j = (int)(k % kHid);
        float d = dlogit[r] * w3[j] * gelu_grad(Z2[k]);
        dZ2[k] = __float2bfloat16_rn(d);
        if (d != 0) atomicAdd(&db2[j], d);
    }
}

// dst[c][r] = src[r][c] for a [R x C] bf16 matrix, 32 x 32 tiles via shared memory
__global__ void k_transpose(const __nv_bfloat16 *__restrict__ src, uint64_t R, uint64_t Cc,
                            __nv_bfloat16 *__restrict__ dst) {
    __shared__ __nv_bfloat16 tile[32][33];
    uint64_t bx = blockIdx.x * 32ull, by = blockIdx.y * 32ull;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        uint64_t r = by + i, c = bx + threadIdx.x;
        tile[i][threadIdx.x] = (r < R && c < Cc) ? src[r * Cc + c] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        uint64_t c = bx + i, r = by + threadIdx.x;
        if (c < Cc && r < R) dst[c * R + r] = tile[threadIdx.x][i];
    }
}

__global__ void k_to_bf16(const float *__restrict__ a, uint64_t n, __nv_bfloat16 *__restrict__ b) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        b[k] = __float2bfloat16_rn(a[k]);
}

// Adam (beta1 0.9, beta2 0.999); grad scaled by gscale
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, uint64_t n, float lr, float bc1, float bc2) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        float gk = g[k];
        float mk = 0.9f * m[k] + 0.1f * gk, vk = 0.999f * v[k] + 0.001f * gk * gk;
        m[k] = mk;
        v[k] = vk;
        p[k] -= lr * (mk / bc1) / (sqrtf(vk / bc2) + 1e-8f);
    }
}

// deterministic small-scale uniform init in [-a, a]
__global__ void k_init(float *__restrict__ p, uint64_t n, float a, uint64_t seed) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed * 0x9E3779B97F4A7C15ull + k;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        p[k] = a * (2.f * ((float)(z >> 40) / 16777216.f) - 1.f);
    }
}

__global__ void k_sigmoid(const float *__restrict__ l, uint64_t n, float *__restrict__ p) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        p[k] = 1.f / (1.f + expf(-l[k]));
}

__global__ void k_gather_rows(const __nv_bfloat16 *__restrict__ X, const uint32_t *__restrict__ idx, uint64_t n,
                              uint64_t rows, const uint8_t *__restrict__ yin, __nv_bfloat16 *__restrict__ out,
                              uint8_t *__restrict__ yout) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < rows * kInPad;
         k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t r = k / kInPad, c = k % kInPad;
        out[k] = r < n ? X[(uint64_t)idx[r] * kInPad + c] : __float2bfloat16_rn(0.f);
        if (c == 0) yout[r] = r < n ? yin[idx[r]] : 0;
    }
}

static unsigned gbm(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    uint64_t cap = 64ull * sm_count();
    if (g > cap) g = cap;
    return (unsigned)(g ? g : 1);
}

void mlp_free(void *p) {
    Mlp *m = static_cast<Mlp *>(p);
    if (!m) return;
    DevBuf *b[] = {&m->W1, &m->W2, &m->W2T, &m->mW1, &m->mW2, &m->b1, &m->b2, &m->w3, &m->adam, &m->X, &m->Z1,
                   &m->H1, &m->Z2, &m->H2, &m->logit, &m->dlogit, &m->dZ2, &m->dZ1, &m->T1, &m->T2, &m->T3,
                   &m->gW1, &m->gW2, &m->gb, &m->err};
    for (DevBuf *x : b) x->release();
    delete m;
}

float mlp_band(farm_store *s, int which) {
    Mlp *m = static_cast<Mlp *>(s->mlp);
    return m ? (which == 2 ? m->lambda : (which ? m->hi : m->lo)) : 0.f;
}

static Mlp *mlp_of(farm_store *s) {
    if (!s->mlp) s->mlp = new Mlp();
    return static_cast<Mlp *>(s->mlp);
}

static int mlp_alloc(Mlp *m) {
    FARM_TRY(m->W1.ensure(2ull * kHid * kInPad));
    FARM_TRY(m->W2.ensure(2ull * kHid * kHid));
    FARM_TRY(m->W2T.ensure(2ull * kHid * kHid));
    FARM_TRY(m->mW1.ensure(4ull * kHid * kInPad));
    FARM_TRY(m->mW2.ensure(4ull * kHid * kHid));
    FARM_TRY(m->b1.ensure(4 * kHid));
    FARM_TRY(m->b2.ensure(4 * kHid));
    FARM_TRY(m->w3.ensure(4 * (kHid + 1)));
    FARM_TRY(m->adam.ensure(8 * n_params()));
    FARM_TRY(m->err.ensure(64));
    return FARM_OK;
}

// refresh the bf16 copies from the masters
static int mlp_sync_bf16(Mlp *m, cudaStream_t st) {
    k_to_bf16<<<gbm(kHid * kInPad), 256, 0, st>>>(m->mW1.as<float>(), (uint64_t)kHid * kInPad,
                                                  m->W1.as<__nv_bfloat16>());
    k_to_bf16<<<gbm(kHid * kHid), 256, 0, st>>>(m->mW2.as<float>(), (uint64_t)kHid * kHid, m->W2.as<__nv_bfloat16>());
    dim3 tb(32, 8), tg(kHid / 32, kHid / 32);
    k_transpose<<<tg, tb, 0, st>>>(m->W2.as<__nv_bfloat16>(), kHid, kHid, m->W2T.as<__nv_bfloat16>());
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

// forward over `rows` (multiple of 128) feature rows already in m->X
static int mlp_forward(Mlp *m, uint64_t rows, cudaStream_t st) {
    FARM_TRY(m->Z1.ensure(4 * rows * kHid));
    FARM_TRY(m->H1.ensure(2 * rows * kHid));
    FARM_TRY(m->Z2.ensure(4 * rows * kHid));
    FARM_TRY(m->H2.ensure(2 * rows * kHid));
    FARM_TRY(m->logit.ensure(4 * rows + 64));
    int *err = m->err.as<int>();
    EpiBiasGelu e1{m->b1.as<float>(), m->Z1.as<float>(), m->H1.as<__nv_bfloat16>(), kHid};
    FARM_TRY(launch_gemm<256>(m->X.as<__nv_bfloat16>(), kInPad, m->W1.as<__nv_bfloat16>(), kInPad, (int)rows, kHid,
                              kInPad, err, e1, st));
    EpiBiasGelu e2{m->b2.as<float>(), m->Z2.as<float>(), m->H2.as<__nv_bfloat16>(), kHid};
    FARM_TRY(launch_gemm<256>(m->H1.as<__nv_bfloat16>(), kHid, m->W2.as<__nv_bfloat16>(), kHid, (int)rows, kHid, kHid,
                              err, e2, st));
    k_logit<<<gbm(32 * rows), 256, 0, st>>>(m->H2.as<__nv_bfloat16>(), m->w3.as<float>(), rows,
                                            m->logit.as<float>());
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

// gradients into m->gW1, m->gW2, m->gb (b1 | b2 | w3 | b3), loss into *loss (device)
static int mlp_backward(Mlp *m, const uint8_t *y, uint64_t n, uint64_t rows, float *dloss, cudaStream_t st) {
    FARM_TRY(m->dlogit.ensure(4 * rows + 64));
    FARM_TRY(m->dZ2.ensure(2 * rows * kHid));
    FARM_TRY(m->dZ1.ensure(2 * rows * kHid));
    FARM_TRY(m->T1.ensure(2 * rows * kHid));
    FARM_TRY(m->T2.ensure(2 * rows * kHid));
    FARM_TRY(m->T3.ensure(2 * rows * kInPad));
    FARM_TRY(m->gW1.ensure(4ull * kHid * kInPad));
    FARM_TRY(m->gW2.ensure(4ull * kHid * kHid));
    FARM_TRY(m->gb.ensure(4ull * (3 * kHid + 1) + 64));
    float *gb = m->gb.as<float>();
    float *db1 = gb, *db2 = gb + kHid, *dw3 = gb + 2 * kHid, *db3 = gb + 3 * kHid;
    FARM_CUDA(cudaMemsetAsync(gb, 0, 4ull * (3 * kHid + 1), st));
    int *err = m->err.as<int>();
    k_bce<<<gbm(32 * rows), 256, 0, st>>>(m->logit.as<float>(), y, n, rows, m->H2.as<__nv_bfloat16>(),
                                          m->dlogit.as<float>(), dw3, db3, dloss);
    k_dz2<<<gbm(rows * kHid), 256, 0, st>>>(m->dlogit.as<float>(), m->w3.as<float>(), m->Z2.as<float>(), rows,
                                            m->dZ2.as<__nv_bfloat16>(), db2);
    // dW2 = dZ2^T x H1 : A = dZ2^T [256 x rows], B = H1^T [256 x rows]
    dim3 tb(32, 8);
    dim3 tg1(kHid / 32, (unsigned)((rows + 31) / 32));
    k_transpose<<<tg1, tb, 0, st>>>(m->dZ2.as<__nv_bfloat16>(), rows, kHid, m->T1.as<__nv_bfloat16>());
    k_transpose<<<tg1, tb, 0, st>>>(m->H1.as<__nv_bfloat16>(), rows, kHid, m->T2.as<__nv_bfloat16>());
    FARM_TRY(launch_gemm<256>(m->T1.as<__nv_bfloat16>(), (int)rows, m->T2.as<__nv_bfloat16>(), (int)rows, kHid, kHid,
                              (int)rows, err, EpiStoreF32{m->gW2.as<float>(), kHid}, st));
    // dH1 = dZ2 x W2 -> dZ1 = dH1 * GELU'(Z1) : A = dZ2 [rows x 256], B = W2^T [256 x 256]
    EpiGeluGrad eg{m->Z1.as<float>(), m->dZ1.as<__nv_bfloat16>(), db1, kHid};
    FARM_TRY(launch_gemm<256>(m->dZ2.as<__nv_bfloat16>(), kHid, m->W2T.as<__nv_bfloat16>(), kHid, (int)rows, kHid,
                              kHid, err, eg, st));
    // dW1 = dZ1^T x X : A = dZ1^T [256 x rows], B = X^T [576 x rows]
    k_transpose<<<tg1, tb, 0, st>>>(m->dZ1.as<__nv_bfloat16>(), rows, kHid, m->T1.as<__nv_bfloat16>());
    dim3 tg2(kInPad / 32, (unsigned)((rows + 31) / 32));
    k_transpose<<<tg2, tb, 0, st>>>(m->X.as<__nv_bfloat16>(), rows, kInPad, m->T3.as<__nv_bfloat16>());
    FARM_TRY(launch_gemm<256>(m->T1.as<__nv_bfloat16>(), (int)rows, m->T3.as<__nv_bfloat16>(), (int)rows, kHid,
                              kInPad, (int)rows, err, EpiStoreF32{m->gW1.as<float>(), kInPad}, st));
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

static int mlp_adam(Mlp *m, float lr, cudaStream_t st) {
    m->step++;
    float bc1 = 1.f - powf(0.9f, (float)m->step), bc2 = 1.f - powf(0.999f, (float)m->step);
    float *am = m->adam.as<float>(), *av = am + n_params();
    uint64_t o = 0;
    auto upd = [&](float *p, const float *g, uint64_t n) {
        k_adam<<<gbm(n), 256, 0, st>>>(p, g, am + o, av + o, n, lr, bc1, bc2);
        o += n;
    };
    const float *gb = m->gb.as<float>();
    upd(m->mW1.as<float>(), m->gW1.as<float>(), (uint64_t)kHid * kInPad);
    upd(m->mW2.as<float>(), m->gW2.as<float>(), (uint64_t)kHid * kHid);
    upd(m->b1.as<float>(), gb, kHid);
    upd(m->b2.as<float>(), gb + kHid, kHid);
    upd(m->w3.as<float>(), gb + 2 * kHid, kHid + 1);  // w3 and b3
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

static int check_err(Mlp *m, cudaStream_t st) {
    int h = 0;
    FARM_CUDA(cudaMemcpyAsync(&h, m->err.p, 4, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error("tcgen05 GEMM: an mbarrier wait timed out");
        return FARM_ETIMEOUT;
    }
    return FARM_OK;
}

static uint64_t pad128(uint64_t n) { return (n + 127) & ~127ull; }

}  // namespace farm

using namespace farm;

extern "C" {

/* Test hook of the tcgen05 GEMM (see farm_gpu.h). */
int farm_tc_gemm_test(const void *A, const void *B, float *C, int M, int N, int K, int BN) {
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || M % 16 || N % 16 || K % 64) {
        set_error("farm_tc_gemm_test: bad shape");
        return FARM_EINVAL;
    }
    int *err = nullptr;
    FARM_CUDA(cudaMalloc(&err, 4));
    FARM_CUDA(cudaMemset(err, 0, 4));
    const __nv_bfloat16 *a = static_cast<const __nv_bfloat16 *>(A), *b = static_cast<const __nv_bfloat16 *>(B);
    EpiStoreF32 epi{C, N};
    int rc;
    if (BN == 64)
        rc = launch_gemm<64>(a, K, b, K, M, N, K, err, epi, 0);
    else if (BN == 128)
        rc = launch_gemm<128>(a, K, b, K, M, N, K, err, epi, 0);
    else
        rc = launch_gemm<256>(a, K, b, K, M, N, K, err, epi, 0);
    int herr = 0;
    if (rc == FARM_OK) {
        cudaError_t e = cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "farm_tc_gemm_test");
    }
    cudaFree(err);
    if (rc == FARM_OK && herr) {
        set_error("farm_tc_gemm_test: an mbarrier wait timed out");
        return FARM_ETIMEOUT;
    }
    return rc;
}

int farm_mlp_init(farm_store *s, uint64_t seed) {
    if (!s) return FARM_EINVAL;
    Mlp *m = mlp_of(s);
    FARM_TRY(mlp_alloc(m));
    cudaStream_t st = s->stream;
    float a1 = sqrtf(6.f / (kIn + kHid)), a2 = sqrtf(6.f / (2 * kHid)), a3 = sqrtf(6.f / (kHid + 1));
    k_init<<<gbm(kHid * kInPad), 256, 0, st>>>(m->mW1.as<float>(), (uint64_t)kHid * kInPad, a1, seed * 4 + 1);
    k_init<<<gbm(kHid * kHid), 256, 0, st>>>(m->mW2.as<float>(), (uint64_t)kHid * kHid, a2, seed * 4 + 2);
    k_init<<<gbm(kHid), 256, 0, st>>>(m->w3.as<float>(), kHid, a3, seed * 4 + 3);
    FARM_CUDA(cudaMemsetAsync(m->w3.as<float>() + kHid, 0, 4, st));
    FARM_CUDA(cudaMemsetAsync(m->b1.p, 0, 4 * kHid, st));
    FARM_CUDA(cudaMemsetAsync(m->b2.p, 0, 4 * kHid, st));
    FARM_CUDA(cudaMemsetAsync(m->adam.p, 0, 8 * n_params(), st));
    m->step = 0;
    FARM_TRY(mlp_sync_bf16(m, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    m->ready = true;
    s->launches += 6;
    return FARM_OK;
}

/* Features of n candidate pairs into X (device, bf16 [n_pad x 576]). */
int farm_mlp_features(farm_store *s, const uint32_t *d_pairs, uint64_t n, void *d_X, uint64_t rows) {
    if (!s || !s->rasterized || rows < n) return FARM_EINVAL;
    FARM_TRY(check_pairs(s, d_pairs, n, FARM_MEM_DEVICE, false, "farm_mlp_features"));
    k_features<<<gbm(32 * rows), 256, 0, s->stream>>>(s->view(), d_pairs, n, rows, s->n_side[0],
                                                      static_cast<__nv_bfloat16 *>(d_X));
    FARM_CUDA(cudaGetLastError());
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    s->launches++;
    return FARM_OK;
}

/* One forward + backward on given features (device bf16 [rows x 576], rows a
 * multiple of 128) and labels (device u8, first n rows): loss and gradients in
 * the layout of farm_mlp_get (W1 | W2 | b1 | b2 | w3 | b3), no update. */
int farm_mlp_grad(farm_store *s, const void *d_X, const uint8_t *d_y, uint64_t n, uint64_t rows, float *h_loss,
                  float *h_grad) {
    if (!s || !s->mlp || rows % 128 || rows < n) return FARM_EINVAL;
    Mlp *m = mlp_of(s);
    cudaStream_t st = s->stream;
    FARM_TRY(m->X.ensure(2 * rows * kInPad));
    FARM_CUDA(cudaMemcpyAsync(m->X.p, d_X, 2 * rows * kInPad, cudaMemcpyDeviceToDevice, st));
    FARM_CUDA(cudaMemsetAsync(m->err.p, 0, 4, st));
    float *dloss;
    FARM_TRY(s->d_counters.ensure(256));
    dloss = s->d_counters.as<float>();
    FARM_CUDA(cudaMemsetAsync(dloss, 0, 4, st));
    FARM_TRY(mlp_forward(m, rows, st));
    FARM_TRY(mlp_backward(m, d_y, n, rows, dloss, st));
    FARM_TRY(check_err(m, st));
    if (h_loss) FARM_CUDA(cudaMemcpy(h_loss, dloss, 4, cudaMemcpyDeviceToHost));
    if (h_grad) {
        float *o = h_grad;
        FARM_CUDA(cudaMemcpy(o, m->gW1.p, 4ull * kHid * kInPad, cudaMemcpyDeviceToHost));
        o += (uint64_t)kHid * kInPad;
        FARM_CUDA(cudaMemcpy(o, m->gW2.p, 4ull * kHid * kHid, cudaMemcpyDeviceToHost));
        o += (uint64_t)kHid * kHid;
        FARM_CUDA(cudaMemcpy(o, m->gb.p, 4ull * (3 * kHid + 1), cudaMemcpyDeviceToHost));
    }
    return FARM_OK;
}

uint64_t farm_mlp_param_count(void) { return n_params(); }

/* Decision band of the learned mode: probability >= hi decides 1, <= lo
 * decides 0, anything between goes to exact refinement. */
int farm_mlp_set_band(farm_store *s, float lo, float hi) {
    if (!s || !(lo <= hi) || !isfinite(lo) || !isfinite(hi)) {
        set_error("farm_mlp_set_band: need finite lo <= hi");
        return FARM_EINVAL;
    }
    Mlp *m = mlp_of(s);
    m->lo = lo;
    m->hi = hi;
    return FARM_OK;
}

int farm_mlp_set_band_cost(farm_store *s, float lambda) {
    if (!s || !(lambda >= 0.f) || !isfinite(lambda)) {
        set_error("farm_mlp_set_band_cost: need a finite lambda >= 0");
        return FARM_EINVAL;
    }
    mlp_of(s)->lambda = lambda;
    return FARM_OK;
}

/* Copy the FP32 master parameters out / in (W1 [256 x 576] | W2 [256 x 256] |
 * b1 | b2 | w3 | b3). */
int farm_mlp_get(farm_store *s, float *out) {
    if (!s || !s->mlp || !out) return FARM_EINVAL;
    Mlp *m = mlp_of(s);
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    float *o = out;
    FARM_CUDA(cudaMemcpy(o, m->mW1.p, 4ull * kHid * kInPad, cudaMemcpyDeviceToHost));
    o += (uint64_t)kHid * kInPad;
    FARM_CUDA(cudaMemcpy(o, m->mW2.p, 4ull * kHid * kHid, cudaMemcpyDeviceToHost));
    o += (uint64_t)kHid * kHid;
    FARM_CUDA(cudaMemcpy(o, m->b1.p, 4 * kHid, cudaMemcpyDeviceToHost));
    o += kHid;
    FARM_CUDA(cudaMemcpy(o, m->b2.p, 4 * kHid, cudaMemcpyDeviceToHost));
    o += kHid;
    FARM_CUDA(cudaMemcpy(o, m->w3.p, 4 * (kHid + 1), cudaMemcpyDeviceToHost));
    return FARM_OK;
}

int farm_mlp_set(farm_store *s, const float *in) {
    if (!s || !in) return FARM_EINVAL;
    Mlp *m = mlp_of(s);
    FARM_TRY(mlp_alloc(m));
    const float *o = in;
    FARM_CUDA(cudaMemcpy(m->mW1.p, o, 4ull * kHid * kInPad, cudaMemcpyHostToDevice));
    o += (uint64_t)kHid * kInPad;
    FARM_CUDA(cudaMemcpy(m->mW2.p, o, 4ull * kHid * kHid, cudaMemcpyHostToDevice));
    o += (uint64_t)kHid * kHid;
    FARM_CUDA(cudaMemcpy(m->b1.p, o, 4 * kHid, cudaMemcpyHostToDevice));
    o += kHid;
    FARM_CUDA(cudaMemcpy(m->b2.p, o, 4 * kHid, cudaMemcpyHostToDevice));
    o += kHid;
    FARM_CUDA(cudaMemcpy(m->w3.p, o, 4 * (kHid + 1), cudaMemcpyHostToDevice));
    FARM_CUDA(cudaMemset(m->adam.p, 0, 8 * n_params()));
    m->step = 0;
    FARM_TRY(mlp_sync_bf16(m, s->stream));
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    m->ready = true;
    return FARM_OK;
}

/* Train on n candidate pairs (device pairs, device u8 labels from exact
 * refinement): epochs x shuffled mini-batches of `batch` rows (multiple of
 * 128), Adam with learning rate lr. Returns the last epoch's mean loss. */
int farm_mlp_train(farm_store *s, const uint32_t *d_pairs, const uint8_t *d_labels, uint64_t n, int epochs,
                   int batch, float lr, uint64_t seed, float *last_loss) {
    if (!s || !s->rasterized || !d_pairs || !d_labels || n == 0 || batch <= 0 || batch % 128) return FARM_EINVAL;
    FARM_TRY(check_pairs(s, d_pairs, n, FARM_MEM_DEVICE, false, "farm_mlp_train"));
    Mlp *m = mlp_of(s);
    if (!m->ready) FARM_TRY(farm_mlp_init(s, seed));
    cudaStream_t st = s->stream;
    const uint64_t rows_all = pad128(n);
    DevBuf &Xall = s->s[Q_SCR0], &perm = s->s[Q_SCR1], &yb = s->s[Q_SCR2];
    FARM_TRY(Xall.ensure(2 * rows_all * kInPad));
    k_features<<<gbm(32 * rows_all), 256, 0, st>>>(s->view(), d_pairs, n, rows_all, s->n_side[0],
                                                   Xall.as<__nv_bfloat16>());
    FARM_TRY(m->X.ensure(2ull * batch * kInPad));
    FARM_TRY(yb.ensure((uint64_t)batch + 64));
    FARM_TRY(perm.ensure(4 * n));
    FARM_TRY(s->d_counters.ensure(256));
    float *dloss = s->d_counters.as<float>();
    FARM_CUDA(cudaMemsetAsync(m->err.p, 0, 4, st));
    std::vector<uint32_t> hp(n);
    uint64_t rng = seed * 0x9E3779B97F4A7C15ull + 12345;
    float loss = 0;
    for (int ep = 0; ep < epochs; ep++) {
        for (uint64_t i = 0; i < n; i++) hp[i] = (uint32_t)i;
        for (uint64_t i = n - 1; i > 0; i--) {  // Fisher-Yates with a splitmix stream
            rng += 0x9E3779B97F4A7C15ull;
            uint64_t z = rng;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            uint64_t j = z % (i + 1);
            uint32_t t = hp[i];
            hp[i] = hp[j];
            hp[j] = t;
        }
        FARM_CUDA(cudaMemcpyAsync(perm.p, hp.data(), 4 * n, cudaMemcpyHostToDevice, st));
        FARM_CUDA(cudaMemsetAsync(dloss, 0, 4, st));
        uint64_t nb = 0;
        for (uint64_t b0 = 0; b0 < n; b0 += (uint64_t)batch, nb++) {
            uint64_t nn = n - b0 < (uint64_t)batch ? n - b0 : (uint64_t)batch;
            uint64_t rows = pad128(nn);
            k_gather_rows<<<gbm(rows * kInPad), 256, 0, st>>>(Xall.as<__nv_bfloat16>(), perm.as<uint32_t>() + b0, nn,
                                                              rows, d_labels, m->X.as<__nv_bfloat16>(),
                                                              yb.as<uint8_t>());
            FARM_TRY(mlp_forward(m, rows, st));
            FARM_TRY(mlp_backward(m, yb.as<uint8_t>(), nn, rows, dloss, st));
            FARM_TRY(mlp_adam(m, lr, st));
            FARM_TRY(mlp_sync_bf16(m, st));
        }
        FARM_CUDA(cudaMemcpyAsync(&loss, dloss, 4, cudaMemcpyDeviceToHost, st));
        FARM_CUDA(cudaStreamSynchronize(st));
        loss /= (float)(nb ? nb : 1);
    }
    FARM_TRY(check_err(m, st));
    if (last_loss) *last_loss = loss;
    return FARM_OK;
}

/* Probabilities for n pairs (device pairs -> device fp32 out). */
int farm_mlp_predict(farm_store *s, const uint32_t *d_pairs, uint64_t n, float *d_prob) {
    if (!s || !s->mlp || !s->rasterized) return FARM_EINVAL;
    Mlp *m = mlp_of(s);
    if (!m->ready) {
        set_error("no trained scorer in this store");
        return FARM_EINVAL;
    }
    FARM_TRY(check_pairs(s, d_pairs, n, FARM_MEM_DEVICE, false, "farm_mlp_predict"));
    cudaStream_t st = s->stream;
    const uint64_t chunk = 1 << 16;
    FARM_CUDA(cudaMemsetAsync(m->err.p, 0, 4, st));
    for (uint64_t b0 = 0; b0 < n; b0 += chunk) {
        uint64_t nn = n - b0 < chunk ? n - b0 : chunk;
        uint64_t rows = pad128(nn);
        FARM_TRY(m->X.ensure(2 * rows * kInPad));
        k_features<<<gbm(32 * rows), 256, 0, st>>>(s->view(), d_pairs + 2 * b0, nn, rows, s->n_side[0],
                                                   m->X.as<__nv_bfloat16>());
        FARM_TRY(mlp_forward(m, rows, st));
        k_sigmoid<<<gbm(nn), 256, 0, st>>>(m->logit.as<float>(), nn, d_prob + b0);
        s->launches += 5;
    }
    FARM_TRY(check_err(m, st));
    return FARM_OK;
}

}  // extern "C"
