// The store's timing and launch-count helpers, and the issue-rate probe that
// gives the rooflines their FP64 / FP32 denominators.
#include "common.cuh"

using namespace farm;

namespace {

// Eight independent chains per thread of x = x * m + c as a separate multiply
// and add (round-to-nearest intrinsics: never contracted into an FMA), the
// instruction mix of the rasterizer's non-fused arithmetic. 2 ops per chain
// step. The result is stored only if it equals an impossible value, so the
// work cannot be dropped.
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

template <typename T>
__global__ void __launch_bounds__(256) k_issue_rate(T *out, T m, T c, int iters) {
    T x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = (T)(threadIdx.x + i) * (T)1e-3;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = add_rn(mul_rn(x[i], m), c);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s = add_rn(s, x[i]);
    if (s == (T)-12345.678) out[blockIdx.x] = s;
}

template <typename T>
int time_rate(int iters, double *ops_per_s) {
    const int blocks = 8 * sm_count(), threads = 256;
    T *d = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(T) * blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float best = 0;
    for (int rep = 0; e == cudaSuccess && rep < 4; rep++) {  // first launch warms up
        cudaEventRecord(a, 0);
        k_issue_rate<T><<<blocks, threads>>>(d, (T)0.999, (T)1e-4, iters);
        cudaEventRecord(b, 0);
        e = cudaEventSynchronize(b);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && (best == 0 || ms < best)) best = ms;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "farm_probe_issue_rates");
    *ops_per_s = (double)blocks * threads * iters * 8 * 2 / (best * 1e-3);
    return FARM_OK;
}

}  // namespace

extern "C" {

/* CUDA-event timing on the store's own stream: record slot, elapsed a -> b.
 * Slots 0-5 belong to the caller; the queries time themselves with 6 and 7. */
int farm_event_record(farm_store *s, int slot) {
    if (!s || slot < 0 || slot >= 6) {
        set_error("invalid event slot");
        return FARM_EINVAL;
    }
    FARM_CUDA(cudaEventRecord(s->ev[slot], s->stream));
    return FARM_OK;
}

int farm_event_elapsed(farm_store *s, int a, int b, double *ms) {
    if (!s || !ms || a < 0 || a >= 6 || b < 0 || b >= 6) {
        set_error("invalid event slot");
        return FARM_EINVAL;
    }
    FARM_CUDA(cudaEventSynchronize(s->ev[b]));
    float f = 0;
    FARM_CUDA(cudaEventElapsedTime(&f, s->ev[a], s->ev[b]));
    *ms = f;
    return FARM_OK;
}

/* Sustained non-fused FP64 and FP32 arithmetic rates of the current device
 * (operations per second, a multiply or an add each), measured with CUDA
 * events over a few launches of a throughput kernel: the denominators of the
 * FP64- and FP32-bound rooflines. Allocates a few bytes; takes ~0.1 s. */
int farm_probe_issue_rates(double *fp64_ops_per_s, double *fp32_ops_per_s) {
    if (!fp64_ops_per_s || !fp32_ops_per_s) {
        set_error("invalid arguments to farm_probe_issue_rates");
        return FARM_EINVAL;
    }
    FARM_TRY(time_rate<double>(4096, fp64_ops_per_s));
    FARM_TRY(time_rate<float>(65536, fp32_ops_per_s));
    return FARM_OK;
}

/* Engine kernels launched by this store since it was created. */
uint64_t farm_store_launches(farm_store *s) { return s ? s->launches : 0; }

}  // extern "C"
