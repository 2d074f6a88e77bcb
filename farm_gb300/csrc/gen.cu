// Device-side synthetic star polygons (the benchmark configurations' generator)
// plus the store's timing and launch-count helpers.
//
// The generator follows the same counter-based recipe as the host generator
// (farm_host.cpp): per polygon a centre, a mean radius and a start angle; per
// vertex an Exp(1) angular gap and a lognormal radius factor. Counts (and so
// offsets) come from the host generator; coordinates are drawn here with the
// device's libm, so they can differ from the host's in the last float bit.
#include <cmath>

#include "common.cuh"

namespace farm {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(uint64_t seed, uint64_t poly, uint32_t stream, uint64_t idx) {
    uint64_t h = mix64(seed ^ 0x5851F42D4C957F2Dull);
    h = mix64(h ^ poly);
    h = mix64(h ^ ((uint64_t)stream << 40) ^ idx);
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

enum : uint32_t { S_CX = 1, S_CY, S_R, S_N, S_PHI, S_GAP, S_NRM_U, S_NRM_V };

struct GenP {
    double dom_lo, dom_hi, r_lo, r_hi, sigma;
    uint64_t seed, first;
};

// Pass 1 (one warp per polygon): sum of the Exp(1) gaps (the angle normaliser).
__global__ void k_gen_gapsum(GenP g, const uint64_t *__restrict__ off, uint32_t n, double *__restrict__ gsum) {
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = w; k < n; k += nw) {
        uint64_t i = g.first + k;
        uint32_t nvert = (uint32_t)(off[k + 1] - off[k] - 1);
        double acc = 0.0;
        for (uint32_t j = lane; j <= nvert; j += 32) acc += -log(u01(g.seed, i, S_GAP, j));
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) gsum[k] = acc;
    }
}

// Pass 2 (one warp per polygon): vertices; the running gap sum is a warp scan.
__global__ void k_gen_fill(GenP g, const uint64_t *__restrict__ off, uint32_t n, const double *__restrict__ gsum,
                           float2 *__restrict__ xy) {
    const double two_pi = 6.283185307179586476925286766559;
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = w; k < n; k += nw) {
        uint64_t i = g.first + k;
        uint64_t b = off[k];
        uint32_t nvert = (uint32_t)(off[k + 1] - b - 1);
        double span = g.dom_hi - g.dom_lo;
        double cx = g.dom_lo + span * u01(g.seed, i, S_CX, 0);
        double cy = g.dom_lo + span * u01(g.seed, i, S_CY, 0);
        double lr0 = log(g.r_lo), lr1 = log(g.r_hi);
        double rbar = exp(lr0 + u01(g.seed, i, S_R, 0) * (lr1 - lr0));
        double phi = two_pi * u01(g.seed, i, S_PHI, 0);
        double total = gsum[k];
        double carry = 0.0;
        float2 first = make_float2(0.f, 0.f);
        for (uint32_t j0 = 0; j0 < nvert; j0 += 32) {
            uint32_t j = j0 + lane;
            double gap = j < nvert ? -log(u01(g.seed, i, S_GAP, j)) : 0.0;
            double incl = gap;
            for (int o = 1; o < 32; o <<= 1) {
                double v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            double cum = carry + incl;
            carry += __shfl_sync(0xffffffffu, incl, 31);
            if (j < nvert) {
                double th = phi + two_pi * (cum / total);
                double u = u01(g.seed, i, S_NRM_U, j), v = u01(g.seed, i, S_NRM_V, j);
                double z = sqrt(-2.0 * log(u)) * cos(two_pi * v);
                double r = rbar * exp(g.sigma * z);
                float2 q = make_float2((float)(cx + r * cos(th)), (float)(cy + r * sin(th)));
                xy[b + j] = q;
                if (j == 0) first = q;
            }
        }
        first = make_float2(__shfl_sync(0xffffffffu, first.x, 0), __shfl_sync(0xffffffffu, first.y, 0));
        if (lane == 0) xy[b + nvert] = first;  // closing copy
    }
}

}  // namespace farm

using namespace farm;

extern "C" {

/* Fill rings on the device: d_off (count + 1, device) must hold the offsets of
 * farm_gen_counts' counts (relative to d_xy); d_xy receives the vertices. */
int farm_gen_device(double dom_lo, double dom_hi, double r_lo, double r_hi, double sigma, uint64_t seed,
                    uint64_t first, uint64_t count, const uint64_t *d_off, float *d_xy) {
    if (!d_off || (count && !d_xy) || !(r_lo > 0) || r_hi < r_lo) {
        set_error("invalid arguments to farm_gen_device");
        return FARM_EINVAL;
    }
    if (count == 0) return FARM_OK;
    GenP g{dom_lo, dom_hi, r_lo, r_hi, sigma, seed, first};
    double *gsum = nullptr;
    FARM_CUDA(cudaMalloc(&gsum, 8 * count));
    unsigned blocks = (unsigned)((count * 32 + 255) / 256);
    unsigned cap = 64u * (unsigned)sm_count();
    if (blocks > cap) blocks = cap;
    k_gen_gapsum<<<blocks, 256>>>(g, d_off, (uint32_t)count, gsum);
    k_gen_fill<<<blocks, 256>>>(g, d_off, (uint32_t)count, gsum, reinterpret_cast<float2 *>(d_xy));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(gsum);
    if (e != cudaSuccess) return cuda_fail(e, "farm_gen_device");
    return FARM_OK;
}

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

/* Engine kernels launched by this store since it was created. */
uint64_t farm_store_launches(farm_store *s) { return s ? s->launches : 0; }

}  // extern "C"
