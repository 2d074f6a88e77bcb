// Learned approximate intersect (FARM_MODE_LEARNED): the MLP scorer decides
// the pairs it is sure about; pairs inside its uncertainty band go to exact
// refinement (the same decision procedure as FARM_MODE_EXACT). It stands where
// the reference's "-a" confidence heuristic stands (query_intersect.cu:100-134).
#include <cstring>

#include "common.cuh"

extern "C" int farm_mlp_predict(farm_store *s, const uint32_t *d_pairs, uint64_t n, float *d_prob);

namespace farm {

float mlp_band(farm_store *s, int which);
int intersect(farm_store *s, const uint32_t *pairs, uint64_t n, int mode, int mem, uint8_t *out, uint64_t *found,
              farm_stats *st);

// confident pairs decided, uncertain ones compacted for exact refinement
__global__ void k_band(const float *__restrict__ prob, const uint32_t *__restrict__ pairs, uint64_t n, float lo,
                       float hi, uint8_t *__restrict__ out, uint32_t *__restrict__ apairs,
                       uint64_t *__restrict__ aidx, unsigned long long *__restrict__ na) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        float p = prob[k];
        if (p >= hi) {
            out[k] = 1;
        } else if (p <= lo) {
            out[k] = 0;
        } else {
            unsigned long long at = atomicAdd(na, 1ull);
            apairs[2 * at] = pairs[2 * k];
            apairs[2 * at + 1] = pairs[2 * k + 1];
            aidx[at] = k;
        }
    }
}

__global__ void k_unband(const uint8_t *__restrict__ aout, const uint64_t *__restrict__ aidx, uint64_t na,
                         uint8_t *__restrict__ out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < na; k += (uint64_t)gridDim.x * blockDim.x)
        out[aidx[k]] = aout[k];
}

__global__ void k_count_ones(const uint8_t *__restrict__ out, uint64_t n, unsigned long long *c) {
    unsigned long long f = 0;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        f += out[k] == 1;
    for (int o = 16; o; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(c, f);
}

int intersect_learned(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint8_t *out, uint64_t *found,
                      farm_stats *st) {
    if (!s->mlp) {
        set_error("learned mode needs a trained scorer (farm_mlp_train or farm_mlp_set)");
        return FARM_EINVAL;
    }
    cudaStream_t stream = s->stream;
    const uint32_t *dpairs = pairs;
    if (mem == FARM_MEM_HOST && n) {
        FARM_TRY(s->d_pairs.ensure(8 * n));
        FARM_CUDA(cudaMemcpyAsync(s->d_pairs.p, pairs, 8 * n, cudaMemcpyHostToDevice, stream));
        dpairs = s->d_pairs.as<uint32_t>();
    }
    uint8_t *dout = out;
    if (mem == FARM_MEM_HOST || !out) {
        FARM_TRY(s->d_out.ensure(n + 64));
        dout = s->d_out.as<uint8_t>();
    }
    DevBuf &prob = s->s[26], &ap = s->s[27], &ao = s->s[28];
    FARM_TRY(prob.ensure(4 * n + 64));
    FARM_TRY(ap.ensure(16 * n + 64));
    FARM_TRY(ao.ensure(n + 64));
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *na = s->d_counters.as<unsigned long long>() + 24;
    FARM_CUDA(cudaEventRecord(s->ev[6], stream));
    int rc = farm_mlp_predict(s, dpairs, n, prob.as<float>());
    if (rc) return rc;
    FARM_CUDA(cudaMemsetAsync(na, 0, 16, stream));
    uint32_t *apairs = ap.as<uint32_t>();
    uint64_t *aidx = reinterpret_cast<uint64_t *>(apairs + 2 * n + 2);
    unsigned blocks = (unsigned)((n + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    if (!blocks) blocks = 1;
    k_band<<<blocks, 256, 0, stream>>>(prob.as<float>(), dpairs, n, mlp_band(s, 0), mlp_band(s, 1), dout, apairs,
                                       aidx, na);
    unsigned long long h_na = 0;
    FARM_CUDA(cudaMemcpyAsync(&h_na, na, 8, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    farm_stats est;
    memset(&est, 0, sizeof est);
    if (h_na) {
        // the band's pairs through the exact path (its own events: 6/7 are reused)
        FARM_TRY(intersect(s, apairs, h_na, FARM_MODE_EXACT, FARM_MEM_DEVICE, ao.as<uint8_t>(), nullptr, &est));
        unsigned ub = (unsigned)((h_na + 255) / 256);
        if (ub > 8192) ub = 8192;
        k_unband<<<ub, 256, 0, stream>>>(ao.as<uint8_t>(), aidx, h_na, dout);
    }
    k_count_ones<<<blocks, 256, 0, stream>>>(dout, n, na + 1);
    unsigned long long h_found = 0;
    FARM_CUDA(cudaMemcpyAsync(&h_found, na + 1, 8, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && out && n) FARM_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    s->launches += 2 + (h_na ? 1 : 0);
    if (found) *found = h_found;
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        st->found = h_found;
        st->fp64_rechecks = h_na;  // pairs refined exactly (abstentions)
        st->segment_tests = est.segment_tests;
        st->border_pairs = est.border_pairs;
        st->ms_stage[1] = est.ms_total;
        st->kernel_launches = 2 + est.kernel_launches;
    }
    return FARM_OK;
}

}  // namespace farm
