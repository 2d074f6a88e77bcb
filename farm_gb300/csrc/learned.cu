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

int intersect_filter(farm_store *s, const uint32_t *dpairs, uint64_t n, uint8_t *dout, uint64_t *in_hits,
                     uint32_t *bb);

// pairs the filter left undecided (code 3), compacted with their positions
__global__ void k_select_undecided(const uint8_t *__restrict__ code, const uint32_t *__restrict__ pairs,
                                   const uint32_t *__restrict__ bb, uint64_t n, uint32_t *__restrict__ upairs,
                                   uint64_t *__restrict__ uidx, uint32_t *__restrict__ ucost,
                                   unsigned long long *__restrict__ nu) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        if (code[k] != 3) continue;
        unsigned long long at = atomicAdd(nu, 1ull);
        upairs[2 * at] = pairs[2 * k];
        upairs[2 * at + 1] = pairs[2 * k + 1];
        uidx[at] = k;
        ucost[at] = bb[k];
    }
}

// confident pairs decided, uncertain ones compacted for exact refinement.
// Confidence is p >= hi / p <= lo, or — cost-aware — an uncertainty
// min(p, 1 - p) no larger than lambda x the pair's refinement cost proxy (its
// BORDER x BORDER pixel pairs x both polygons' edges per pixel), so the error
// budget goes where deciding saves the most refinement.
__global__ void k_band(const float *__restrict__ prob, const uint32_t *__restrict__ upairs,
                       const uint64_t *__restrict__ uidx, const uint32_t *__restrict__ ucost, uint64_t nu, float lo,
                       float hi, float lambda, uint8_t *__restrict__ out, uint32_t *__restrict__ apairs,
                       uint64_t *__restrict__ aidx, unsigned long long *__restrict__ na) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nu; k += (uint64_t)gridDim.x * blockDim.x) {
        const float p = prob[k];
        const float u = p < 0.5f ? p : 1.f - p;
        const bool cheap = lambda > 0.f && u <= lambda * __uint_as_float(ucost[k]);
        if (p >= hi || (cheap && p >= 0.5f)) {
            out[uidx[k]] = 1;
        } else if (p <= lo || cheap) {
            out[uidx[k]] = 0;
        } else {
            unsigned long long at = atomicAdd(na, 1ull);
            apairs[2 * at] = upairs[2 * k];
            apairs[2 * at + 1] = upairs[2 * k + 1];
            aidx[at] = uidx[k];
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

static unsigned blocks_for(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    return (unsigned)(b > 8192 ? 8192 : (b ? b : 1));
}

// Three stages: (1) the exact filter decides the pairs it can without
// refinement (an IN overlap: true; no BORDER x BORDER pixel pair: false, and
// pairs on an unrasterizable polygon: 2); (2) the scorer decides the rest
// where its probability lies outside the band; (3) the band's pairs are
// refined exactly. Stages 1 and 3 are the exact procedure, so every error
// comes from stage 2's confident decisions.
int intersect_learned(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint8_t *out, uint64_t *found,
                      farm_stats *st) {
    if (!s->mlp) {
        set_error("learned mode needs a trained scorer (farm_mlp_train or farm_mlp_set)");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("farm_intersect: rasterize first");
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
    DevBuf &prob = s->s[Q_SCR0], &up = s->s[Q_SCR1], &ap = s->s[Q_SCR2], &ao = s->s[Q_SCR3], &cost = s->s[Q_SCR4];
    FARM_TRY(prob.ensure(4 * n + 64));
    FARM_TRY(up.ensure(16 * n + 64));
    FARM_TRY(ap.ensure(16 * n + 64));
    FARM_TRY(ao.ensure(n + 64));
    FARM_TRY(cost.ensure(8 * n + 64));
    uint32_t *bb = cost.as<uint32_t>(), *ucost = bb + n + 16;
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *cnt = s->d_counters.as<unsigned long long>() + 24;  // [0] undecided [1] band [2] found
    FARM_CUDA(cudaMemsetAsync(cnt, 0, 24, stream));
    // own events: the exact call below records the store's internal pair
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    if (t0) cudaEventRecord(t0, stream);
    uint64_t in_hits = 0;
    if (n) FARM_TRY(intersect_filter(s, dpairs, n, dout, &in_hits, bb));
    uint32_t *upairs = up.as<uint32_t>();
    uint64_t *uidx = reinterpret_cast<uint64_t *>(upairs + 2 * n + 2);
    k_select_undecided<<<blocks_for(n), 256, 0, stream>>>(dout, dpairs, bb, n, upairs, uidx, ucost, cnt);
    unsigned long long h_nu = 0;
    FARM_CUDA(cudaMemcpyAsync(&h_nu, cnt, 8, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    unsigned long long h_na = 0;
    farm_stats est;
    memset(&est, 0, sizeof est);
    if (h_nu) {
        int rc = farm_mlp_predict(s, upairs, h_nu, prob.as<float>());
        if (rc) return rc;
        uint32_t *apairs = ap.as<uint32_t>();
        uint64_t *aidx = reinterpret_cast<uint64_t *>(apairs + 2 * n + 2);
        k_band<<<blocks_for(h_nu), 256, 0, stream>>>(prob.as<float>(), upairs, uidx, ucost, h_nu, mlp_band(s, 0),
                                                     mlp_band(s, 1), mlp_band(s, 2), dout, apairs, aidx, cnt + 1);
        FARM_CUDA(cudaMemcpyAsync(&h_na, cnt + 1, 8, cudaMemcpyDeviceToHost, stream));
        FARM_CUDA(cudaStreamSynchronize(stream));
        if (h_na) {
            // the band's pairs through the exact path (its own events: 6/7 are reused)
            FARM_TRY(intersect(s, apairs, h_na, FARM_MODE_EXACT, FARM_MEM_DEVICE, ao.as<uint8_t>(), nullptr, &est));
            k_unband<<<blocks_for(h_na), 256, 0, stream>>>(ao.as<uint8_t>(), aidx, h_na, dout);
        }
    }
    k_count_ones<<<blocks_for(n), 256, 0, stream>>>(dout, n, cnt + 2);
    unsigned long long h_found = 0;
    FARM_CUDA(cudaMemcpyAsync(&h_found, cnt + 2, 8, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && out && n) FARM_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream));
    if (t1) cudaEventRecord(t1, stream);
    FARM_CUDA(cudaStreamSynchronize(stream));
    s->launches += 2 + (h_nu ? 1 : 0) + (h_na ? 1 : 0);
    if (found) *found = h_found;
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        st->found = h_found;
        st->in_hits = in_hits;
        st->fp64_rechecks = h_na;  // pairs refined exactly (abstentions)
        st->segment_tests = est.segment_tests;
        st->border_pairs = h_nu;   // pairs the scorer saw
        float ms = 0;
        if (t0 && t1) cudaEventElapsedTime(&ms, t0, t1);
        st->ms_total = ms;
        st->ms_stage[1] = est.ms_total;
        st->kernel_launches = 3 + est.kernel_launches;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    return FARM_OK;
}
}  // namespace farm
