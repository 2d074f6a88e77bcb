// The store's timing and launch-count helpers.
#include "common.cuh"

using namespace farm;

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

/* Engine kernels launched by this store since it was created. */
uint64_t farm_store_launches(farm_store *s) { return s ? s->launches : 0; }

}  // extern "C"
