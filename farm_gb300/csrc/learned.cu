// Learned approximate intersect (MLP scorer); see mlp kernels.
#include "common.cuh"

namespace farm {

int intersect_learned(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint8_t *out, uint64_t *found,
                      farm_stats *st) {
    (void)s; (void)pairs; (void)n; (void)mem; (void)out; (void)found; (void)st;
    set_error("learned mode needs a trained scorer: none is loaded in this store");
    return FARM_EINVAL;
}

}  // namespace farm
