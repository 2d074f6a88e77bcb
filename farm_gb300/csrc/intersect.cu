// Stages (b) + (c) for intersect: pixel-pair raster filter and border
// refinement, one warp per candidate pair, in a persistent kernel that pulls
// pairs from a global counter (work stealing at pair granularity).
//
// Reference decision procedure (Ideal::intersect, Ideal.cpp:1329-1422):
//   for every non-OUT source pixel in the target MBR window (shrunk by 1e-6,
//   MyRaster.cpp:332-346) and every non-OUT target pixel in that pixel's box:
//   an IN pixel on either side decides "true"; BORDER x BORDER pixel pairs are
//   refined with segment_intersect over their edge sequences
//   (geometry_computation.h:215-237, FP32 cross products, Point.h:93-97).
// The order the reference visits pixel pairs in (sorted by fill probability)
// cannot change the boolean, so the warp visits them in any order and stops
// at the first decisive hit.
#include <cub/cub.cuh>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"
#include "segments.cuh"

namespace farm {

constexpr int kWarpsPerBlock = 8;
constexpr int kQueue = 256;  // BORDER x BORDER pixel pairs buffered per warp

struct PairView {
    const uint32_t *pairs;
    uint64_t n;
    uint64_t tgt_base;         // global index of target 0
    uint32_t *bb = nullptr;    // K_FILTER: per pair, refinement cost proxy (float bits)
    const uint32_t *order = nullptr;  // pairs taken in this order (largest first), else in index order
};

struct IxCounters {
    unsigned long long found, in_hits, border_pairs, segment_tests, src_window, tgt_window;
};

// (decodePixelArea(low) + decodePixelArea(high)) / 2 of a fill class
// (Ideal.cpp:47-62), as the reference's -a heuristic averages them
__device__ __forceinline__ double apx_area(uint8_t f, double pa, int cc) {
    if (f == 0) return 0.0;
    if (f == cc - 1) return (pa + pa) / 2;
    return ((1.0 * f - 1) / (cc - 2) * pa + (1.0 * f - 0) / (cc - 2) * pa) / 2;
}

// The warp's queue of BORDER x BORDER pixel pairs in descending fill
// probability, the order the reference refines candidates in (Ideal.cpp:
// 1393-1395): a bitonic network over the queue in shared memory, each lane
// taking every 32nd element. The boolean does not depend on the order; the
// order decides how soon an intersecting pair meets its first crossing.
__device__ void sort_queue_desc(float *key, uint2 *val, int n, int lane) {
    int N = 1;
    while (N < n) N <<= 1;
    for (int i = n + lane; i < N; i += 32) key[i] = -INFINITY;
    __syncwarp();
    for (int k = 2; k <= N; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < N; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const float a = key[i], b = key[ixj];
                    if ((a < b) == ((i & k) == 0)) {
                        key[i] = b;
                        key[ixj] = a;
                        const uint2 t = val[i];
                        val[i] = val[ixj];
                        val[ixj] = t;
                    }
                }
            }
            __syncwarp();
        }
}

// kMode: K_EXACT refines; K_APPROX is the reference's -a heuristic
// (kernel_calculate_probability, query_intersect.cu:100-134) instead of
// refinement — a BORDER x BORDER pixel pair decides "true" when
// (apx_s + apx_t) / max(pixel areas) > 1, and a pair with no IN overlap and no
// such pixel pair is "false"; K_FILTER runs the filter alone and writes 1 (an
// IN overlap: exact "true"), 0 (no non-OUT pixel pair at all: exact "false")
// or 3 (BORDER x BORDER pixel pairs to refine), the learned mode's first stage.
enum { K_EXACT = 0, K_APPROX = 1, K_FILTER = 2 };
template <int kMode>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_intersect(const StoreView sv, PairView pv, unsigned long long *__restrict__ next, uint8_t *__restrict__ out,
                IxCounters *__restrict__ ctr) {
    __shared__ uint2 queue[kWarpsPerBlock][kQueue];
    __shared__ float qkeys[kWarpsPerBlock][kQueue];
    __shared__ float4 tbufs[kWarpsPerBlock][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint2 *q = queue[wib];
    float *qk = qkeys[wib];
    float4 *tb = tbufs[wib];
    const int cc = sv.category_count;
    unsigned long long my_found = 0, my_in = 0, my_bb = 0, my_tests = 0, my_ws = 0, my_wt = 0;
    for (;;) {
        unsigned long long pid = 0;
        if (lane == 0) {
            pid = atomicAdd(next, 1ull);
            if (pv.order && pid < pv.n) pid = pv.order[pid];
        }
        pid = __shfl_sync(0xffffffffu, pid, 0);
        if (pid >= pv.n) break;
        const uint32_t s = pv.pairs[2 * pid], t = pv.pairs[2 * pid + 1];
        const PolyHdr &S = sv.hdr[s];
        const PolyHdr &T = sv.hdr[pv.tgt_base + t];
        if (S.err || T.err) {  // the reference aborts on one of the two polygons
            if (lane == 0 && out) out[pid] = 2;
            continue;
        }
        const uint8_t *sst = sv.status + S.st, *tst = sv.status + T.st;
        Window w = retrieve(S.mbr, S.step_x, S.step_y, S.dimx, S.dimy, T.mbr[0], T.mbr[1], T.mbr[2], T.mbr[3]);
        const int wh = w.ey - w.sy + 1;
        const long nw = (long)(w.ex - w.sx + 1) * wh;
        bool decided = false, has_bb = false;
        uint32_t pair_bb = 0;
        int qn = 0;  // warp-uniform queue fill
        auto flush = [&]() {
            // the warp refines the queued pixel pairs one after another, most
            // probable first, and stops at the first hit
            if (qn > 1) sort_queue_desc(qk, q, qn, lane);
            bool hit = false;
            for (int k = 0; k < qn && !hit; k++) {
                const uint2 pp = q[k];
                hit = refine_pixel_pair(sv, S, T, pp.x, pp.y, tb, my_tests);
            }
            qn = 0;
            __syncwarp();
            return hit;
        };
        for (long base = 0; base < nw && !decided; base += 32) {
            // one source window pixel per lane (x outer, y inner)
            long k = base + lane;
            int tw_sx = 0, tw_ex = -1, tw_sy = 0, tw_ey = -1;
            uint32_t pa = 0;
            int pa_st = 0;
            uint32_t cnt = 0;
            if (k < nw) {
                int i = w.sx + (int)(k / wh), j = w.sy + (int)(k % wh);
                pa = (uint32_t)(j * S.dimx + i);
                pa_st = show_status(sst[pa], cc);
                if (pa_st != 0) {
                    double b0 = S.mbr[0] + i * S.step_x, b1 = S.mbr[1] + j * S.step_y;
                    double b2 = S.mbr[0] + (i + 1) * S.step_x, b3 = S.mbr[1] + (j + 1) * S.step_y;
                    Window tw = retrieve(T.mbr, T.step_x, T.step_y, T.dimx, T.dimy, b0, b1, b2, b3);
                    tw_sx = tw.sx;
                    tw_ex = tw.ex;
                    tw_sy = tw.sy;
                    tw_ey = tw.ey;
                    cnt = (uint32_t)((tw.ex - tw.sx + 1) * (tw.ey - tw.sy + 1));
                }
            }
            // flatten the lanes' target windows across the warp
            uint32_t incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            uint32_t excl = incl - cnt;
            if (lane == 0) {
                my_ws += (unsigned long long)min((long)32, nw - base);
                my_wt += total;
            }
            for (uint32_t f = 0; f < total && !decided; f += 32) {
                uint32_t item = f + lane;
                bool valid = item < total;
                // owner lane: the last lane whose exclusive prefix <= item
                int owner = 0;
                for (int b = 16; b; b >>= 1) {
                    int cand = owner + b;
                    uint32_t ex = __shfl_sync(0xffffffffu, excl, cand);
                    if (cand < 32 && ex <= item) owner = cand;
                }
                uint32_t o_excl = __shfl_sync(0xffffffffu, excl, owner);
                int o_sx = __shfl_sync(0xffffffffu, tw_sx, owner), o_sy = __shfl_sync(0xffffffffu, tw_sy, owner);
                int o_ey = __shfl_sync(0xffffffffu, tw_ey, owner);
                uint32_t o_pa = __shfl_sync(0xffffffffu, pa, owner);
                int o_st = __shfl_sync(0xffffffffu, pa_st, owner);
                bool in_hit = false, bb = false;
                float prob = 0.f;  // fill probability of a BORDER x BORDER pair (refinement order)
                uint32_t pb = 0;
                if (valid) {
                    uint32_t r = item - o_excl;
                    int th = o_ey - o_sy + 1;
                    int u = o_sx + (int)(r / (uint32_t)th), v = o_sy + (int)(r % (uint32_t)th);
                    pb = (uint32_t)(v * T.dimx + u);
                    int pb_st = show_status(tst[pb], cc);
                    if (pb_st != 0) {
                        if (o_st == 2 || pb_st == 2) {
                            in_hit = true;
                        } else if (kMode == K_APPROX) {
                            const double spa = S.step_x * S.step_y, tpa = T.step_x * T.step_y;
                            const double pr = (apx_area(sst[o_pa], spa, cc) + apx_area(tst[pb], tpa, cc)) /
                                              (spa > tpa ? spa : tpa);
                            in_hit = pr > 1.0;
                            bb = true;
                        } else {
                            const double spa = S.step_x * S.step_y, tpa = T.step_x * T.step_y;
                            prob = (float)((apx_area(sst[o_pa], spa, cc) + apx_area(tst[pb], tpa, cc)) /
                                           (spa > tpa ? spa : tpa));
                            bb = true;
                        }
                    }
                }
                if (__any_sync(0xffffffffu, in_hit)) {
                    decided = true;
                    if (lane == 0) my_in++;
                    break;
                }
                unsigned m = __ballot_sync(0xffffffffu, bb);
                if (kMode != K_EXACT) {  // nothing to refine
                    if (lane == 0) my_bb += __popc(m);
                    has_bb |= m != 0;
                    pair_bb += __popc(m);
                    m = 0;
                }
                if (m) {
                    int nb = __popc(m);
                    if (qn + nb > kQueue) {
                        __syncwarp();
                        if (flush()) {
                            decided = true;
                            break;
                        }
                    }
                    if (bb) {
                        const int at = qn + __popc(m & ((1u << lane) - 1));
                        q[at] = make_uint2(o_pa, pb);
                        qk[at] = prob;
                    }
                    qn += nb;
                    if (lane == 0) my_bb += nb;
                    __syncwarp();
                }
            }
        }
        if (!decided && qn > 0) {
            __syncwarp();
            decided = flush();
        }
        if (lane == 0) {
            if (out) out[pid] = decided ? 1 : (kMode == K_FILTER && has_bb ? 3 : 0);
            if (kMode == K_FILTER && pv.bb) {
                // refinement cost proxy: BORDER x BORDER pixel pairs x the two
                // polygons' edges per pixel (segment tests per pixel pair)
                const float c = (float)pair_bb * ((float)S.nv / (float)(S.P ? S.P : 1)) *
                                ((float)T.nv / (float)(T.P ? T.P : 1));
                pv.bb[pid] = __float_as_uint(c);
            }
            my_found += decided;
        }
        __syncwarp();
    }
    // counters: one atomic per warp
    for (int o = 16; o; o >>= 1) my_tests += __shfl_xor_sync(0xffffffffu, my_tests, o);
    if (lane == 0) {
        atomicAdd(&ctr->found, my_found);
        atomicAdd(&ctr->in_hits, my_in);
        atomicAdd(&ctr->border_pairs, my_bb);
        atomicAdd(&ctr->segment_tests, my_tests);
        atomicAdd(&ctr->src_window, my_ws);
        atomicAdd(&ctr->tgt_window, my_wt);
    }
}

int intersect_learned(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint8_t *out, uint64_t *found,
                      farm_stats *st);

// The filter alone over n device pairs: out[k] = 1 / 0 / 3 (K_FILTER). Counts
// IN-decided pairs into *in_hits.
int intersect_filter(farm_store *s, const uint32_t *dpairs, uint64_t n, uint8_t *dout, uint64_t *in_hits,
                     uint32_t *bb) {
    cudaStream_t stream = s->stream;
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *next = s->d_counters.as<unsigned long long>() + 8;
    IxCounters *ctr = reinterpret_cast<IxCounters *>(next + 1);
    FARM_CUDA(cudaMemsetAsync(next, 0, 8 + sizeof(IxCounters), stream));
    PairView pv{dpairs, n, s->n_side[0], bb};
    k_intersect<K_FILTER><<<sm_count() * 8, kWarpsPerBlock * 32, 0, stream>>>(s->view(), pv, next, dout, ctr);
    s->launches++;
    FARM_CUDA(cudaGetLastError());
    IxCounters h{};
    FARM_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    if (in_hits) *in_hits = h.in_hits;
    return FARM_OK;
}

// Work order for the exact query: pairs by descending product of their
// polygons' vertex counts, so that the heaviest pairs start first and the
// pass does not end on a long pair that started last (longest-first
// scheduling). Results are written by pair index, so the order is invisible.
__global__ void k_pair_cost(const StoreView sv, const uint32_t *__restrict__ pairs, uint64_t n, uint64_t tgt_base,
                            uint32_t *__restrict__ key, uint32_t *__restrict__ idx) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const float c = (float)sv.hdr[pairs[2 * k]].nv * (float)sv.hdr[tgt_base + pairs[2 * k + 1]].nv;
        key[k] = ~__float_as_uint(c);  // positive floats order as their bits; ~ for descending
        idx[k] = (uint32_t)k;
    }
}

// FARM_PAIR_ORDER=0 takes the pairs in index order
static bool pair_order_on() {
    const char *v = getenv("FARM_PAIR_ORDER");
    return !(v && *v == '0');
}

static int pair_order(farm_store *s, const uint32_t *dpairs, uint64_t n, const uint32_t **order) {
    *order = nullptr;
    if (n < 2 || n > 0xFFFFFFFFull) return FARM_OK;
    cudaStream_t stream = s->stream;
    FARM_TRY(s->s[Q_PAIR_ORDER].ensure(16 * n + 64));
    uint32_t *key = s->s[Q_PAIR_ORDER].as<uint32_t>(), *key_s = key + n, *idx = key_s + n, *idx_s = idx + n;
    unsigned blocks = grid_for(n, 256);
    if (blocks > 16u * (unsigned)sm_count()) blocks = 16u * (unsigned)sm_count();
    k_pair_cost<<<blocks, 256, 0, stream>>>(s->view(), dpairs, n, s->n_side[0], key, idx);
    FARM_CUDA(cudaGetLastError());
    s->launches++;
    size_t bytes = 0;
    FARM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, key, key_s, idx, idx_s, (int64_t)n, 0, 32, stream));
    FARM_TRY(s->cub_tmp.ensure(bytes + 64));
    FARM_CUDA(cub::DeviceRadixSort::SortPairs(s->cub_tmp.p, bytes, key, key_s, idx, idx_s, (int64_t)n, 0, 32,
                                              stream));
    *order = idx_s;
    return FARM_OK;
}

int intersect(farm_store *s, const uint32_t *pairs, uint64_t n, int mode, int mem, uint8_t *out, uint64_t *found,
              farm_stats *st) {
    if (!s->rasterized) {
        set_error("farm_intersect: rasterize first");
        return FARM_EINVAL;
    }
    if (s->n_side[1] == 0) {
        set_error("farm_intersect: no target side loaded");
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
    if (mem == FARM_MEM_HOST) {
        FARM_TRY(s->d_out.ensure(n + 16));
        dout = s->d_out.as<uint8_t>();
    }
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *next = s->d_counters.as<unsigned long long>();
    IxCounters *ctr = reinterpret_cast<IxCounters *>(next + 1);
    FARM_CUDA(cudaMemsetAsync(next, 0, 8 + sizeof(IxCounters), stream));
    PairView pv{dpairs, n, s->n_side[0]};
    StoreView sv = s->view();
    FARM_CUDA(cudaEventRecord(s->ev[6], stream));
    if (mode == FARM_MODE_EXACT && pair_order_on()) FARM_TRY(pair_order(s, dpairs, n, &pv.order));
    int blocks = sm_count() * 8;
    if (mode == FARM_MODE_APPROX)
        k_intersect<K_APPROX><<<blocks, kWarpsPerBlock * 32, 0, stream>>>(sv, pv, next, dout, ctr);
    else
        k_intersect<K_EXACT><<<blocks, kWarpsPerBlock * 32, 0, stream>>>(sv, pv, next, dout, ctr);
    s->launches++;
    FARM_CUDA(cudaGetLastError());
    FARM_CUDA(cudaEventRecord(s->ev[7], stream));
    IxCounters h{};
    FARM_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && out && n) FARM_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    if (found) *found = h.found;
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        st->found = h.found;
        st->in_hits = h.in_hits;
        st->border_pairs = h.border_pairs;
        st->segment_tests = h.segment_tests;
        st->src_window_pixels = h.src_window;
        st->tgt_window_pixels = h.tgt_window;
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[6], s->ev[7]);
        st->ms_total = ms;
        st->ms_stage[1] = ms;
        st->kernel_launches = 1;
    }
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_intersect_filter(farm_store *s, const uint32_t *d_pairs, uint64_t n, uint8_t *d_code,
                                     float *d_cost) {
    using namespace farm;
    if (!s || (n && (!d_pairs || !d_code || !d_cost))) {
        set_error("invalid arguments to farm_intersect_filter");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("farm_intersect_filter: rasterize first");
        return FARM_EINVAL;
    }
    if (!n) return FARM_OK;
    FARM_TRY(check_pairs(s, d_pairs, n, FARM_MEM_DEVICE, false, "farm_intersect_filter"));
    return intersect_filter(s, d_pairs, n, d_code, nullptr, reinterpret_cast<uint32_t *>(d_cost));
}

extern "C" int farm_intersect(farm_store *s, const uint32_t *pairs, uint64_t n, int mode, int mem, uint8_t *out,
                              uint64_t *found, farm_stats *st) {
    using namespace farm;
    if (!s || (n && !pairs)) {
        set_error("invalid arguments to farm_intersect");
        return FARM_EINVAL;
    }
    if (s->rasterized && s->n_side[1]) FARM_TRY(check_pairs(s, pairs, n, mem, false, "farm_intersect"));
    if (mode == FARM_MODE_LEARNED) return intersect_learned(s, pairs, n, mem, out, found, st);
    if (mode == FARM_MODE_FILTER) {
        if (!s->rasterized) {
            set_error("farm_intersect: rasterize first");
            return FARM_EINVAL;
        }
        if (mem != FARM_MEM_DEVICE || (n && !out)) {
            set_error("farm_intersect: FARM_MODE_FILTER takes device pairs and a device output");
            return FARM_EINVAL;
        }
        uint64_t in_hits = 0;
        FARM_TRY(intersect_filter(s, pairs, n, out, &in_hits, nullptr));
        if (found) *found = in_hits;
        if (st) {
            memset(st, 0, sizeof *st);
            st->pairs = n;
            st->found = in_hits;
            st->in_hits = in_hits;
        }
        return FARM_OK;
    }
    if (mode != FARM_MODE_EXACT && mode != FARM_MODE_APPROX) {
        set_error("farm_intersect: unknown mode");
        return FARM_EINVAL;
    }
    return intersect(s, pairs, n, mode, mem, out, found, st);
}

// ------------------------------------------------ allocation-free entry --
// farm_intersect_static: the same filter + refine kernel, but every device
// byte it needs beyond the store (the staged pair list, the result bytes and
// the work/stat counters) lives in one file-scope __device__ array instead of
// store buffers that farm_intersect grows with cudaMalloc. It is for callers
// that must not allocate device memory at query time: code whose device memory
// is owned by another allocator (a framework's caching allocator that has
// reserved the HBM), and host threads that must not trigger the device-wide
// synchronisation a cudaMalloc/cudaFree implies while other streams run.
namespace farm {

constexpr uint64_t kStaticMaxPairs = 1ull << 20;  // 1,048,576 pairs per call
constexpr size_t kStaticCtrBytes = 256;
constexpr size_t kStaticBytes = kStaticCtrBytes + 8 * kStaticMaxPairs + kStaticMaxPairs;  // ~9 MiB
constexpr int kStaticMaxDevices = 64;

// Shared by every call on a device and kept for the life of the process.
static __device__ __align__(256) unsigned char g_intersect_static[kStaticBytes];

static std::mutex g_static_mu;
static unsigned char *g_static_addr[kStaticMaxDevices] = {};

// Device address of the array on the current device, looked up once per device.
static int static_scratch(int dev, unsigned char **p) {
    if (dev < 0 || dev >= kStaticMaxDevices) {
        set_error("farm_intersect_static: device ordinal out of range");
        return FARM_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[dev]) {
        void *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&q, g_intersect_static);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_intersect_static)");
        g_static_addr[dev] = static_cast<unsigned char *>(q);
    }
    *p = g_static_addr[dev];
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_intersect_static(farm_store *s, const uint32_t *pairs, uint64_t n, uint8_t *out,
                                     uint64_t *found) {
    using namespace farm;
    if (!s || (n && (!pairs || !out))) {
        set_error("invalid arguments to farm_intersect_static");
        return FARM_EINVAL;
    }
    if (n > kStaticMaxPairs) {
        set_error("farm_intersect_static: " + std::to_string(n) + " pairs exceed its fixed scratch of " +
                  std::to_string(kStaticMaxPairs) + " pairs; split the list or use farm_intersect");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("farm_intersect_static: rasterize first");
        return FARM_EINVAL;
    }
    if (s->n_side[1] == 0) {
        set_error("farm_intersect_static: no target side loaded");
        return FARM_EINVAL;
    }
    // host-side range check of every pair before any device work
    FARM_TRY(check_pairs(s, pairs, n, FARM_MEM_HOST, false, "farm_intersect_static"));
    int cur = 0;
    FARM_CUDA(cudaGetDevice(&cur));
    if (cur != s->device) FARM_CUDA(cudaSetDevice(s->device));
    unsigned char *base = nullptr;
    int rc = static_scratch(s->device, &base);
    if (rc == FARM_OK) {
        cudaStream_t stream = s->stream;
        unsigned long long *next = reinterpret_cast<unsigned long long *>(base);
        IxCounters *ctr = reinterpret_cast<IxCounters *>(next + 1);
        uint32_t *dpairs = reinterpret_cast<uint32_t *>(base + kStaticCtrBytes);
        uint8_t *dout = base + kStaticCtrBytes + 8 * kStaticMaxPairs;
        IxCounters h{};
        cudaError_t e = cudaMemsetAsync(base, 0, kStaticCtrBytes, stream);  // counters start at zero
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(dpairs, pairs, 8 * n, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess && n) {
            PairView pv{dpairs, n, s->n_side[0]};
            k_intersect<K_EXACT><<<sm_count() * 8, kWarpsPerBlock * 32, 0, stream>>>(s->view(), pv, next, dout, ctr);
            e = cudaGetLastError();
            if (e == cudaSuccess) s->launches++;
        }
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "farm_intersect_static");
        else if (found)
            *found = h.found;
    }
    if (cur != s->device) cudaSetDevice(cur);
    return rc;
}
