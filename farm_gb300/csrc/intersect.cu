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

#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace farm {

constexpr int kWarpsPerBlock = 8;
constexpr int kQueue = 256;  // BORDER x BORDER pixel pairs buffered per warp

struct PairView {
    const uint32_t *pairs;
    uint64_t n;
    uint64_t tgt_base;  // global index of target 0
};

// Point.h:93-97: (a - o) x (b - o) in float, no fused multiply-add
__device__ __forceinline__ float cross3(float2 o, float2 a, float2 b) {
    float ax = __fsub_rn(a.x, o.x), ay = __fsub_rn(a.y, o.y);
    float bx = __fsub_rn(b.x, o.x), by = __fsub_rn(b.y, o.y);
    return __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
}

__device__ __forceinline__ int sgnf(float x) { return x >= 0 ? (x != 0 ? 1 : 0) : -1; }

__device__ __forceinline__ bool inter1(double a, double b, double c, double d) {
    double t;
    if (a > b) { t = a; a = b; b = t; }
    if (c > d) { t = c; c = d; d = t; }
    return fmax(a, c) <= fmin(b, d);
}

// geometry_computation.h:215-221
__device__ __forceinline__ bool seg_intersect(float2 a, float2 b, float2 c, float2 d) {
    if (cross3(c, a, d) == 0.0f && cross3(c, b, d) == 0.0f)
        return inter1(a.x, b.x, c.x, d.x) && inter1(a.y, b.y, c.y, d.y);
    return sgnf(cross3(a, b, c)) != sgnf(cross3(a, b, d)) && sgnf(cross3(c, d, a)) != sgnf(cross3(c, d, b));
}

struct Window {
    int sx, ex, sy, ey;
};

// MyRaster.cpp:332-346
__device__ __forceinline__ Window retrieve(const double *mbr, double stx, double sty, int dimx, int dimy,
                                           double b0, double b1, double b2, double b3) {
    Window w;
    w.sx = offset_x(mbr, stx, dimx, b0 + 1e-6);
    w.sy = offset_y(mbr, sty, dimy, b1 + 1e-6);
    w.ex = offset_x(mbr, stx, dimx, b2 - 1e-6);
    w.ey = offset_y(mbr, sty, dimy, b3 - 1e-6);
    return w;
}

struct IxCounters {
    unsigned long long found, in_hits, border_pairs, segment_tests, src_window, tgt_window;
};

// Refine one BORDER x BORDER pixel pair: any edge-sequence pair with an
// intersecting segment pair (geometry_computation.h:224-237).
__device__ bool refine_pixel_pair(const StoreView &sv, const PolyHdr &S, const PolyHdr &T, uint32_t pa, uint32_t pb,
                                  unsigned long long &tests) {
    const uint32_t *so = sv.offset + S.off, *to = sv.offset + T.off;
    uint32_t a0 = so[pa], a1 = so[pa + 1], b0 = to[pb], b1 = to[pb + 1];
    const uint2 *sseq = sv.seq + S.seq, *tseq = sv.seq + T.seq;
    const float2 *sr = sv.ring + S.ring, *tr = sv.ring + T.ring;
    for (uint32_t i = a0; i < a1; i++) {
        uint2 r = sseq[i];
        for (uint32_t j = b0; j < b1; j++) {
            uint2 r2 = tseq[j];
            for (uint32_t u = 0; u < r.y; u++) {
                float2 a = sr[r.x + u], b = sr[r.x + u + 1];
                for (uint32_t v = 0; v < r2.y; v++) {
                    tests++;
                    if (seg_intersect(a, b, tr[r2.x + v], tr[r2.x + v + 1])) return true;
                }
            }
        }
    }
    return false;
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_intersect(const StoreView sv, PairView pv, unsigned long long *__restrict__ next, uint8_t *__restrict__ out,
                IxCounters *__restrict__ ctr) {
    __shared__ uint2 queue[kWarpsPerBlock][kQueue];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint2 *q = queue[wib];
    const int cc = sv.category_count;
    unsigned long long my_found = 0, my_in = 0, my_bb = 0, my_tests = 0, my_ws = 0, my_wt = 0;
    for (;;) {
        unsigned long long pid = 0;
        if (lane == 0) pid = atomicAdd(next, 1ull);
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
        bool decided = false;
        int qn = 0;  // warp-uniform queue fill
        auto flush = [&]() {
            // lanes take queued pixel pairs; stop at the first hit
            bool hit = false;
            for (int k = lane; k < qn; k += 32) {
                if (refine_pixel_pair(sv, S, T, q[k].x, q[k].y, my_tests)) {
                    hit = true;
                    break;
                }
            }
            qn = 0;
            return __any_sync(0xffffffffu, hit);
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
                uint32_t pb = 0;
                if (valid) {
                    uint32_t r = item - o_excl;
                    int th = o_ey - o_sy + 1;
                    int u = o_sx + (int)(r / (uint32_t)th), v = o_sy + (int)(r % (uint32_t)th);
                    pb = (uint32_t)(v * T.dimx + u);
                    int pb_st = show_status(tst[pb], cc);
                    if (pb_st != 0) {
                        if (o_st == 2 || pb_st == 2)
                            in_hit = true;
                        else
                            bb = true;
                    }
                }
                if (__any_sync(0xffffffffu, in_hit)) {
                    decided = true;
                    if (lane == 0) my_in++;
                    break;
                }
                unsigned m = __ballot_sync(0xffffffffu, bb);
                if (m) {
                    int nb = __popc(m);
                    if (qn + nb > kQueue) {
                        __syncwarp();
                        if (flush()) {
                            decided = true;
                            break;
                        }
                    }
                    if (bb) q[qn + __popc(m & ((1u << lane) - 1))] = make_uint2(o_pa, pb);
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
            if (out) out[pid] = decided ? 1 : 0;
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
    int blocks = sm_count() * 8;
    k_intersect<<<blocks, kWarpsPerBlock * 32, 0, stream>>>(sv, pv, next, dout, ctr);
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
    (void)mode;
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_intersect(farm_store *s, const uint32_t *pairs, uint64_t n, int mode, int mem, uint8_t *out,
                              uint64_t *found, farm_stats *st) {
    using namespace farm;
    if (!s || (n && !pairs)) {
        set_error("invalid arguments to farm_intersect");
        return FARM_EINVAL;
    }
    if (mode != FARM_MODE_EXACT) return intersect_learned(s, pairs, n, mem, out, found, st);
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
            k_intersect<<<sm_count() * 8, kWarpsPerBlock * 32, 0, stream>>>(s->view(), pv, next, dout, ctr);
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
