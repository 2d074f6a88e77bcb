// Candidate generation on the GPU: the MBR join that precedes every query.
//
// The reference builds an R-tree over the source MBRs and searches it once
// per target (RTree.h:581-600, driven by intersect_cpu.cpp:18-36 and
// within_polygon_cpu.cpp:20-49, the within query widening each target's box
// by the distance as Box.cpp:200-214 does). The result is the set of
// (source, target) pairs whose closed MBRs overlap; farm_mbr_join
// (farm_host.cpp) computes that set on the host. Here it is computed from the
// rings already in the store, so an end-to-end query needs no host join:
//
//   k_join_mbr     per polygon (a warp each): its MBR from the stored vertices,
//                  the Box.h:6-12 start values and the float bias of
//                  vertex_sequence.cpp:152-168, as farm_mbr and k_header do;
//   sort           sources by their low x (order-preserving 64-bit keys);
//   k_join_width   the widest source box;
//   k_join_count   per target (a thread each): the sources whose low x lies in
//                  [q.lo.x - widest, q.hi.x] (q the widened target box), each
//                  tested by the same closed-overlap comparisons as the host;
//   scan, k_join_fill with the same loop, one 64-bit key per pair
//                  (source << 32 | target), and a radix sort of the keys: the
//                  host join's ascending (source, target) order.
#include <cub/cub.cuh>

#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace farm {

__device__ __forceinline__ uint64_t jkey(double v) {  // order-preserving bits of a double
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// MBR (lx, ly, hx, hy) of polygons [p0, p0 + n) of the store, by warp.
__global__ void k_join_mbr(const float2 *__restrict__ ring, const uint64_t *__restrict__ off, uint64_t p0, uint32_t n,
                           double4 *__restrict__ mbr) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = warp; k < n; k += nw) {
        const uint64_t p = p0 + k;
        const uint64_t b = off[p], e = off[p + 1];
        const float2 *r = ring + b + 2ull * p;
        const uint32_t m = (uint32_t)(e - b);
        double lx = 100000.0, ly = 100000.0, hx = -100000.0, hy = -100000.0;
        for (uint32_t j = lane; j < m; j += 32) {
            const float2 q = r[j];
            lx = fmin(lx, (double)q.x);
            hx = fmax(hx, (double)q.x);
            ly = fmin(ly, (double)q.y);
            hy = fmax(hy, (double)q.y);
        }
        for (int o = 16; o; o >>= 1) {
            lx = fmin(lx, __shfl_xor_sync(0xffffffffu, lx, o));
            hx = fmax(hx, __shfl_xor_sync(0xffffffffu, hx, o));
            ly = fmin(ly, __shfl_xor_sync(0xffffffffu, ly, o));
            hy = fmax(hy, __shfl_xor_sync(0xffffffffu, hy, o));
        }
        if (lane == 0) {
            const double bias = (double)1e-9f;
            mbr[k] = make_double4(lx - bias, ly - bias, hx + bias, hy + bias);
        }
    }
}

__global__ void k_join_keys(const double4 *__restrict__ mbr, uint32_t n, uint64_t *__restrict__ key,
                            uint32_t *__restrict__ idx) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        key[k] = jkey(mbr[k].x);
        idx[k] = k;
    }
}

// the widest source box (widths are >= 0, so their keys order as the widths)
__global__ void k_join_width(const double4 *__restrict__ mbr, uint32_t n, unsigned long long *__restrict__ wkey) {
    unsigned long long mine = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        mine = max(mine, (unsigned long long)jkey(mbr[k].z - mbr[k].x));
    for (int o = 16; o; o >>= 1) mine = max(mine, __shfl_xor_sync(0xffffffffu, mine, o));
    if ((threadIdx.x & 31) == 0 && mine) atomicMax(wkey, mine);
}

struct JoinArgs {
    const double4 *src;      // source MBRs
    const double4 *tgt;      // target MBRs
    const uint64_t *skey;    // sources' low-x keys, ascending
    const uint32_t *sidx;    // their source indices
    uint32_t ns, nt;
    double expand;
    int geography, self;
    const double *deg;       // longitude degree table (900), geography only
    const unsigned long long *wkey;
};

// Box.cpp:200-214: the target's box widened by the distance (in degrees
// when geography is set), exactly as farm_mbr_join widens it
__device__ __forceinline__ double4 widen(const JoinArgs &a, double4 b) {
    double sx = a.expand, sy = a.expand;
    if (a.geography && a.expand != 0.0) {
        double l = fabs(b.y);
        if (l == 90) l = 89.9;
        int i = (int)(l * 10);
        if (i < 0 || i >= 900) i = 899;  // the reference indexes out of range here
        sx = sx * a.deg[i];
        sy = sy * (360.0 / 40076.0);
    }
    return make_double4(b.x - sx, b.y - sy, b.z + sx, b.w + sy);
}

// Candidate sources of target t: [lo, hi) in the sorted order. The lower
// end allows for the widest source (a source reaching q.x lies at most the
// widest width to its left), widened by a relative 1e-9 for the rounding of
// the widths; the exact test below removes the extra ones.
__device__ __forceinline__ void cand_range(const JoinArgs &a, const double4 &q, uint32_t &lo, uint32_t &hi) {
    const uint64_t wk = *a.wkey;
    const double w = wk ? __longlong_as_double((long long)(wk & 0x7FFFFFFFFFFFFFFFull)) : 0.0;
    const uint64_t klo = jkey(q.x - w - 1e-9 * (w + fabs(q.x)) - 1e-300), khi = jkey(q.z);
    uint32_t l = 0, h = a.ns;
    while (l < h) {
        const uint32_t m = (l + h) >> 1;
        if (a.skey[m] < klo) l = m + 1; else h = m;
    }
    lo = l;
    h = a.ns;
    while (l < h) {
        const uint32_t m = (l + h) >> 1;
        if (a.skey[m] <= khi) l = m + 1; else h = m;
    }
    hi = l;
}

// the host's test: !(a.lo.x > q.hi.x || q.lo.x > a.hi.x || a.lo.y > q.hi.y || q.lo.y > a.hi.y)
__device__ __forceinline__ bool overlap(const double4 &s, const double4 &q) {
    return !(s.x > q.z || q.x > s.z || s.y > q.w || q.y > s.w);
}

__global__ void k_join_count(JoinArgs a, uint64_t *__restrict__ cnt) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < a.nt; t += gridDim.x * blockDim.x) {
        const double4 q = widen(a, a.tgt[t]);
        uint32_t lo, hi;
        cand_range(a, q, lo, hi);
        uint64_t c = 0;
        for (uint32_t k = lo; k < hi; k++) {
            const uint32_t s = a.sidx[k];
            if (a.self && s == t) continue;
            c += overlap(a.src[s], q);
        }
        cnt[t] = c;
    }
}

__global__ void k_join_fill(JoinArgs a, const uint64_t *__restrict__ start, uint64_t *__restrict__ out) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < a.nt; t += gridDim.x * blockDim.x) {
        const double4 q = widen(a, a.tgt[t]);
        uint32_t lo, hi;
        cand_range(a, q, lo, hi);
        uint64_t at = start[t];
        for (uint32_t k = lo; k < hi; k++) {
            const uint32_t s = a.sidx[k];
            if (a.self && s == t) continue;
            if (overlap(a.src[s], q)) out[at++] = ((uint64_t)s << 32) | t;
        }
    }
}

__global__ void k_join_unpack(const uint64_t *__restrict__ key, uint64_t n, uint32_t *__restrict__ pairs) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = key[k];
        pairs[2 * k] = (uint32_t)(v >> 32);
        pairs[2 * k + 1] = (uint32_t)v;
    }
}

static unsigned grid_cap(uint64_t n) {
    uint64_t g = (n + 255) / 256, cap = 16ull * sm_count();
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

static std::mutex g_deg_mu;

int mbr_join_gpu(farm_store *s, double expand, int geography, int self, uint32_t *pairs, uint64_t cap, int mem,
                 uint64_t *n_out) {
    const uint64_t ns = s->n_side[0], nt = self ? s->n_side[0] : s->n_side[1];
    *n_out = 0;
    if (ns == 0 || nt == 0) return FARM_OK;
    cudaStream_t st = s->stream;
    const uint64_t tfirst = self ? 0 : ns;
    // scratch (the query slots: the join runs between loading and querying)
    DevBuf &bm = s->s[Q_SCR0], &bk = s->s[Q_SCR1], &bc = s->s[Q_SCR2], &bo = s->s[Q_SCR3], &bt = s->s[Q_SCR4];
    FARM_TRY(bm.ensure(32 * (ns + nt) + 64));
    double4 *msrc = bm.as<double4>(), *mtgt = self ? msrc : msrc + ns;
    k_join_mbr<<<grid_cap(32 * ns), 256, 0, st>>>(s->d_ring.as<float2>(), s->d_off.as<uint64_t>(), 0, (uint32_t)ns,
                                                  msrc);
    if (!self)
        k_join_mbr<<<grid_cap(32 * nt), 256, 0, st>>>(s->d_ring.as<float2>(), s->d_off.as<uint64_t>(), tfirst,
                                                      (uint32_t)nt, mtgt);
    // sources by low x
    FARM_TRY(bk.ensure(24 * (ns + 1) + 8 * 900 + 64));
    uint64_t *key = bk.as<uint64_t>(), *key_s = key + ns;
    uint32_t *idx = reinterpret_cast<uint32_t *>(key_s + ns), *idx_s = idx + ns;
    double *deg = reinterpret_cast<double *>(idx_s + ns + 2);
    unsigned long long *wkey = reinterpret_cast<unsigned long long *>(deg + 900);
    k_join_keys<<<grid_cap(ns), 256, 0, st>>>(msrc, (uint32_t)ns, key, idx);
    {
        size_t bytes = 0;
        FARM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, key, key_s, idx, idx_s, (int64_t)ns, 0, 64, st));
        FARM_TRY(s->cub_tmp.ensure(bytes + 16));
        FARM_CUDA(cub::DeviceRadixSort::SortPairs(s->cub_tmp.p, bytes, key, key_s, idx, idx_s, (int64_t)ns, 0, 64, st));
    }
    FARM_CUDA(cudaMemsetAsync(wkey, 0, 8, st));
    k_join_width<<<grid_cap(ns), 256, 0, st>>>(msrc, (uint32_t)ns, wkey);
    if (geography) {
        // util.h:73, regenerated from the formula its entries were printed from
        double h[900];
        const double PI = 3.14159265;
        for (int i = 0; i < 900; i++) {
            char buf[64];
            snprintf(buf, sizeof buf, "%.6f", 360.0 / (sin((90 - i / 10.0) * PI / 180) * 40076));
            h[i] = strtod(buf, nullptr);
        }
        std::lock_guard<std::mutex> lock(g_deg_mu);
        FARM_CUDA(cudaMemcpyAsync(deg, h, sizeof h, cudaMemcpyHostToDevice, st));
        FARM_CUDA(cudaStreamSynchronize(st));  // h leaves scope
    }
    JoinArgs a{msrc, mtgt, key_s, idx_s, (uint32_t)ns, (uint32_t)nt, expand, geography, self, deg, wkey};
    FARM_TRY(bc.ensure(16 * (nt + 1) + 64));
    uint64_t *cnt = bc.as<uint64_t>(), *start = cnt + (nt + 1);
    k_join_count<<<grid_cap(nt), 256, 0, st>>>(a, cnt);
    FARM_CUDA(cudaMemsetAsync(cnt + nt, 0, 8, st));
    {
        size_t bytes = 0;
        FARM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, cnt, start, (int64_t)(nt + 1), st));
        FARM_TRY(s->cub_tmp.ensure(bytes + 16));
        FARM_CUDA(cub::DeviceScan::ExclusiveSum(s->cub_tmp.p, bytes, cnt, start, (int64_t)(nt + 1), st));
    }
    uint64_t total = 0;
    FARM_CUDA(cudaMemcpyAsync(&total, start + nt, 8, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    s->launches += self ? 5 : 6;
    *n_out = total;
    if (total > cap) {
        set_error("farm_mbr_join_gpu: " + std::to_string(total) + " candidate pairs exceed the buffer's " +
                  std::to_string(cap));
        return FARM_EOVERFLOW;
    }
    if (!total) return FARM_OK;
    FARM_TRY(bo.ensure(16 * total + 64));
    uint64_t *pk = bo.as<uint64_t>(), *pk_s = pk + total;
    k_join_fill<<<grid_cap(nt), 256, 0, st>>>(a, start, pk);
    {
        size_t bytes = 0;
        FARM_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, bytes, pk, pk_s, (int64_t)total, 0, 64, st));
        FARM_TRY(s->cub_tmp.ensure(bytes + 16));
        FARM_CUDA(cub::DeviceRadixSort::SortKeys(s->cub_tmp.p, bytes, pk, pk_s, (int64_t)total, 0, 64, st));
    }
    uint32_t *dst = pairs;
    if (mem == FARM_MEM_HOST) {
        FARM_TRY(bt.ensure(8 * total + 64));
        dst = bt.as<uint32_t>();
    }
    k_join_unpack<<<grid_cap(total), 256, 0, st>>>(pk_s, total, dst);
    s->launches += 2;
    if (mem == FARM_MEM_HOST) FARM_CUDA(cudaMemcpyAsync(pairs, dst, 8 * total, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_mbr_join_gpu(farm_store *s, double expand, int geography, int target_is_source, uint32_t *pairs,
                                 uint64_t cap, int mem, uint64_t *n) {
    using namespace farm;
    if (!s || !n || (cap && !pairs) || (mem != FARM_MEM_HOST && mem != FARM_MEM_DEVICE)) {
        set_error("invalid arguments to farm_mbr_join_gpu");
        return FARM_EINVAL;
    }
    if (s->n_side[0] == 0 || (!target_is_source && s->n_side[1] == 0)) {
        set_error("farm_mbr_join_gpu: load the source side (and the target side unless target_is_source)");
        return FARM_EINVAL;
    }
    if (s->n_side[0] > 0xFFFFFFFFull || s->n_side[1] > 0xFFFFFFFFull) {
        set_error("farm_mbr_join_gpu: more than 2^32 polygons on one side");
        return FARM_EOVERFLOW;
    }
    return mbr_join_gpu(s, expand, geography, target_is_source, pairs, cap, mem, n);
}
