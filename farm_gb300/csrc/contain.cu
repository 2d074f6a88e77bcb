// Containment queries on the raster store (the reference's Ideal::contain;
// its GPU form, query_contain.cu, is commented out and never launched).
//
//   farm_contain_points: does polygon p hold point q (Ideal::contain(Point &),
//     Ideal.cpp:1101-1157). One thread per (polygon, point) pair: the MBR test
//     (box::contain, Box.cpp:65-70), the pixel's class, and for a BORDER pixel
//     the parity of the pixel's edges whose FP32 crossing abscissa lies in
//     [x, the pixel's right border] plus the nodes below y on the grid line at
//     that border (count_intersection_nodes, Ideal.cpp:988-1006).
//   farm_contain: does source s hold target t (Ideal::contain(Ideal *),
//     Ideal.cpp:1159-1231). One warp per candidate pair, pairs pulled from a
//     global counter: the MBR test, the source pixels' classes over t's MBR
//     window (all OUT: no; all IN: yes), then the pixel pairs under every
//     non-IN source pixel, where an OUT source pixel over an IN target pixel,
//     a target edge of a BORDER pixel crossing the border of an OUT source
//     pixel, or a crossing edge pair of BORDER x BORDER pixels means "no";
//     t's first vertex decides the rest. Every pixel-pair check can only say
//     "no", so visiting the pairs in any order gives the reference's answer.
#include <cstring>
#include <string>

#include "common.cuh"
#include "segments.cuh"

namespace farm {

namespace {

constexpr int kContainWarps = 8;

struct ContainCounters {
    unsigned long long found, pixel_pairs, segment_tests;
};

// Ideal::contain(Point &) on polygon H; (px, py) as float, the reference's Point.
__device__ bool contain_point(const StoreView &sv, const PolyHdr &H, float px, float py) {
    if (!(px >= H.mbr[0] && px <= H.mbr[2] && py >= H.mbr[1] && py <= H.mbr[3])) return false;
    const int cc = sv.category_count;
    const int xo = offset_x(H.mbr, H.step_x, H.dimx, px);
    const int yo = offset_y(H.mbr, H.step_y, H.dimy, py);
    const uint32_t pix = (uint32_t)(yo * H.dimx + xo);
    const int st = show_status(sv.status[H.st + pix], cc);
    if (st == 2) return true;
    if (st == 0) return false;
    const double bx_high = H.mbr[0] + (xo + 1) * H.step_x;
    const uint32_t *off = sv.offset + H.off;
    const uint2 *seq = sv.seq + H.seq;
    const float2 *r = sv.ring + H.ring;
    bool ret = false;
    for (uint32_t q = off[pix]; q < off[pix + 1]; q++) {
        const uint2 sq = seq[q];
        for (uint32_t k = 0; k < sq.y; k++) {
            const float2 a = r[sq.x + k], b = r[sq.x + k + 1];
            if ((a.y >= py) != (b.y >= py)) {
                // every operand is a float, so the reference evaluates the
                // crossing abscissa in FP32, one rounding per operation
                const float ix =
                    __fadd_rn(__fdiv_rn(__fmul_rn(__fsub_rn(b.x, a.x), __fsub_rn(py, a.y)), __fsub_rn(b.y, a.y)), a.x);
                if (px <= ix && (double)ix <= bx_high) ret = !ret;
            }
        }
    }
    // nodes of the grid line at the pixel's right border lying below py: the
    // line's nodes are sorted, so the reference's counting loop stops at the
    // first node >= py, the lower bound of py
    const uint32_t *voff = sv.voff + H.vline;
    const double *vn = sv.vnodes + H.vnode;
    uint32_t lo = voff[xo + 1], hi = voff[xo + 2];
    const uint32_t first = lo;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (vn[mid] < (double)py) lo = mid + 1;
        else hi = mid;
    }
    if ((lo - first) & 1u) ret = !ret;
    return ret;
}

__global__ void k_contain_points(const StoreView sv, uint64_t side_base, const float2 *__restrict__ pts,
                                 const uint32_t *__restrict__ pairs, uint64_t n, uint8_t *__restrict__ out,
                                 ContainCounters *__restrict__ ctr) {
    unsigned long long mine = 0;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 pq = reinterpret_cast<const uint2 *>(pairs)[k];
        const PolyHdr &H = sv.hdr[side_base + pq.x];
        uint8_t v;
        if (H.err) {
            v = 2;
        } else {
            const float2 P = pts[pq.y];
            v = contain_point(sv, H, P.x, P.y) ? 1 : 0;
        }
        out[k] = v;
        mine += v == 1;
    }
    for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&ctr->found, mine);
}

// A target pixel's edges against the border of source pixel box (b0, b1, b2, b3)
// (the five float corners Ideal.cpp:1196-1200 builds): true on any crossing.
// Lanes take the pixel's edges, flattened over its sequences by a warp scan.
__device__ bool edges_cross_box(const StoreView &sv, const PolyHdr &T, uint32_t pb, double b0, double b1, double b2,
                                double b3, unsigned long long &tests) {
    const int lane = threadIdx.x & 31;
    const float2 c0 = make_float2((float)b0, (float)b1), c1 = make_float2((float)b0, (float)b3);
    const float2 c2 = make_float2((float)b2, (float)b3), c3 = make_float2((float)b2, (float)b1);
    const uint32_t *to = sv.offset + T.off;
    const uint2 *tseq = sv.seq + T.seq;
    const float2 *tr = sv.ring + T.ring;
    const uint32_t q0 = to[pb], q1 = to[pb + 1];
    for (uint32_t g = q0; g < q1; g += 32) {
        const uint32_t k = g + lane;
        const uint2 r = k < q1 ? tseq[k] : make_uint2(0u, 0u);
        uint32_t total;
        const uint32_t excl = warp_excl_scan(r.y, lane, total);
        for (uint32_t sb = 0; sb < total; sb += 32) {
            const uint32_t f = sb + lane;
            bool hit = false;
            const int owner = warp_owner(excl, f);
            const uint32_t ostart = __shfl_sync(0xffffffffu, r.x, owner);
            const uint32_t oex = __shfl_sync(0xffffffffu, excl, owner);
            if (f < total) {
                const float2 a = tr[ostart + (f - oex)], b = tr[ostart + (f - oex) + 1];
                hit = seg_intersect(a, b, c0, c1) || seg_intersect(a, b, c1, c2) || seg_intersect(a, b, c2, c3) ||
                      seg_intersect(a, b, c3, c0);
                tests += 4;
            }
            if (__any_sync(0xffffffffu, hit)) return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(kContainWarps * 32)
    k_contain(const StoreView sv, const uint32_t *__restrict__ pairs, uint64_t n, uint64_t tgt_base,
              unsigned long long *__restrict__ next, uint8_t *__restrict__ out, ContainCounters *__restrict__ ctr) {
    __shared__ float4 tbufs[kContainWarps][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float4 *tb = tbufs[wib];
    const int cc = sv.category_count;
    unsigned long long my_found = 0, my_pp = 0, my_tests = 0;
    for (;;) {
        unsigned long long pid = 0;
        if (lane == 0) pid = atomicAdd(next, 1ull);
        pid = __shfl_sync(0xffffffffu, pid, 0);
        if (pid >= n) break;
        const uint32_t s = pairs[2 * pid], t = pairs[2 * pid + 1];
        const PolyHdr &S = sv.hdr[s];
        const PolyHdr &T = sv.hdr[tgt_base + t];
        if (S.err || T.err) {
            if (lane == 0) out[pid] = 2;
            continue;
        }
        // box::contain(box) (Box.cpp:59-64) of the MBRs
        if (!(T.mbr[0] >= S.mbr[0] && T.mbr[2] <= S.mbr[2] && T.mbr[1] >= S.mbr[1] && T.mbr[3] <= S.mbr[3])) {
            if (lane == 0) out[pid] = 0;
            continue;
        }
        const uint8_t *sst = sv.status + S.st, *tst = sv.status + T.st;
        const Window w = retrieve(S.mbr, S.step_x, S.step_y, S.dimx, S.dimy, T.mbr[0], T.mbr[1], T.mbr[2], T.mbr[3]);
        const int wh = w.ey - w.sy + 1;
        const long nw = (w.ex >= w.sx && w.ey >= w.sy) ? (long)(w.ex - w.sx + 1) * wh : 0;
        // the window's OUT and IN counts
        long n_out = 0, n_in = 0;
        for (long base = 0; base < nw; base += 32) {
            const long k = base + lane;
            int st = 1;
            if (k < nw) st = show_status(sst[(w.sy + (int)(k % wh)) * S.dimx + w.sx + (int)(k / wh)], cc);
            n_out += __popc(__ballot_sync(0xffffffffu, k < nw && st == 0));
            n_in += __popc(__ballot_sync(0xffffffffu, k < nw && st == 2));
        }
        int result;
        if (n_out == nw) {
            result = 0;
        } else if (n_in == nw) {
            result = 1;
        } else {
            bool violated = false;
            for (long base = 0; base < nw && !violated; base += 32) {
                // one source window pixel per lane (x outer, y inner); IN
                // pixels are skipped
                const long k = base + lane;
                int tw_sx = 0, tw_sy = 0, tw_ey = -1;
                uint32_t pa = 0, cnt = 0;
                int pa_st = 2;
                double b0 = 0, b1 = 0, b2 = 0, b3 = 0;
                if (k < nw) {
                    const int i = w.sx + (int)(k / wh), j = w.sy + (int)(k % wh);
                    pa = (uint32_t)(j * S.dimx + i);
                    pa_st = show_status(sst[pa], cc);
                    if (pa_st != 2) {
                        b0 = S.mbr[0] + i * S.step_x;
                        b1 = S.mbr[1] + j * S.step_y;
                        b2 = S.mbr[0] + (i + 1) * S.step_x;
                        b3 = S.mbr[1] + (j + 1) * S.step_y;
                        const Window tw = retrieve(T.mbr, T.step_x, T.step_y, T.dimx, T.dimy, b0, b1, b2, b3);
                        if (tw.ex >= tw.sx && tw.ey >= tw.sy) {
                            tw_sx = tw.sx;
                            tw_sy = tw.sy;
                            tw_ey = tw.ey;
                            cnt = (uint32_t)((tw.ex - tw.sx + 1) * (tw.ey - tw.sy + 1));
                        }
                    }
                }
                uint32_t total;
                const uint32_t excl = warp_excl_scan(cnt, lane, total);
                for (uint32_t f = 0; f < total && !violated; f += 32) {
                    const uint32_t item = f + lane;
                    const int owner = warp_owner(excl, item);
                    const uint32_t o_excl = __shfl_sync(0xffffffffu, excl, owner);
                    const int o_sx = __shfl_sync(0xffffffffu, tw_sx, owner);
                    const int o_sy = __shfl_sync(0xffffffffu, tw_sy, owner);
                    const int o_ey = __shfl_sync(0xffffffffu, tw_ey, owner);
                    const int o_st = __shfl_sync(0xffffffffu, pa_st, owner);
                    bool out_in = false, ob = false, bb = false;
                    uint32_t pb = 0;
                    if (item < total) {
                        const uint32_t r = item - o_excl;
                        const int th = o_ey - o_sy + 1;
                        const int u = o_sx + (int)(r / (uint32_t)th), v = o_sy + (int)(r % (uint32_t)th);
                        pb = (uint32_t)(v * T.dimx + u);
                        const int pb_st = show_status(tst[pb], cc);
                        out_in = o_st == 0 && pb_st == 2;
                        ob = o_st == 0 && pb_st == 1;
                        bb = o_st == 1 && pb_st == 1;
                    }
                    if (__any_sync(0xffffffffu, out_in)) {
                        violated = true;
                        break;
                    }
                    // pixel pairs that need edges: the whole warp takes one at a time
                    for (unsigned m = __ballot_sync(0xffffffffu, ob || bb); m && !violated; m &= m - 1) {
                        const int src = __ffs(m) - 1;
                        const uint32_t qb = __shfl_sync(0xffffffffu, pb, src);
                        const bool q_ob = __shfl_sync(0xffffffffu, ob, src);
                        const int ow = __shfl_sync(0xffffffffu, owner, src);
                        const uint32_t qa = __shfl_sync(0xffffffffu, pa, ow);
                        if (lane == 0) my_pp++;
                        if (q_ob) {
                            const double e0 = __shfl_sync(0xffffffffu, b0, ow), e1 = __shfl_sync(0xffffffffu, b1, ow);
                            const double e2 = __shfl_sync(0xffffffffu, b2, ow), e3 = __shfl_sync(0xffffffffu, b3, ow);
                            violated = edges_cross_box(sv, T, qb, e0, e1, e2, e3, my_tests);
                        } else {
                            violated = refine_pixel_pair(sv, S, T, qa, qb, tb, my_tests);
                        }
                    }
                }
            }
            if (violated) {
                result = 0;
            } else {
                // t's first vertex (Ideal.cpp:1228-1230)
                bool in = false;
                if (lane == 0) {
                    const float2 p0 = sv.ring[T.ring];
                    in = contain_point(sv, S, p0.x, p0.y);
                }
                result = __shfl_sync(0xffffffffu, in, 0) ? 1 : 0;
            }
        }
        if (lane == 0) {
            out[pid] = (uint8_t)result;
            my_found += result == 1;
        }
        __syncwarp();
    }
    for (int o = 16; o; o >>= 1) my_tests += __shfl_xor_sync(0xffffffffu, my_tests, o);
    if (lane == 0) {
        atomicAdd(&ctr->found, my_found);
        atomicAdd(&ctr->pixel_pairs, my_pp);
        atomicAdd(&ctr->segment_tests, my_tests);
    }
}

}  // namespace

}  // namespace farm

using namespace farm;

extern "C" int farm_contain(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint8_t *out, uint64_t *found,
                            farm_stats *st) {
    if (!s || (n && (!pairs || !out))) {
        set_error("invalid arguments to farm_contain");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("farm_contain: rasterize first");
        return FARM_EINVAL;
    }
    if (s->n_side[1] == 0) {
        set_error("farm_contain: no target side loaded");
        return FARM_EINVAL;
    }
    FARM_TRY(check_pairs(s, pairs, n, mem, false, "farm_contain"));
    cudaStream_t stream = s->stream;
    const uint32_t *dpairs = pairs;
    uint8_t *dout = out;
    if (mem == FARM_MEM_HOST && n) {
        FARM_TRY(s->d_pairs.ensure(8 * n));
        FARM_CUDA(cudaMemcpyAsync(s->d_pairs.p, pairs, 8 * n, cudaMemcpyHostToDevice, stream));
        dpairs = s->d_pairs.as<uint32_t>();
        FARM_TRY(s->d_out.ensure(n + 16));
        dout = s->d_out.as<uint8_t>();
    }
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *next = s->d_counters.as<unsigned long long>();
    ContainCounters *ctr = reinterpret_cast<ContainCounters *>(next + 1);
    FARM_CUDA(cudaMemsetAsync(next, 0, 8 + sizeof(ContainCounters), stream));
    FARM_CUDA(cudaEventRecord(s->ev[6], stream));
    if (n) {
        k_contain<<<sm_count() * 8, kContainWarps * 32, 0, stream>>>(s->view(), dpairs, n, s->n_side[0], next, dout,
                                                                     ctr);
        FARM_CUDA(cudaGetLastError());
        s->launches++;
    }
    FARM_CUDA(cudaEventRecord(s->ev[7], stream));
    ContainCounters h{};
    FARM_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && n) FARM_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    if (found) *found = h.found;
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        st->found = h.found;
        st->border_pairs = h.pixel_pairs;
        st->segment_tests = h.segment_tests;
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[6], s->ev[7]);
        st->ms_total = ms;
        st->ms_stage[2] = ms;
        st->kernel_launches = n ? 1 : 0;
    }
    return FARM_OK;
}

extern "C" int farm_contain_points(farm_store *s, int side, const float *xy, uint64_t npoints, const uint32_t *pairs,
                                   uint64_t n, int mem, uint8_t *out, uint64_t *found) {
    if (!s || side < 0 || side > 1 || (n && (!pairs || !out || !xy))) {
        set_error("invalid arguments to farm_contain_points");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("farm_contain_points: rasterize first");
        return FARM_EINVAL;
    }
    FARM_TRY(check_pair_limits(s, pairs, n, mem, s->n_side[side], npoints, "farm_contain_points", "polygons",
                               "points"));
    if (mem == FARM_MEM_DEVICE && n && (reinterpret_cast<uintptr_t>(xy) & 7u)) {
        // the kernel reads whole (x, y) pairs: 8-byte loads
        set_error("farm_contain_points: device points must start on an 8-byte boundary");
        return FARM_EINVAL;
    }
    cudaStream_t stream = s->stream;
    const uint32_t *dpairs = pairs;
    const float2 *dpts = reinterpret_cast<const float2 *>(xy);
    uint8_t *dout = out;
    if (mem == FARM_MEM_HOST && n) {
        FARM_TRY(s->d_pairs.ensure(8 * n));
        FARM_CUDA(cudaMemcpyAsync(s->d_pairs.p, pairs, 8 * n, cudaMemcpyHostToDevice, stream));
        dpairs = s->d_pairs.as<uint32_t>();
        FARM_TRY(s->d_points.ensure(8 * npoints + 16));
        FARM_CUDA(cudaMemcpyAsync(s->d_points.p, xy, 8 * npoints, cudaMemcpyHostToDevice, stream));
        dpts = s->d_points.as<float2>();
        FARM_TRY(s->d_out.ensure(n + 16));
        dout = s->d_out.as<uint8_t>();
    }
    FARM_TRY(s->d_counters.ensure(256));
    ContainCounters *ctr = reinterpret_cast<ContainCounters *>(s->d_counters.as<unsigned long long>() + 1);
    FARM_CUDA(cudaMemsetAsync(ctr, 0, sizeof(ContainCounters), stream));
    if (n) {
        unsigned blocks = grid_for(n, 256);
        if (blocks > 16u * (unsigned)sm_count()) blocks = 16u * (unsigned)sm_count();
        k_contain_points<<<blocks, 256, 0, stream>>>(s->view(), side == 0 ? 0 : s->n_side[0], dpts, dpairs, n, dout,
                                                     ctr);
        FARM_CUDA(cudaGetLastError());
        s->launches++;
    }
    ContainCounters h{};
    FARM_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && n) FARM_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    if (found) *found = h.found;
    return FARM_OK;
}
