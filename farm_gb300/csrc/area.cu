// Stage (d): FP64 intersection area of candidate pairs.
//
// The reference stops before computing any area (Ideal.cpp:1683; its GPU
// rebuild step is never launched, query_intersection.cu:724-737), so this is
// the project's own formulation, checked against the FP64 CPU oracle.
//
// Boundary integral: area(A n B) = 1/2 * [ integral over the parts of dA inside
// B + over the parts of dB inside A ] of (x dy - y dx), each boundary taken
// with its own orientation sign. Along a straight edge P -> Q (d = Q - P) the
// integrand is the constant P x d per unit of the edge parameter, so an edge
// contributes (P x d) * (total parameter length of its inside parts). Those
// parts are delimited by the edge's crossings with the other boundary; the
// state at a chunk's first vertex comes from one point-in-polygon test on the
// other polygon's raster, and flips at each crossing after it.
//
// Work: items are (pair, side, chunk of that side's edges), taken by persistent
// warps from a global counter. A lane takes one edge: it finds its crossings
// through the other polygon's raster (edge sequences of the BORDER pixels
// around the edge), ranks them, and adds its signed inside length. Per-item
// partial sums are reduced per pair in a fixed order (deterministic results).
// Coordinates are taken relative to the pair's source first vertex.
// General position is assumed (no collinear overlaps, no crossing exactly at a
// vertex); crossings at a shared vertex are counted once by half-open ranges.
#include <cub/cub.cuh>

#include <cstring>

#include "common.cuh"

namespace farm {

struct AreaArgs {
    const uint32_t *pairs;
    uint64_t n;
    uint64_t tgt_base;
    uint32_t chunk;              // edges per item
    const uint64_t *item_start;  // per pair: first item (n + 1)
    uint64_t nitems;
    double *partial;             // per item
    const int8_t *orient;        // per polygon: +1 counter-clockwise, -1 clockwise
    unsigned long long *next;
    unsigned long long *overflow;
};

constexpr int kMaxCross = 48;

__device__ __forceinline__ double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// Point-in-polygon of (px, py) for polygon H through its raster: a ray to the
// right along the pixel row; the first non-BORDER pixel tells its side, edges
// of BORDER pixels before it flip the parity (each edge counted in the pixel
// whose x-range holds its crossing).
__device__ bool pip_raster(const StoreView &sv, const PolyHdr &H, double px, double py, int cc) {
    if (px < H.mbr[0] || px > H.mbr[2] || py < H.mbr[1] || py > H.mbr[3]) return false;
    int row = offset_y(H.mbr, H.step_y, H.dimy, py);
    int col = offset_x(H.mbr, H.step_x, H.dimx, px);
    const uint8_t *st = sv.status + H.st;
    const uint32_t *off = sv.offset + H.off;
    const uint2 *seq = sv.seq + H.seq;
    const float2 *r = sv.ring + H.ring;
    bool odd = false;
    for (int c = col; c < H.dimx; c++) {
        uint32_t pid = (uint32_t)(row * H.dimx + c);
        int s = show_status(st[pid], cc);
        if (s != 1) return c == col ? (s == 2) : (odd ^ (s == 2));
        double x_lo = c == col ? -1e300 : H.mbr[0] + c * H.step_x;
        double x_hi = c == H.dimx - 1 ? 1e300 : H.mbr[0] + (c + 1) * H.step_x;
        for (uint32_t q = off[pid]; q < off[pid + 1]; q++) {
            uint2 sq = seq[q];
            for (uint32_t k = 0; k < sq.y; k++) {
                float2 a = r[sq.x + k], b = r[sq.x + k + 1];
                if ((a.y > py) != (b.y > py)) {
                    double xi = (double)a.x + (py - a.y) * ((double)b.x - a.x) / ((double)b.y - a.y);
                    if (xi > px && xi >= x_lo && xi < x_hi) odd = !odd;
                }
            }
        }
    }
    return odd;  // past the raster: outside, so the crossings decide
}

// Edges of polygon O that may cross segment (P, Q): sequences of O's BORDER
// pixels in a one-pixel-padded window around the segment. Calls f(edge index).
template <typename F>
__device__ void for_candidate_edges(const StoreView &sv, const PolyHdr &O, double x0, double y0, double x1, double y1,
                                    int cc, F f) {
    double mnx = fmin(x0, x1), mxx = fmax(x0, x1), mny = fmin(y0, y1), mxy = fmax(y0, y1);
    if (mxx < O.mbr[0] || mnx > O.mbr[2] || mxy < O.mbr[1] || mny > O.mbr[3]) return;
    int sx = offset_x(O.mbr, O.step_x, O.dimx, mnx) - 1, ex = offset_x(O.mbr, O.step_x, O.dimx, mxx) + 1;
    int sy = offset_y(O.mbr, O.step_y, O.dimy, mny) - 1, ey = offset_y(O.mbr, O.step_y, O.dimy, mxy) + 1;
    sx = sx < 0 ? 0 : sx;
    sy = sy < 0 ? 0 : sy;
    ex = ex >= O.dimx ? O.dimx - 1 : ex;
    ey = ey >= O.dimy ? O.dimy - 1 : ey;
    const uint8_t *st = sv.status + O.st;
    const uint32_t *off = sv.offset + O.off;
    const uint2 *seq = sv.seq + O.seq;
    for (int y = sy; y <= ey; y++)
        for (int x = sx; x <= ex; x++) {
            uint32_t pid = (uint32_t)(y * O.dimx + x);
            if (show_status(st[pid], cc) != 1) continue;
            for (uint32_t q = off[pid]; q < off[pid + 1]; q++) {
                uint2 sq = seq[q];
                for (uint32_t k = 0; k < sq.y; k++) f(sq.x + k);
            }
        }
}

// Crossing parameter t of segment p -> p + d with edge e of ring r, in [0, 1)
// on both (half-open, so a crossing at a shared vertex counts once).
__device__ __forceinline__ bool crossing(double px, double py, double dx, double dy, const float2 *r, uint32_t e,
                                         double ox, double oy, double &t, double &den) {
    float2 a = r[e], b = r[e + 1];
    double ax = (double)a.x - ox, ay = (double)a.y - oy;
    double gx = (double)b.x - a.x, gy = (double)b.y - a.y;
    if (gx == 0 && gy == 0) return false;
    den = cross2(dx, dy, gx, gy);
    if (den == 0) return false;
    double rx = ax - px, ry = ay - py;
    t = cross2(rx, ry, gx, gy) / den;
    double u = cross2(rx, ry, dx, dy) / den;
    return t >= 0 && t < 1 && u >= 0 && u < 1;
}

__global__ void __launch_bounds__(256) k_area(const StoreView sv, AreaArgs a) {
    const int lane = threadIdx.x & 31;
    const int cc = sv.category_count;
    for (;;) {
        unsigned long long it = 0;
        if (lane == 0) it = atomicAdd(a.next, 1ull);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= a.nitems) break;
        uint32_t p = find_segment(a.item_start, (uint32_t)a.n, it);
        uint64_t rel = it - a.item_start[p];
        const PolyHdr &S = sv.hdr[a.pairs[2 * p]];
        const PolyHdr &T = sv.hdr[a.tgt_base + a.pairs[2 * p + 1]];
        uint32_t es = S.nv - 1, et = T.nv - 1;  // edges (the ring's last edge is the zero-length closing one)
        uint64_t cs = (es + a.chunk - 1) / a.chunk;
        bool side_t = rel >= cs;
        const PolyHdr &M = side_t ? T : S;  // the boundary integrated
        const PolyHdr &O = side_t ? S : T;  // the polygon it is clipped by
        uint32_t first = (uint32_t)((side_t ? rel - cs : rel) * a.chunk);
        uint32_t me = side_t ? et : es;
        uint32_t last = first + a.chunk < me ? first + a.chunk : me;
        const float2 *mr = sv.ring + M.ring, *orr = sv.ring + O.ring;
        const float2 o0 = sv.ring[S.ring];
        const double ox = o0.x, oy = o0.y;
        const double sign = a.orient[side_t ? a.tgt_base + a.pairs[2 * p + 1] : a.pairs[2 * p]];
        // state at the chunk's first vertex
        bool in0 = false;
        if (lane == 0) in0 = pip_raster(sv, O, mr[first].x, mr[first].y, cc);
        in0 = __shfl_sync(0xffffffffu, in0, 0);
        double acc = 0;
        bool state = in0;
        // a crossing leaves O when O's edge turns the way O's interior lies:
        // entering iff (d x g) has the opposite sign of O's orientation
        const double osign = a.orient[side_t ? a.pairs[2 * p] : a.tgt_base + a.pairs[2 * p + 1]];
        for (uint32_t b0 = first; b0 < last; b0 += 32) {
            uint32_t e = b0 + lane;
            bool valid = e < last;
            double px = 0, py = 0, dx = 0, dy = 0;
            double sum_t = 0;  // leaving t minus entering t
            int nc = 0;
            if (valid) {
                float2 P = mr[e], Q = mr[e + 1];
                px = (double)P.x - ox;
                py = (double)P.y - oy;
                dx = (double)Q.x - P.x;
                dy = (double)Q.y - P.y;
                if (dx != 0 || dy != 0) {
                    // an edge of O may be listed by several pixels: count it once
                    uint32_t seen[kMaxCross];
                    int ns = 0;
                    bool slow = false;
                    for_candidate_edges(sv, O, P.x, P.y, Q.x, Q.y, cc, [&](uint32_t f) {
                        double t, den;
                        if (slow || !crossing(px, py, dx, dy, orr, f, ox, oy, t, den)) return;
                        for (int q = 0; q < ns; q++)
                            if (seen[q] == f) return;
                        if (ns == kMaxCross) {
                            slow = true;
                            return;
                        }
                        seen[ns++] = f;
                        nc++;
                        sum_t += (osign * den > 0) ? t : -t;
                    });
                    if (slow) {
                        // many crossings: find earlier listings of the same edge by re-enumeration
                        nc = 0;
                        sum_t = 0;
                        uint64_t pos = 0;
                        for_candidate_edges(sv, O, P.x, P.y, Q.x, Q.y, cc, [&](uint32_t f) {
                            uint64_t mine = pos++;
                            double t, den;
                            if (!crossing(px, py, dx, dy, orr, f, ox, oy, t, den)) return;
                            bool dup = false;
                            uint64_t p2 = 0;
                            for_candidate_edges(sv, O, P.x, P.y, Q.x, Q.y, cc, [&](uint32_t g) {
                                if (p2++ < mine && g == f) dup = true;
                            });
                            if (dup) return;
                            nc++;
                            sum_t += (osign * den > 0) ? t : -t;
                        });
                    }
                }
            }
            // parity of crossings of earlier edges of the chunk
            unsigned odd = __ballot_sync(0xffffffffu, valid && (nc & 1));
            bool s_here = state ^ (__popc(odd & ((1u << lane) - 1)) & 1);
            if (valid) {
                double len = sum_t + ((s_here ^ (nc & 1)) ? 1.0 : 0.0);
                acc += cross2(px, py, dx, dy) * len;
            }
            state ^= (__popc(odd) & 1);
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) a.partial[it] = 0.5 * sign * acc;
    }
}

// orientation sign of every polygon (shoelace about its first vertex)
__global__ void k_orient(const StoreView sv, uint32_t npoly, int8_t *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = w; p < npoly; p += nw) {
        const PolyHdr &h = sv.hdr[p];
        const float2 *r = sv.ring + h.ring;
        double ox = r[0].x, oy = r[0].y, sa = 0;
        for (uint32_t k = lane; k + 1 < h.nv; k += 32)
            sa += cross2((double)r[k].x - ox, (double)r[k].y - oy, (double)r[k + 1].x - ox, (double)r[k + 1].y - oy);
        for (int o = 16; o; o >>= 1) sa += __shfl_xor_sync(0xffffffffu, sa, o);
        if (lane == 0) out[p] = sa >= 0 ? 1 : -1;
    }
}

__global__ void k_area_items(const StoreView sv, const uint32_t *__restrict__ pairs, uint64_t n, uint64_t tgt_base,
                             uint32_t chunk, uint64_t *__restrict__ cnt) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= n; k += (uint64_t)gridDim.x * blockDim.x) {
        if (k == n) {
            cnt[k] = 0;
            continue;
        }
        const PolyHdr &S = sv.hdr[pairs[2 * k]];
        const PolyHdr &T = sv.hdr[tgt_base + pairs[2 * k + 1]];
        if (S.err || T.err) {
            cnt[k] = 0;
            continue;
        }
        uint32_t es = S.nv - 1, et = T.nv - 1;
        cnt[k] = (es + chunk - 1) / chunk + (et + chunk - 1) / chunk;
    }
}

// fixed-order sum of each pair's item partials
__global__ void k_area_reduce(const uint64_t *__restrict__ item_start, uint64_t n, const double *__restrict__ partial,
                              const StoreView sv, const uint32_t *__restrict__ pairs, uint64_t tgt_base,
                              double *__restrict__ out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const PolyHdr &S = sv.hdr[pairs[2 * k]];
        const PolyHdr &T = sv.hdr[tgt_base + pairs[2 * k + 1]];
        if (S.err || T.err) {
            out[k] = nan("");
            continue;
        }
        double s = 0;
        for (uint64_t i = item_start[k]; i < item_start[k + 1]; i++) s += partial[i];
        out[k] = fabs(s);
    }
}

int intersection_area(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, double *out, farm_stats *st) {
    if (!s->rasterized) {
        set_error("farm_intersection_area: rasterize first");
        return FARM_EINVAL;
    }
    if (s->n_side[1] == 0) {
        set_error("farm_intersection_area: no target side loaded");
        return FARM_EINVAL;
    }
    cudaStream_t stream = s->stream;
    const uint64_t tgt_base = s->n_side[0];
    const uint32_t *dpairs = pairs;
    if (mem == FARM_MEM_HOST && n) {
        FARM_TRY(s->d_pairs.ensure(8 * n));
        FARM_CUDA(cudaMemcpyAsync(s->d_pairs.p, pairs, 8 * n, cudaMemcpyHostToDevice, stream));
        dpairs = s->d_pairs.as<uint32_t>();
    }
    double *dout = out;
    if (mem == FARM_MEM_HOST || !out) {
        FARM_TRY(s->d_out.ensure(8 * n + 64));
        dout = s->d_out.as<double>();
    }
    StoreView sv = s->view();
    const uint32_t chunk = 256;
    DevBuf &cnt = s->s[26], &start = s->s[27], &part = s->s[28], &tmp = s->cub_tmp;
    FARM_TRY(cnt.ensure(8 * (n + 1) + 64));
    FARM_TRY(start.ensure(8 * (n + 1) + 64));
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *ctr = s->d_counters.as<unsigned long long>();
    FARM_CUDA(cudaMemsetAsync(ctr, 0, 64, stream));
    FARM_CUDA(cudaEventRecord(s->ev[6], stream));
    unsigned blocks = (unsigned)((n + 256) / 256);
    if (blocks > 4096) blocks = 4096;
    k_area_items<<<blocks, 256, 0, stream>>>(sv, dpairs, n, tgt_base, chunk, cnt.as<uint64_t>());
    size_t bytes = 0;
    FARM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, cnt.as<uint64_t>(), start.as<uint64_t>(), (int64_t)(n + 1),
                                            stream));
    FARM_TRY(tmp.ensure(bytes + 64));
    FARM_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, bytes, cnt.as<uint64_t>(), start.as<uint64_t>(), (int64_t)(n + 1),
                                            stream));
    uint64_t nitems = 0;
    FARM_CUDA(cudaMemcpyAsync(&nitems, start.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    FARM_TRY(part.ensure(8 * nitems + 64));
    DevBuf &ori = s->s[29];
    FARM_TRY(ori.ensure(s->n_poly + 64));
    {
        unsigned ob = (unsigned)((32ull * s->n_poly + 255) / 256);
        if (ob > 8192) ob = 8192;
        k_orient<<<ob, 256, 0, stream>>>(sv, (uint32_t)s->n_poly, ori.as<int8_t>());
    }
    AreaArgs aa{dpairs, n, tgt_base, chunk, start.as<uint64_t>(), nitems, part.as<double>(), ori.as<int8_t>(), ctr,
                ctr + 1};
    if (nitems) k_area<<<sm_count() * 8, 256, 0, stream>>>(sv, aa);
    k_area_reduce<<<blocks, 256, 0, stream>>>(start.as<uint64_t>(), n, part.as<double>(), sv, dpairs, tgt_base, dout);
    FARM_CUDA(cudaGetLastError());
    FARM_CUDA(cudaEventRecord(s->ev[7], stream));
    unsigned long long over = 0;
    FARM_CUDA(cudaMemcpyAsync(&over, ctr + 1, 8, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && out && n) FARM_CUDA(cudaMemcpyAsync(out, dout, 8 * n, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    s->launches += 4 + (nitems ? 1 : 0);
    (void)over;
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[6], s->ev[7]);
        st->ms_total = ms;
        st->ms_stage[2] = ms;
        st->kernel_launches = 4 + (nitems ? 1 : 0);
    }
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_intersection_area(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, double *out,
                                      farm_stats *st) {
    using namespace farm;
    if (!s || (n && !pairs)) {
        set_error("invalid arguments to farm_intersection_area");
        return FARM_EINVAL;
    }
    return intersection_area(s, pairs, n, mem, out, st);
}
