// Segment predicates and the warp-cooperative pixel-pair refinement shared
// by the intersect and contain queries.
//
//   segment_intersect (geometry_computation.h:215-221) with Point::cross
//   (Point.h:93-97) in FP32 without fused multiply-add, inter1
//   (geometry_computation.h:195-212), retrieve_pixels (MyRaster.cpp:332-346)
//   and segment_intersect_batch over two pixels' edge sequences
//   (geometry_computation.h:224-237).
#pragma once

#include "common.cuh"

namespace farm {

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

__device__ __forceinline__ int sgn_code(float v) { return (v > 0.f) - (v < 0.f); }

// (b - o) x (p - o) with e = b - o precomputed: the same roundings as cross3(o, b, p)
__device__ __forceinline__ float cross_e(float2 o, float ex, float ey, float2 p) {
    return __fsub_rn(__fmul_rn(ex, __fsub_rn(p.y, o.y)), __fmul_rn(ey, __fsub_rn(p.x, o.x)));
}

__device__ __forceinline__ bool inter1f(float a, float b, float c, float d) {
    return fmaxf(fminf(a, b), fminf(c, d)) <= fminf(fmaxf(a, b), fmaxf(c, d));
}

// exclusive warp scan of cnt; total of all lanes in `total`
__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t cnt, int lane, uint32_t &total) {
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - cnt;
}

// the last lane whose exclusive prefix is <= item (the lane that owns item)
__device__ __forceinline__ int warp_owner(uint32_t excl, uint32_t item) {
    int owner = 0;
#pragma unroll
    for (int b = 16; b; b >>= 1) {
        int cand = owner + b;
        uint32_t ex = __shfl_sync(0xffffffffu, excl, cand);
        if (ex <= item) owner = cand;
    }
    return owner;
}

// Refine one BORDER x BORDER pixel pair: true iff some segment of the source
// pixel's edge sequences intersects some segment of the target pixel's
// (segment_intersect_batch over every sequence pair, geometry_computation.h:
// 215-237; the reference stops at the first hit, so the set of segment pairs
// it tests differs only in where it stops, and the boolean is the same).
//
// Whole-warp tile: each lane holds one source segment (a, b) (sequences of the
// pixel flattened by a warp scan), and the warp walks the target pixel's
// vertices in order, 32 at a time staged in shared memory and read as
// broadcasts. segment_intersect's four cross products are shared along the
// walk without changing a single rounding:
//   a.cross(b, c) = cross3(a, b, c) is computed once per target vertex c and
//     reused for the two target segments that end at c;
//   c.cross(a, d) = -(c.cross(d, a)) exactly (the two products are the same
//     IEEE products and round-to-nearest is symmetric), so the collinear test
//     c.cross(a,d) == 0 && c.cross(b,d) == 0 reads the sign codes of
//     c.cross(d, a) and c.cross(d, b) that the general test needs anyway;
//   for the target segment c -> d, c.cross(d, a) = (d-c) x (a-c) takes the
//     differences a - c, which are the exact negations of the differences
//     c - a the lane formed one vertex earlier for a.cross(b, c); the lane
//     keeps c - a and c - b and evaluates (d-c) x (c-a), the same products
//     and difference negated, so its sign code is the reference's negated;
//   the target segment's own d - c is formed once, by the lane that stages d.
// A group of R < 32 source segments (a pixel's last group, or a small pixel)
// would leave lanes idle for the whole target walk, so the group is repeated
// across G = floor(32 / R) slices of lanes and each slice walks its share of
// every staged chunk of target vertices, starting from the vertex before its
// share. Every (source segment, target segment) pair is still tested once.
// Collinear cases are rare; a chunk that has one (in a valid lane) is walked
// again with the interval test (inter1, geometry_computation.h:195-212).
// tbuf holds 32 float4 per warp: the vertex and its difference from the
// vertex before it.
static __device__ bool refine_pixel_pair(const StoreView &sv, const PolyHdr &S, const PolyHdr &T, uint32_t pa,
                                         uint32_t pb, float4 *tbuf, unsigned long long &tests) {
    const int lane = threadIdx.x & 31;
    const uint32_t *so = sv.offset + S.off, *to = sv.offset + T.off;
    const uint32_t a0 = so[pa], a1 = so[pa + 1], b0 = to[pb], b1 = to[pb + 1];
    const uint2 *sseq = sv.seq + S.seq, *tseq = sv.seq + T.seq;
    const float2 *sr = sv.ring + S.ring, *tr = sv.ring + T.ring;
    for (uint32_t g = a0; g < a1; g += 32) {
        const uint32_t k = g + lane;
        const uint2 r = k < a1 ? sseq[k] : make_uint2(0u, 0u);
        uint32_t total;
        const uint32_t excl = warp_excl_scan(r.y, lane, total);  // r.y segments per sequence
        for (uint32_t sb = 0; sb < total; sb += 32) {
            // this group's R source segments, repeated over G slices of lanes
            const uint32_t R = min(32u, total - sb);
            const uint32_t G = 32u / R;
            const uint32_t slice = (uint32_t)lane / R;
            const uint32_t f = sb + (uint32_t)lane % R;
            const bool valid = slice < G;
            const int owner = warp_owner(excl, f);
            const uint32_t ostart = __shfl_sync(0xffffffffu, r.x, owner);
            const uint32_t oex = __shfl_sync(0xffffffffu, excl, owner);
            float2 a = make_float2(0.f, 0.f), b = a;
            if (valid) {
                a = sr[ostart + (f - oex)];
                b = sr[ostart + (f - oex) + 1];
            }
            const float ex = __fsub_rn(b.x, a.x), ey = __fsub_rn(b.y, a.y);
            bool hit = false;
            float2 cp = make_float2(0.f, 0.f);  // last vertex of the previous chunk (warp-uniform)
            bool pseg = false;                  // it starts a segment
            for (uint32_t tg = b0; tg < b1; tg += 32) {
                const uint32_t kk = tg + lane;
                const uint2 r2 = kk < b1 ? tseq[kk] : make_uint2(0u, 0u);
                uint32_t total2;
                const uint32_t excl2 = warp_excl_scan(kk < b1 ? r2.y + 1 : 0u, lane, total2);  // vertices
                for (uint32_t tb = 0; tb < total2; tb += 32) {
                    const uint32_t f2 = tb + lane;
                    const bool v2 = f2 < total2;
                    const int o2 = warp_owner(excl2, f2);
                    const uint32_t o_start = __shfl_sync(0xffffffffu, r2.x, o2);
                    const uint32_t o_ex = __shfl_sync(0xffffffffu, excl2, o2);
                    const uint32_t o_len = __shfl_sync(0xffffffffu, r2.y, o2);
                    const uint32_t off = f2 - o_ex;
                    float2 c = make_float2(0.f, 0.f);
                    if (v2) c = tr[o_start + off];
                    const unsigned segmask = __ballot_sync(0xffffffffu, v2 && off < o_len);
                    // the vertex before c in the walk: lane - 1's, or the last of the previous chunk
                    float px = __shfl_up_sync(0xffffffffu, c.x, 1), py = __shfl_up_sync(0xffffffffu, c.y, 1);
                    if (lane == 0) {
                        px = cp.x;
                        py = cp.y;
                    }
                    __syncwarp();
                    tbuf[lane] = make_float4(c.x, c.y, __fsub_rn(c.x, px), __fsub_rn(c.y, py));
                    __syncwarp();
                    const uint32_t m = min(32u, total2 - tb);
                    // this slice's share [j0, j1) of the chunk, and the vertex before it
                    const uint32_t q = (m + G - 1) / G;
                    const uint32_t j0 = valid ? min(m, slice * q) : m, j1 = min(m, j0 + q);
                    float2 pv = cp;
                    bool ps = pseg;
                    if (j0 > 0) {
                        const float4 t = tbuf[j0 - 1];
                        pv = make_float2(t.x, t.y);
                        ps = (segmask >> (j0 - 1)) & 1u;
                    }
                    float uxp = __fsub_rn(pv.x, a.x), uyp = __fsub_rn(pv.y, a.y);
                    float wxp = __fsub_rn(pv.x, b.x), wyp = __fsub_rn(pv.y, b.y);
                    int sxp = sgn_code(__fsub_rn(__fmul_rn(ex, uyp), __fmul_rn(ey, uxp)));
                    const float2 pv0 = pv;
                    const bool ps0 = ps;
                    bool coll = false;
#pragma unroll 4
                    for (uint32_t j = j0; j < j1; j++) {
                        const float4 t = tbuf[j];
                        const float ux = __fsub_rn(t.x, a.x), uy = __fsub_rn(t.y, a.y);
                        const int sxn = sgn_code(__fsub_rn(__fmul_rn(ex, uy), __fmul_rn(ey, ux)));
                        if (ps) {  // target segment pv -> t: (t - pv) x (pv - a), (t - pv) x (pv - b)
                            const float pa_ = __fsub_rn(__fmul_rn(t.z, uyp), __fmul_rn(t.w, uxp));
                            const float pb_ = __fsub_rn(__fmul_rn(t.z, wyp), __fmul_rn(t.w, wxp));
                            const int sya = sgn_code(pa_), syb = sgn_code(pb_);
                            hit |= (sxp != sxn) & (sya != syb);
                            coll |= (sya | syb) == 0;
                        }
                        uxp = ux;
                        uyp = uy;
                        wxp = __fsub_rn(t.x, b.x);
                        wyp = __fsub_rn(t.y, b.y);
                        sxp = sxn;
                        ps = (segmask >> j) & 1u;
                    }
                    if (__any_sync(0xffffffffu, coll && valid)) {
                        float2 cq = pv0;
                        bool pq = ps0;
                        for (uint32_t j = j0; j < j1; j++) {
                            const float2 cc = make_float2(tbuf[j].x, tbuf[j].y);
                            if (pq) {
                                const float dx = __fsub_rn(cc.x, cq.x), dy = __fsub_rn(cc.y, cq.y);
                                const int sya = sgn_code(cross_e(cq, dx, dy, a));
                                const int syb = sgn_code(cross_e(cq, dx, dy, b));
                                if ((sya | syb) == 0)
                                    hit |= inter1f(a.x, b.x, cq.x, cc.x) && inter1f(a.y, b.y, cq.y, cc.y);
                            }
                            cq = cc;
                            pq = (segmask >> j) & 1u;
                        }
                    }
                    // segment tests of this slice: one per vertex of [j0, j1) whose predecessor starts a segment
                    if (valid && j1 > j0) {
                        const unsigned below = j1 - 1 > 31u ? 0xffffffffu : ((1u << (j1 - 1)) - 1u);
                        const unsigned from = j0 > 0 ? ~((1u << (j0 - 1)) - 1u) : 0xffffffffu;
                        tests += (j0 == 0 && pseg ? 1u : 0u) + (unsigned)__popc(segmask & below & from);
                    }
                    cp = make_float2(tbuf[m - 1].x, tbuf[m - 1].y);
                    pseg = (segmask >> (m - 1)) & 1u;
                    if (__any_sync(0xffffffffu, hit && valid)) return true;
                }
            }
        }
    }
    return false;
}

}  // namespace farm
