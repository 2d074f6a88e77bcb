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
// around the edge, each crossing edge counted at its first listing), and adds
// its signed inside length: the leaving parameters minus the entering ones,
// plus the tail when it ends inside. Per-item
// partial sums are reduced per pair in a fixed order (deterministic results).
// Coordinates are taken relative to the pair's source first vertex.
// General position is assumed (no collinear overlaps, no crossing exactly at a
// vertex); crossings at a shared vertex are counted once by half-open ranges.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace farm {

// The two tuning knobs of the area pass by size bucket (bucket b holds pairs
// whose larger edge count has floor(log2) == b), chosen by farm_area_autotune:
// c, the edges per work item (default 16), and w, the candidate-window size in
// pixels above which an edge is searched by the whole warp instead of its own
// lane (default 200).
struct Chunks {
    uint16_t c[32];
    uint16_t w[32];
    __host__ __device__ static int bucket(uint32_t es, uint32_t et) {
        uint32_t m = es > et ? es : et;
        return m ? 31 - clz32(m) : 0;
    }
    __host__ __device__ uint32_t of(uint32_t es, uint32_t et) const { return c[bucket(es, et)]; }
    __host__ __device__ uint32_t wide_of(uint32_t es, uint32_t et) const { return w[bucket(es, et)]; }
    __host__ __device__ static int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
        return __clz(x);
#else
        return __builtin_clz(x);
#endif
    }
};

struct AreaArgs {
    const uint32_t *pairs;
    const uint64_t *n;           // pair count (device scalar)
    uint64_t tgt_base;
    Chunks chunks;               // edges per item, by size bucket
    const uint64_t *item_start;  // per pair: first item; item_start[*n] = item count
    uint64_t cap_items;          // partial's capacity
    double *partial;             // per item
    const int8_t *orient;        // per polygon: +1 counter-clockwise, -1 clockwise
    const uint64_t *ep_off;      // per ring position: first entry of the edge's pixel list
    const uint32_t *ep_pix;      // pixels listing each edge (edge -> pixel CSR)
    unsigned long long *next;
    unsigned long long *overflow;  // [0] unused, [1] items beyond cap_items
    unsigned long long *work;      // [0] FP64 crossing tests, [1] crossings counted
    int spread;                    // take items in a spread order (see k_area)
};

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

// The pixels of polygon O searched for edges that may cross segment
// (x0, y0) -> (x1, y1): rows sy..ey of a one-pixel-padded window, and in each
// row the columns row_cols gives.
struct SegWin {
    double x0, y0, x1, y1;
    int sx, ex, sy, ey;
};

__device__ __forceinline__ bool seg_window(const PolyHdr &O, double x0, double y0, double x1, double y1, SegWin &w) {
    const double mnx = fmin(x0, x1), mxx = fmax(x0, x1), mny = fmin(y0, y1), mxy = fmax(y0, y1);
    if (mxx < O.mbr[0] || mnx > O.mbr[2] || mxy < O.mbr[1] || mny > O.mbr[3]) return false;
    w.x0 = x0;
    w.y0 = y0;
    w.x1 = x1;
    w.y1 = y1;
    w.sx = offset_x(O.mbr, O.step_x, O.dimx, mnx) - 1;
    w.ex = offset_x(O.mbr, O.step_x, O.dimx, mxx) + 1;
    w.sy = offset_y(O.mbr, O.step_y, O.dimy, mny) - 1;
    w.ey = offset_y(O.mbr, O.step_y, O.dimy, mxy) + 1;
    w.sx = w.sx < 0 ? 0 : w.sx;
    w.sy = w.sy < 0 ? 0 : w.sy;
    w.ex = w.ex >= O.dimx ? O.dimx - 1 : w.ex;
    w.ey = w.ey >= O.dimy ? O.dimy - 1 : w.ey;
    return true;
}

// Columns xa..xb of window row y; false when the row holds none. Only the
// columns the segment spans within rows y-1 .. y+1, one more on either side:
// every pixel within a pixel of the segment's path, which holds every edge of
// O that the segment crosses (an edge is listed in each pixel it passes
// through, or, where the reference's walk cuts a grid corner, in the diagonal
// neighbours).
// Both for_candidate_edges and first_listing call it, so its products and sums
// are explicit roundings: no contraction may differ between the two.
__device__ __forceinline__ bool row_cols(const PolyHdr &O, const SegWin &w, int y, int &xa, int &xb) {
    xa = w.sx;
    xb = w.ex;
    if (w.y1 != w.y0) {
        const double ylo = __dadd_rn(O.mbr[1], __dmul_rn((double)(y - 1), O.step_y));
        const double yhi = __dadd_rn(O.mbr[1], __dmul_rn((double)(y + 2), O.step_y));
        const double dy = __dsub_rn(w.y1, w.y0);
        double ta = __ddiv_rn(__dsub_rn(ylo, w.y0), dy), tb = __ddiv_rn(__dsub_rn(yhi, w.y0), dy);
        if (ta > tb) {
            const double tmp = ta;
            ta = tb;
            tb = tmp;
        }
        ta = ta < 0 ? 0 : ta;
        tb = tb > 1 ? 1 : tb;
        if (ta > tb) return false;
        const double dx = __dsub_rn(w.x1, w.x0);
        double xa_ = __dadd_rn(w.x0, __dmul_rn(ta, dx)), xb_ = __dadd_rn(w.x0, __dmul_rn(tb, dx));
        if (xa_ > xb_) {
            const double tmp = xa_;
            xa_ = xb_;
            xb_ = tmp;
        }
        const int ca = offset_x(O.mbr, O.step_x, O.dimx, xa_) - 1, cb = offset_x(O.mbr, O.step_x, O.dimx, xb_) + 1;
        xa = ca > w.sx ? ca : w.sx;
        xb = cb < w.ex ? cb : w.ex;
    }
    return true;
}

// Column ranges of the last kRowCache window rows the enumeration computed,
// in a ring indexed by row & (kRowCache - 1) (an empty row is stored as
// xa > xb), so that first_listing reads them instead of recomputing: the
// earlier listings of an edge that crosses the segment lie within a few rows
// of the current one, even when the window spans hundreds of rows.
constexpr int kRowCache = 16;
struct RowCache {
    int2 r[kRowCache];
};

// Edges of polygon O listed by the BORDER pixels of window w, row by row, left
// to right, sequence by sequence. Calls f(pixel, first column of its row,
// sequence index, edge index); an edge listed by several of these pixels (or
// sequences) comes once per listing. Pixel ids grow in this order (row-major).
template <typename F>
__device__ void for_candidate_edges(const StoreView &sv, const PolyHdr &O, const SegWin &w, int cc, RowCache &rc,
                                    F f) {
    const uint8_t *st = sv.status + O.st;
    const uint32_t *off = sv.offset + O.off;
    const uint2 *seq = sv.seq + O.seq;
    for (int y = w.sy; y <= w.ey; y++) {
        int xa, xb;
        const bool ok = row_cols(O, w, y, xa, xb);
        rc.r[y & (kRowCache - 1)] = ok ? make_int2(xa, xb) : make_int2(1, 0);
        if (!ok) continue;
        for (int x = xa; x <= xb; x++) {
            const uint32_t pid = (uint32_t)(y * O.dimx + x);
            if (show_status(st[pid], cc) != 1) continue;
            for (uint32_t q = off[pid]; q < off[pid + 1]; q++) {
                const uint2 sq = seq[q];
                for (uint32_t k = 0; k < sq.y; k++) f(pid, xa, q, sq.x + k);
            }
        }
    }
}

// The same enumeration with the warp sharing one segment: every lane walks
// the window in the same order (so each holds the same row cache), and the
// candidate listings of each row — all sequences of all its pixels, in
// order — are dealt to the lanes round robin; f runs for the lane's share.
// A long edge across a dense polygon meets thousands of candidates, which a
// single lane would otherwise test one after another.
template <typename F>
__device__ void for_candidate_edges_warp(const StoreView &sv, const PolyHdr &O, const SegWin &w, int cc,
                                         RowCache &rc, int lane, F f) {
    const uint8_t *st = sv.status + O.st;
    const uint32_t *off = sv.offset + O.off;
    const uint2 *seq = sv.seq + O.seq;
    for (int y = w.sy; y <= w.ey; y++) {
        int xa, xb;
        const bool ok = row_cols(O, w, y, xa, xb);
        rc.r[y & (kRowCache - 1)] = ok ? make_int2(xa, xb) : make_int2(1, 0);
        if (!ok) continue;
        uint32_t base = 0;  // listings of the row before the current sequence
        for (int x = xa; x <= xb; x++) {
            const uint32_t pid = (uint32_t)(y * O.dimx + x);
            if (show_status(st[pid], cc) != 1) continue;
            for (uint32_t q = off[pid]; q < off[pid + 1]; q++) {
                const uint2 sq = seq[q];
                // this lane's listings k of the sequence: (base + k) % 32 == lane
                uint32_t k = (uint32_t)((lane - (int)(base & 31u) + 32) & 31);
                for (; k < sq.y; k += 32) f(pid, xa, q, sq.x + k);
                base += sq.y;
            }
        }
    }
}

// Whether the listing of edge f met in pixel pid (sequence q, its row's first
// column xa) is the first listing of f that for_candidate_edges meets: no
// BORDER pixel of the window with a smaller id (an earlier row, or the same
// row further left) lists f, and no earlier sequence of pid holds it. Each
// edge that crosses the segment is then counted exactly once, whatever the
// number of pixels listing it, with no per-edge memory. The pixels listing f
// come from the edge -> pixel index (ascending ids, so the scan stops at pid),
// and window membership from the rows the enumeration computed (or the same
// row_cols for rows older than the cache), so both agree to the bit.
__device__ bool first_listing(const StoreView &sv, const PolyHdr &O, const SegWin &w, int cc, const RowCache &rc,
                              const uint64_t *ep_off, const uint32_t *ep_pix, uint32_t pid, int xa, uint32_t q,
                              uint32_t f) {
    const uint64_t g = O.ring + f;
    const uint32_t dimx = (uint32_t)O.dimx;
    const int py = (int)(pid / dimx);
    int self = 0;
    for (uint64_t i = ep_off[g], e = ep_off[g + 1]; i < e; i++) {
        const uint32_t r = ep_pix[i];
        if (r > pid) break;
        if (r == pid) {
            self++;
            continue;
        }
        const int ry = (int)(r / dimx), rx = (int)(r - (uint32_t)ry * dimx);
        if (ry < w.sy) continue;  // above the window
        if (show_status(sv.status[O.st + r], cc) != 1) continue;
        if (ry == py) {
            if (rx >= xa) return false;
            continue;
        }
        int cxa, cxb;
        if (ry > py - kRowCache) {  // still in the ring (rows sy .. py were enumerated in order)
            const int2 c = rc.r[ry & (kRowCache - 1)];
            cxa = c.x;
            cxb = c.y;
        } else if (!row_cols(O, w, ry, cxa, cxb)) {
            continue;
        }
        if (rx >= cxa && rx <= cxb) return false;
    }
    if (self > 1) {  // pid holds f in more than one sequence: the first counts
        const uint2 *seq = sv.seq + O.seq;
        for (uint32_t p = sv.offset[O.off + pid]; p < q; p++) {
            const uint2 sq = seq[p];
            if (f >= sq.x && f - sq.x < sq.y) return false;
        }
    }
    return true;
}

// Crossing parameter t of segment p -> p + d with edge e of ring r, in [0, 1)
// on both (half-open, so a crossing at a shared vertex counts once).
// FP32 rejection ahead of crossing(): edge A->B lies strictly on one side of
// the line through P->Q, or P->Q strictly on one side of the line through
// A->B, by a margin of 1e-6 (~17 u32) times the orientation products'
// magnitudes. That is far above the rounding of this test (~4 u32) and of
// crossing()'s FP64 arithmetic, so such segments cannot cross and crossing()
// would return false as well; only the candidates near a crossing pay for
// FP64, which on GB300 issues at 1/64 of the FP32 rate.
__device__ __forceinline__ bool apart32(float2 P, float2 Q, float2 A, float2 B) {
    const float ex = Q.x - P.x, ey = Q.y - P.y;
    const float ax = A.x - P.x, ay = A.y - P.y, bx = B.x - P.x, by = B.y - P.y;
    const float oa = ex * ay - ey * ax, ob = ex * by - ey * bx;
    const float ma = 1e-6f * (fabsf(ex * ay) + fabsf(ey * ax)), mb = 1e-6f * (fabsf(ex * by) + fabsf(ey * bx));
    if ((oa > ma && ob > mb) || (oa < -ma && ob < -mb)) return true;
    const float gx = B.x - A.x, gy = B.y - A.y;
    const float px = P.x - A.x, py = P.y - A.y, qx = Q.x - A.x, qy = Q.y - A.y;
    const float op = gx * py - gy * px, oq = gx * qy - gy * qx;
    const float mp = 1e-6f * (fabsf(gx * py) + fabsf(gy * px)), mq = 1e-6f * (fabsf(gx * qy) + fabsf(gy * qx));
    return (op > mp && oq > mq) || (op < -mp && oq < -mq);
}

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

// Default knobs: edges per item, and the window size (pixels) above which an
// edge is searched by the whole warp (for_candidate_edges_warp) instead of
// its own lane. FARM_AREA_WIDE_WINDOW overrides the window size of every
// bucket.
constexpr int kDefaultChunk = 16;
constexpr int kDefaultWide = 200;

static long wide_window_env() {
    const char *v = getenv("FARM_AREA_WIDE_WINDOW");
    if (!v || !*v) return 0;
    const long x = strtol(v, nullptr, 10);
    return x > 0 && x < 65536 ? x : 0;
}

// FARM_AREA_SPREAD=0 takes the items in pair order
static int spread_items() {
    const char *v = getenv("FARM_AREA_SPREAD");
    return (v && *v == '0') ? 0 : 1;
}


__global__ void __launch_bounds__(256) k_area(const StoreView sv, AreaArgs a) {
    const int lane = threadIdx.x & 31;
    const int cc = sv.category_count;
    unsigned long long my_tests = 0, my_cross = 0;
    for (;;) {
        const uint64_t n = *a.n;
        const uint64_t nitems = a.item_start[n];
        if (nitems > a.cap_items) {  // a plan's capacity was exceeded: report, compute nothing
            if (lane == 0 && blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&a.overflow[1], 1ull);
            break;
        }
        unsigned long long it = 0;
        if (lane == 0) it = atomicAdd(a.next, 1ull);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= nitems) break;
        // Items lie pair after pair, and the heavy pairs' items are each slow:
        // taken in that order, a heavy pair near the end leaves a tail. The
        // k-th item taken is item k * P mod nitems (P prime, coprime to
        // nitems: a bijection), which spreads every pair's items over the
        // pass. Each item writes its own partial, and the per-pair reduction
        // runs in item order, so the results do not depend on this order.
        if (a.spread) {
            const uint64_t P = (nitems % 1000003ull) ? 1000003ull : 999983ull;
            it = (unsigned long long)((it * P) % nitems);
        }
        uint32_t p = find_segment(a.item_start, (uint32_t)n, it);
        uint64_t rel = it - a.item_start[p];
        const PolyHdr &S = sv.hdr[a.pairs[2 * p]];
        const PolyHdr &T = sv.hdr[a.tgt_base + a.pairs[2 * p + 1]];
        uint32_t es = S.nv - 1, et = T.nv - 1;  // edges (the ring's last edge is the zero-length closing one)
        const uint32_t chunk = a.chunks.of(es, et);
        const long wide_window = (long)a.chunks.wide_of(es, et);
        uint64_t cs = (es + chunk - 1) / chunk;
        bool side_t = rel >= cs;
        const PolyHdr &M = side_t ? T : S;  // the boundary integrated
        const PolyHdr &O = side_t ? S : T;  // the polygon it is clipped by
        uint32_t first = (uint32_t)((side_t ? rel - cs : rel) * chunk);
        uint32_t me = side_t ? et : es;
        uint32_t last = first + chunk < me ? first + chunk : me;
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
            float2 P = make_float2(0.f, 0.f), Q = P;
            bool wide = false;
            if (valid) {
                P = mr[e];
                Q = mr[e + 1];
                px = (double)P.x - ox;
                py = (double)P.y - oy;
                dx = (double)Q.x - P.x;
                dy = (double)Q.y - P.y;
                SegWin w;
                const bool has_w = (dx != 0 || dy != 0) && seg_window(O, P.x, P.y, Q.x, Q.y, w);
                wide = has_w && (long)(w.ex - w.sx + 1) * (long)(w.ey - w.sy + 1) > wide_window;
                if (has_w && !wide) {
                    // an edge of O may be listed by several pixels: count it
                    // at its first listing only (tested before the FP64
                    // crossing, which then runs once per edge pair)
                    RowCache rc;
                    for_candidate_edges(sv, O, w, cc, rc, [&](uint32_t pid, int xa, uint32_t q, uint32_t f) {
                        double t, den;
                        if (apart32(P, Q, orr[f], orr[f + 1]) ||
                            !first_listing(sv, O, w, cc, rc, a.ep_off, a.ep_pix, pid, xa, q, f))
                            return;
                        my_tests++;
                        if (!crossing(px, py, dx, dy, orr, f, ox, oy, t, den)) return;
                        nc++;
                        sum_t += (osign * den > 0) ? t : -t;
                    });
                }
            }
            // edges with wide windows: the whole warp takes one at a time
            for (unsigned wm = __ballot_sync(0xffffffffu, wide); wm; wm &= wm - 1) {
                const int src = __ffs(wm) - 1;
                const float2 Pw = make_float2(__shfl_sync(0xffffffffu, P.x, src), __shfl_sync(0xffffffffu, P.y, src));
                const float2 Qw = make_float2(__shfl_sync(0xffffffffu, Q.x, src), __shfl_sync(0xffffffffu, Q.y, src));
                const double pxw = (double)Pw.x - ox, pyw = (double)Pw.y - oy;
                const double dxw = (double)Qw.x - Pw.x, dyw = (double)Qw.y - Pw.y;
                SegWin ww;
                seg_window(O, Pw.x, Pw.y, Qw.x, Qw.y, ww);  // the owner's window, recomputed identically
                RowCache rc;
                double st_l = 0;
                int nc_l = 0;
                for_candidate_edges_warp(sv, O, ww, cc, rc, lane, [&](uint32_t pid, int xa, uint32_t q, uint32_t f) {
                    double t, den;
                    if (apart32(Pw, Qw, orr[f], orr[f + 1]) ||
                        !first_listing(sv, O, ww, cc, rc, a.ep_off, a.ep_pix, pid, xa, q, f))
                        return;
                    my_tests++;
                    if (!crossing(pxw, pyw, dxw, dyw, orr, f, ox, oy, t, den)) return;
                    nc_l++;
                    st_l += (osign * den > 0) ? t : -t;
                });
                for (int o = 16; o; o >>= 1) {
                    st_l += __shfl_xor_sync(0xffffffffu, st_l, o);
                    nc_l += __shfl_xor_sync(0xffffffffu, nc_l, o);
                }
                if (lane == src) {
                    sum_t = st_l;
                    nc = nc_l;
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
            if (valid) my_cross += (unsigned long long)nc;
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) a.partial[it] = 0.5 * sign * acc;
    }
    if (my_tests) atomicAdd(&a.work[0], my_tests);
    if (my_cross) atomicAdd(&a.work[1], my_cross);
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

// Edge -> pixel index of every rasterized polygon, by ring position: pass 0
// counts the pixels listing each edge, pass 1 writes them (in any order). One
// warp per polygon, lanes over its pixels.
template <bool kFill>
__global__ void k_edge_pix(const StoreView sv, uint32_t npoly, const uint64_t *__restrict__ ep_off,
                           unsigned long long *__restrict__ cnt, uint32_t *__restrict__ ep_pix) {
    const int lane = threadIdx.x & 31;
    const uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = w0; p < npoly; p += nw) {
        const PolyHdr &h = sv.hdr[p];
        if (h.err) continue;
        const uint32_t *off = sv.offset + h.off;
        const uint2 *seq = sv.seq + h.seq;
        for (uint32_t pid = lane; pid < h.P; pid += 32) {
            for (uint32_t q = off[pid]; q < off[pid + 1]; q++) {
                const uint2 sq = seq[q];
                for (uint32_t k = 0; k < sq.y; k++) {
                    if (sq.x + k > h.nv) break;  // past the polygon's ring slots (never, by construction)
                    const uint64_t g = h.ring + sq.x + k;
                    const unsigned long long at = atomicAdd(&cnt[g], 1ull);
                    if (kFill) ep_pix[ep_off[g] + at] = pid;
                }
            }
        }
    }
}

// Each edge's pixel list in ascending pixel id (insertion sort: an edge is
// listed by at most dimx + dimy pixels, a few in the common case).
__global__ void k_edge_pix_sort(const uint64_t *__restrict__ ep_off, uint64_t nring, uint32_t *__restrict__ ep_pix) {
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nring; g += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = ep_off[g], e = ep_off[g + 1];
        for (uint64_t i = b + 1; i < e; i++) {
            const uint32_t v = ep_pix[i];
            uint64_t j = i;
            while (j > b && ep_pix[j - 1] > v) {
                ep_pix[j] = ep_pix[j - 1];
                j--;
            }
            ep_pix[j] = v;
        }
    }
}

// items per pair, for every slot up to cap (0 past the pair count)
__global__ void k_area_items(const StoreView sv, const uint32_t *__restrict__ pairs, const uint64_t *__restrict__ np,
                             uint64_t cap, uint64_t tgt_base, Chunks chunks, uint64_t *__restrict__ cnt) {
    const uint64_t n = *np;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= cap; k += (uint64_t)gridDim.x * blockDim.x) {
        if (k >= n) {
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
        const uint32_t chunk = chunks.of(es, et);
        cnt[k] = (es + chunk - 1) / chunk + (et + chunk - 1) / chunk;
    }
}

// fixed-order sum of each pair's item partials
__global__ void k_area_reduce(const uint64_t *__restrict__ item_start, const uint64_t *__restrict__ np,
                              const double *__restrict__ partial, const StoreView sv,
                              const uint32_t *__restrict__ pairs, uint64_t tgt_base, double *__restrict__ out) {
    const uint64_t n = *np;
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

// ---------------------------------------------------------------- host --

static Chunks chunks_of(const farm_store *s) {
    Chunks c;
    const long env_w = wide_window_env();
    for (int b = 0; b < 32; b++) {
        c.c[b] = (uint16_t)(s->area_chunk[b] > 0 ? s->area_chunk[b] : kDefaultChunk);
        c.w[b] = (uint16_t)(env_w ? env_w : (s->area_wide[b] > 0 ? s->area_wide[b] : kDefaultWide));
    }
    return c;
}

// polygon orientations, computed once per rasterization, in a scratch slot of
// their own (a captured plan holds its address)
constexpr int kOrientSlot = Q_AREA_ORIENT;
static int ensure_orient(farm_store *s, cudaStream_t st) {
    DevBuf &ori = s->s[kOrientSlot];
    if (s->orient_epoch == s->raster_epoch && ori.cap >= s->n_poly) return FARM_OK;
    FARM_TRY(ori.ensure(s->n_poly + 64));
    unsigned ob = (unsigned)((32ull * s->n_poly + 255) / 256);
    if (ob > 8192) ob = 8192;
    k_orient<<<ob, 256, 0, st>>>(s->view(), (uint32_t)s->n_poly, ori.as<int8_t>());
    s->launches++;
    FARM_CUDA(cudaGetLastError());
    s->orient_epoch = s->raster_epoch;
    return FARM_OK;
}

// The edge -> pixel index, built once per rasterization in scratch slots of
// its own (a captured plan holds their addresses). Counts go through Q_SCR3.
static int ensure_edge_pix(farm_store *s, cudaStream_t st) {
    if (s->edgepix_epoch == s->raster_epoch) return FARM_OK;
    const uint64_t nring = s->n_edges + 2 * s->n_poly;
    DevBuf &off = s->s[Q_AREA_EPOFF], &pix = s->s[Q_AREA_EPPIX], &cnt = s->s[Q_SCR3];
    FARM_TRY(off.ensure(8 * (nring + 1) + 64));
    FARM_TRY(cnt.ensure(8 * (nring + 1) + 64));
    unsigned long long *c = cnt.as<unsigned long long>();
    uint64_t *o = off.as<uint64_t>();
    unsigned blocks = (unsigned)((32ull * s->n_poly + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    if (!blocks) blocks = 1;
    FARM_CUDA(cudaMemsetAsync(c, 0, 8 * (nring + 1), st));
    k_edge_pix<false><<<blocks, 256, 0, st>>>(s->view(), (uint32_t)s->n_poly, nullptr, c, nullptr);
    FARM_CUDA(cudaGetLastError());
    size_t bytes = 0;
    FARM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, (const uint64_t *)c, o, (int64_t)(nring + 1)));
    FARM_TRY(s->cub_tmp.ensure(bytes + 64));
    FARM_CUDA(cub::DeviceScan::ExclusiveSum(s->cub_tmp.p, bytes, (const uint64_t *)c, o, (int64_t)(nring + 1), st));
    uint64_t total = 0;
    FARM_CUDA(cudaMemcpyAsync(&total, o + nring, 8, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    FARM_TRY(pix.ensure(4 * total + 64));
    FARM_CUDA(cudaMemsetAsync(c, 0, 8 * (nring + 1), st));
    k_edge_pix<true><<<blocks, 256, 0, st>>>(s->view(), (uint32_t)s->n_poly, o, c, pix.as<uint32_t>());
    FARM_CUDA(cudaGetLastError());
    unsigned sb = (unsigned)((nring + 255) / 256);
    if (sb > 8192) sb = 8192;
    k_edge_pix_sort<<<sb ? sb : 1, 256, 0, st>>>(o, nring, pix.as<uint32_t>());
    FARM_CUDA(cudaGetLastError());
    s->launches += 4;
    s->edgepix_epoch = s->raster_epoch;
    return FARM_OK;
}

// Buffers of one area pass. Everything the kernels need to know about the
// batch (pair count, item count) is read on the device, so the same sequence
// can be captured once in a CUDA graph and replayed for any batch that fits.
struct AreaBufs {
    const uint32_t *pairs;
    const uint64_t *n;  // device scalar
    uint64_t cap_pairs;
    uint64_t *cnt, *start;  // cap_pairs + 1 each
    double *partial;
    uint64_t cap_items;
    unsigned long long *ctr;  // [0] work counter, [1] [2] overflow flags
    void *scan_tmp;
    size_t scan_bytes;
    double *out;
    Chunks chunks;
};

static int scan_bytes(uint64_t cap, size_t *bytes) {
    FARM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, *bytes, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                            (int64_t)(cap + 1)));
    return FARM_OK;
}

static int area_items(farm_store *s, const AreaBufs &b, cudaStream_t st) {
    unsigned blocks = (unsigned)((b.cap_pairs + 256) / 256);
    if (blocks > 4096) blocks = 4096;
    k_area_items<<<blocks, 256, 0, st>>>(s->view(), b.pairs, b.n, b.cap_pairs, s->n_side[0], b.chunks, b.cnt);
    FARM_CUDA(cudaGetLastError());
    size_t bytes = b.scan_bytes;
    FARM_CUDA(cub::DeviceScan::ExclusiveSum(b.scan_tmp, bytes, b.cnt, b.start, (int64_t)(b.cap_pairs + 1), st));
    return FARM_OK;
}

static int area_compute(farm_store *s, const AreaBufs &b, cudaStream_t st) {
    FARM_CUDA(cudaMemsetAsync(b.ctr, 0, 40, st));
    AreaArgs aa{b.pairs,
                b.n,
                s->n_side[0],
                b.chunks,
                b.start,
                b.cap_items,
                b.partial,
                s->s[kOrientSlot].as<int8_t>(),
                s->s[Q_AREA_EPOFF].as<uint64_t>(),
                s->s[Q_AREA_EPPIX].as<uint32_t>(),
                b.ctr,
                b.ctr + 1,
                b.ctr + 3,
                spread_items()};
    k_area<<<sm_count() * 8, 256, 0, st>>>(s->view(), aa);
    FARM_CUDA(cudaGetLastError());
    unsigned blocks = (unsigned)((b.cap_pairs + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (!blocks) blocks = 1;
    k_area_reduce<<<blocks, 256, 0, st>>>(b.start, b.n, b.partial, s->view(), b.pairs, s->n_side[0], b.out);
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

static int area_checks(farm_store *s, const char *who) {
    if (!s->rasterized) {
        set_error(std::string(who) + ": rasterize first");
        return FARM_EINVAL;
    }
    if (s->n_side[1] == 0) {
        set_error(std::string(who) + ": no target side loaded");
        return FARM_EINVAL;
    }
    return FARM_OK;
}

int intersection_area(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, double *out, farm_stats *st) {
    FARM_TRY(area_checks(s, "farm_intersection_area"));
    FARM_TRY(check_pairs(s, pairs, n, mem, false, "farm_intersection_area"));
    cudaStream_t stream = s->stream;
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
    DevBuf &cnt = s->s[Q_SCR0], &start = s->s[Q_SCR1], &part = s->s[Q_SCR2];
    FARM_TRY(cnt.ensure(8 * (n + 1) + 64));
    FARM_TRY(start.ensure(8 * (n + 1) + 64));
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *ctr = s->d_counters.as<unsigned long long>();
    uint64_t *dn = reinterpret_cast<uint64_t *>(ctr + 8);
    FARM_CUDA(cudaMemcpyAsync(dn, &n, 8, cudaMemcpyHostToDevice, stream));
    FARM_TRY(ensure_orient(s, stream));
    FARM_TRY(ensure_edge_pix(s, stream));
    AreaBufs b{};
    b.pairs = dpairs;
    b.n = dn;
    b.cap_pairs = n;
    b.cnt = cnt.as<uint64_t>();
    b.start = start.as<uint64_t>();
    b.ctr = ctr;
    b.out = dout;
    b.chunks = chunks_of(s);
    FARM_TRY(scan_bytes(n, &b.scan_bytes));
    FARM_TRY(s->cub_tmp.ensure(b.scan_bytes + 64));
    b.scan_tmp = s->cub_tmp.p;
    FARM_CUDA(cudaEventRecord(s->ev[6], stream));
    FARM_TRY(area_items(s, b, stream));
    uint64_t nitems = 0;
    FARM_CUDA(cudaMemcpyAsync(&nitems, b.start + n, 8, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    FARM_TRY(part.ensure(8 * nitems + 64));
    b.partial = part.as<double>();
    b.cap_items = nitems;
    FARM_TRY(area_compute(s, b, stream));
    FARM_CUDA(cudaEventRecord(s->ev[7], stream));
    if (mem == FARM_MEM_HOST && out && n) FARM_CUDA(cudaMemcpyAsync(out, dout, 8 * n, cudaMemcpyDeviceToHost, stream));
    unsigned long long work[2] = {0, 0};
    FARM_CUDA(cudaMemcpyAsync(work, ctr + 3, 16, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    s->launches += 4;
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        st->segment_tests = work[0];
        st->border_pairs = work[1];
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[6], s->ev[7]);
        st->ms_total = ms;
        st->ms_stage[2] = ms;
        st->kernel_launches = 4;
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

// ------------------------------------------------------ plans and tuning --
// A plan owns fixed-capacity buffers for one area pass and the CUDA graph of
// that pass (items, scan, the persistent work-stealing kernel, the per-pair
// reduction), captured once. Running it copies a batch of pairs in and
// replays the graph: one launch for any batch within capacity, whatever its
// mix of tiny and huge pairs.
struct farm_area_plan {
    farm_store *s = nullptr;
    uint64_t cap_pairs = 0, cap_items = 0, epoch = 0;
    farm::DevBuf pairs, n, cnt, start, partial, ctr, tmp, out;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {
void plan_free(farm_area_plan *p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    for (farm::DevBuf *b : {&p->pairs, &p->n, &p->cnt, &p->start, &p->partial, &p->ctr, &p->tmp, &p->out})
        b->release();
    delete p;
}
}  // namespace

extern "C" int farm_area_plan_create(farm_store *s, uint64_t max_pairs, uint64_t max_items, farm_area_plan **out) {
    using namespace farm;
    if (!s || !out || max_pairs == 0 || max_items == 0) {
        set_error("invalid arguments to farm_area_plan_create");
        return FARM_EINVAL;
    }
    *out = nullptr;
    FARM_TRY(area_checks(s, "farm_area_plan_create"));
    cudaStream_t st = s->stream;
    FARM_TRY(ensure_orient(s, st));
    FARM_TRY(ensure_edge_pix(s, st));
    farm_area_plan *p = new farm_area_plan();
    p->s = s;
    p->cap_pairs = max_pairs;
    p->cap_items = max_items;
    p->epoch = s->raster_epoch;
    AreaBufs b{};
    int rc = FARM_OK;
    if (rc == FARM_OK) rc = p->pairs.ensure(8 * max_pairs + 64);
    if (rc == FARM_OK) rc = p->n.ensure(64);
    if (rc == FARM_OK) rc = p->cnt.ensure(8 * (max_pairs + 1) + 64);
    if (rc == FARM_OK) rc = p->start.ensure(8 * (max_pairs + 1) + 64);
    if (rc == FARM_OK) rc = p->partial.ensure(8 * max_items + 64);
    if (rc == FARM_OK) rc = p->ctr.ensure(64);
    if (rc == FARM_OK) rc = p->out.ensure(8 * max_pairs + 64);
    if (rc == FARM_OK) rc = scan_bytes(max_pairs, &b.scan_bytes);
    if (rc == FARM_OK) rc = p->tmp.ensure(b.scan_bytes + 64);
    if (rc == FARM_OK) {
        cudaError_t e = cudaMemsetAsync(p->n.p, 0, 8, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "farm_area_plan_create");
    }
    if (rc != FARM_OK) {
        plan_free(p);
        return rc;
    }
    b.pairs = p->pairs.as<uint32_t>();
    b.n = p->n.as<uint64_t>();
    b.cap_pairs = max_pairs;
    b.cnt = p->cnt.as<uint64_t>();
    b.start = p->start.as<uint64_t>();
    b.partial = p->partial.as<double>();
    b.cap_items = max_items;
    b.ctr = p->ctr.as<unsigned long long>();
    b.scan_tmp = p->tmp.p;
    b.out = p->out.as<double>();
    b.chunks = chunks_of(s);
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        plan_free(p);
        return cuda_fail(e, "cudaStreamBeginCapture");
    }
    int rc1 = area_items(s, b, st);
    int rc2 = rc1 == FARM_OK ? area_compute(s, b, st) : rc1;
    e = cudaStreamEndCapture(st, &p->graph);
    if (rc2 != FARM_OK || e != cudaSuccess) {
        plan_free(p);
        return rc2 != FARM_OK ? rc2 : cuda_fail(e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    if (e != cudaSuccess) {
        plan_free(p);
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    *out = p;
    return FARM_OK;
}

extern "C" int farm_area_plan_run(farm_area_plan *p, const uint32_t *pairs, uint64_t n, int mem, double *out,
                                  farm_stats *st_out) {
    using namespace farm;
    if (!p || (n && (!pairs || !out))) {
        set_error("invalid arguments to farm_area_plan_run");
        return FARM_EINVAL;
    }
    farm_store *s = p->s;
    if (n > p->cap_pairs) {
        set_error("farm_area_plan_run: " + std::to_string(n) + " pairs exceed the plan's capacity of " +
                  std::to_string(p->cap_pairs));
        return FARM_EINVAL;
    }
    if (s->raster_epoch != p->epoch) {
        set_error("farm_area_plan_run: the store was reloaded or rasterized again since the plan was made");
        return FARM_EINVAL;
    }
    FARM_TRY(check_pairs(s, pairs, n, mem, false, "farm_area_plan_run"));
    cudaStream_t st = s->stream;
    const cudaMemcpyKind k_in = mem == FARM_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    const cudaMemcpyKind k_out = mem == FARM_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (n) FARM_CUDA(cudaMemcpyAsync(p->pairs.p, pairs, 8 * n, k_in, st));
    FARM_CUDA(cudaMemcpyAsync(p->n.p, &n, 8, cudaMemcpyHostToDevice, st));
    FARM_CUDA(cudaEventRecord(s->ev[6], st));
    FARM_CUDA(cudaGraphLaunch(p->exec, st));
    FARM_CUDA(cudaEventRecord(s->ev[7], st));
    unsigned long long flags[5] = {0, 0, 0, 0, 0};  // next, -, overflow, crossing tests, crossings
    FARM_CUDA(cudaMemcpyAsync(flags, p->ctr.p, 40, cudaMemcpyDeviceToHost, st));
    if (n) FARM_CUDA(cudaMemcpyAsync(out, p->out.p, 8 * n, k_out, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    s->launches += 3;
    if (flags[2]) {
        set_error("farm_area_plan_run: the batch needs more work items than the plan's capacity of " +
                  std::to_string(p->cap_items));
        return FARM_EOVERFLOW;
    }
    if (st_out) {
        memset(st_out, 0, sizeof *st_out);
        st_out->pairs = n;
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[6], s->ev[7]);
        st_out->ms_total = ms;
        st_out->ms_stage[2] = ms;
        st_out->kernel_launches = 1;  // one graph launch
        st_out->segment_tests = flags[3];
        st_out->border_pairs = flags[4];
    }
    return FARM_OK;
}

extern "C" void farm_area_plan_destroy(farm_area_plan *p) { plan_free(p); }

extern "C" int farm_area_set_chunks(farm_store *s, const int32_t *chunk_by_bucket) {
    using namespace farm;
    if (!s || !chunk_by_bucket) {
        set_error("invalid arguments to farm_area_set_chunks");
        return FARM_EINVAL;
    }
    for (int b = 0; b < 32; b++)
        if (chunk_by_bucket[b] < 0 || chunk_by_bucket[b] > 32768) {
            set_error("farm_area_set_chunks: chunk sizes must lie in 1..32768 (0 = default)");
            return FARM_EINVAL;
        }
    for (int b = 0; b < 32; b++) s->area_chunk[b] = chunk_by_bucket[b];
    return FARM_OK;
}

extern "C" int farm_area_set_wide(farm_store *s, const int32_t *wide_by_bucket) {
    using namespace farm;
    if (!s || !wide_by_bucket) {
        set_error("invalid arguments to farm_area_set_wide");
        return FARM_EINVAL;
    }
    for (int b = 0; b < 32; b++)
        if (wide_by_bucket[b] < 0 || wide_by_bucket[b] > 65535) {
            set_error("farm_area_set_wide: window sizes must lie in 1..65535 (0 = default)");
            return FARM_EINVAL;
        }
    for (int b = 0; b < 32; b++) s->area_wide[b] = wide_by_bucket[b];
    return FARM_OK;
}

// Autotuner: for every size bucket present in the sample (floor(log2) of a
// pair's larger edge count), time the area pass on up to 2048 of its pairs,
// first over the candidate chunk sizes 8..256 (edges per work item), then, at the
// best chunk, over the candidate window thresholds (pixels above which an
// edge is searched by the whole warp), and keep the fastest of each. One
// untimed pass per bucket warms up. The store keeps both tables
// (farm_area_set_chunks, farm_area_set_wide); they are also returned.
extern "C" int farm_area_autotune(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, int32_t *chunk_out,
                                  int32_t *wide_out) {
    using namespace farm;
    if (!s || (n && !pairs)) {
        set_error("invalid arguments to farm_area_autotune");
        return FARM_EINVAL;
    }
    FARM_TRY(area_checks(s, "farm_area_autotune"));
    FARM_TRY(check_pairs(s, pairs, n, mem, false, "farm_area_autotune"));
    std::vector<uint32_t> hp(2 * n);
    if (n) {
        if (mem == FARM_MEM_HOST) {
            memcpy(hp.data(), pairs, 8 * n);
        } else {
            FARM_CUDA(cudaMemcpyAsync(hp.data(), pairs, 8 * n, cudaMemcpyDeviceToHost, s->stream));
            FARM_CUDA(cudaStreamSynchronize(s->stream));
        }
    }
    auto edges = [&](int side, uint32_t k) -> uint32_t {
        const std::vector<uint64_t> &o = s->h_off[side];
        return (uint32_t)(o[k + 1] - o[k]);  // stored vertices = edges of the in-memory ring
    };
    std::vector<std::vector<uint32_t>> byb(32);
    for (uint64_t i = 0; i < n; i++) {
        if (hp[2 * i] >= s->n_side[0] || hp[2 * i + 1] >= s->n_side[1]) {
            set_error("farm_area_autotune: pair index out of range");
            return FARM_EINVAL;
        }
        const int b = Chunks::bucket(edges(0, hp[2 * i]), edges(1, hp[2 * i + 1]));
        if (byb[b].size() < 2 * 2048) {
            byb[b].push_back(hp[2 * i]);
            byb[b].push_back(hp[2 * i + 1]);
        }
    }
    static const int32_t kChunkCand[] = {8, 16, 32, 64, 128, 256};
    static const int32_t kWideCand[] = {24, 48, 200, 800};
    int32_t saved_c[32], saved_w[32];
    memcpy(saved_c, s->area_chunk, sizeof saved_c);
    memcpy(saved_w, s->area_wide, sizeof saved_w);
    int32_t best_c[32], best_w[32];
    memcpy(best_c, s->area_chunk, sizeof best_c);
    memcpy(best_w, s->area_wide, sizeof best_w);
    auto restore = [&]() {
        memcpy(s->area_chunk, saved_c, sizeof saved_c);
        memcpy(s->area_wide, saved_w, sizeof saved_w);
    };
    // one pass of bucket b's pairs with chunk c and window w everywhere
    auto timed = [&](int b, int32_t c, int32_t w, double *ms) -> int {
        for (int q = 0; q < 32; q++) {
            s->area_chunk[q] = c;
            s->area_wide[q] = w;
        }
        farm_stats stt;
        const int rc = intersection_area(s, byb[b].data(), byb[b].size() / 2, FARM_MEM_HOST, nullptr, &stt);
        *ms = stt.ms_total;
        return rc;
    };
    for (int b = 0; b < 32; b++) {
        if (byb[b].empty()) continue;
        double ms = 0, best_ms = 1e300;
        int rc = timed(b, kDefaultChunk, kDefaultWide, &ms);  // warm-up
        int32_t bc = kDefaultChunk, bw = kDefaultWide;
        for (int32_t c : kChunkCand) {
            if (rc == FARM_OK) rc = timed(b, c, kDefaultWide, &ms);
            if (rc == FARM_OK && ms < best_ms) {
                best_ms = ms;
                bc = c;
            }
        }
        for (int32_t w : kWideCand) {
            if (w == kDefaultWide) continue;  // timed above at bc
            if (rc == FARM_OK) rc = timed(b, bc, w, &ms);
            if (rc == FARM_OK && ms < best_ms) {
                best_ms = ms;
                bw = w;
            }
        }
        if (rc != FARM_OK) {
            restore();
            return rc;
        }
        best_c[b] = bc;
        best_w[b] = bw;
    }
    memcpy(s->area_chunk, best_c, sizeof best_c);
    memcpy(s->area_wide, best_w, sizeof best_w);
    if (chunk_out) memcpy(chunk_out, best_c, sizeof best_c);
    if (wide_out) memcpy(wide_out, best_w, sizeof best_w);
    return FARM_OK;
}
