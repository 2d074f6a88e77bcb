// Stages (b) + (c) for within-distance: hierarchical BORDER x BORDER descent,
// candidate ordering and border refinement with point-segment distances.
//
// Reference decision procedure (Ideal::within, Ideal.cpp:2475-2643):
//  * descend the two polygons' raster hierarchies together (the coarser side
//    advances); at each level the BORDER children of the queued pixels form
//    two sets, their cross product gives the smallest box max-distance (any
//    max-distance <= d decides "true") and keeps the pairs whose box distance
//    is <= d and below that smallest max-distance;
//  * at the finest level the kept pairs are ordered by (approximate distance,
//    low, high, ids) and refined in that order with the minimum point-segment
//    distance of their edge sequences; "true" once the running minimum is
//    below d, "false" once it is below every later pair's lower bound.
// Below the finest level the queue only matters through the two sets of
// pixels it holds (the children of its members), so each level here keeps
// two pixel sets instead of an explicit pair queue.
//
// Kernels: k_within_descend (one warp per pair) writes the finest level's
// candidate pairs; a merge sort orders them by pair and the reference's tuple;
// k_within_refine (one warp per pair) runs the ordered refinement, with the
// point-segment distances of each edge-sequence pair spread over the lanes.
#include <cub/cub.cuh>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace farm {

// util.h:68 (float constants) and the 900-entry longitude table (util.h:73),
// regenerated on the host from its defining formula.
__constant__ float c_mean20[20];
__constant__ double c_deg_lon[900];
__constant__ float c_inv_deg_lon_f[900];  // 1 / c_deg_lon, rounded to float (FP32 first pass only)

static std::mutex g_tab_mu;
static bool g_tab_ready[64] = {};

static int ensure_tables(int dev) {
    std::lock_guard<std::mutex> lock(g_tab_mu);
    if (dev >= 0 && dev < 64 && g_tab_ready[dev]) return FARM_OK;
    const float mean20[20] = {0.0f,  0.7f,  0.62f, 0.55f, 0.52f, 0.45f, 0.42f, 0.4f,  0.38f, 0.34f,
                              0.31f, 0.28f, 0.25f, 0.22f, 0.18f, 0.15f, 0.1f,  0.05f, 0.0f,  0.0f};
    double deg[900];
    const double PI = 3.14159265;
    for (int i = 0; i < 900; i++) {
        double lat = i / 10.0;
        double v = 360.0 / (sin((90 - lat) * PI / 180) * 40076);
        char buf[64];
        snprintf(buf, sizeof buf, "%.6f", v);
        deg[i] = strtod(buf, nullptr);
    }
    FARM_CUDA(cudaMemcpyToSymbol(c_mean20, mean20, sizeof mean20));
    FARM_CUDA(cudaMemcpyToSymbol(c_deg_lon, deg, sizeof deg));
    float inv[900];
    for (int i = 0; i < 900; i++) inv[i] = (float)(1.0 / deg[i]);
    FARM_CUDA(cudaMemcpyToSymbol(c_inv_deg_lon_f, inv, sizeof inv));
    if (dev >= 0 && dev < 64) g_tab_ready[dev] = true;
    return FARM_OK;
}

__device__ __forceinline__ double deg_lon(double lat) {
    double a = fabs(lat);
    if (a == 90) a = 89.9;
    int idx = (int)(a * 10);
    if (idx < 0 || idx >= 900) idx = 899;  // the reference indexes past the table here
    return c_deg_lon[idx];
}
#define DEG_LAT (360.0 / 40076.0)

struct Box {
    double lo0, lo1, hi0, hi1;
};

__device__ __forceinline__ Box pixel_box(const LayerGeom &g, int id) {
    int x = id % g.dimx, y = id / g.dimx;
    Box b;
    b.lo0 = g.mbr[0] + x * g.step_x;
    b.lo1 = g.mbr[1] + y * g.step_y;
    b.hi0 = g.mbr[0] + (x + 1) * g.step_x;
    b.hi1 = g.mbr[1] + (y + 1) * g.step_y;
    return b;
}

// Box.cpp:90-118
__device__ double box_distance(const Box &a, const Box &t, bool geo) {
    if (!(t.lo0 > a.hi0 || t.hi0 < a.lo0 || t.lo1 > a.hi1 || t.hi1 < a.lo1)) return 0;
    double dx = 0, dy = 0;
    if (t.lo1 > a.hi1)
        dy = t.lo1 - a.hi1;
    else if (t.hi1 < a.lo1)
        dy = a.lo1 - t.hi1;
    if (t.lo0 > a.hi0)
        dx = t.lo0 - a.hi0;
    else if (t.hi0 < a.lo0)
        dx = a.lo0 - t.hi0;
    if (geo) {
        dy = dy / DEG_LAT;
        dx = dx / deg_lon(a.lo1);
    }
    return sqrt(dx * dx + dy * dy);
}

// Box.cpp:120-149: the corners become float points first, and the result is
// the largest of the 16 corner-to-corner distances. A corner pair's x
// difference depends only on the two corners' x choices and its y difference
// only on their y choices, so the 16 pairs are every combination of one of
// the 4 x differences with one of the 4 y differences. Every step of a
// distance — the float subtraction, the division by the degree scale, the
// square, the sum and sqrt — is monotone in |dx| and |dy| under
// round-to-nearest, so the largest distance is the one built from the
// largest |dx| and the largest |dy|: the same double, with 2 divisions and
// one sqrt instead of 32 and 16.
__device__ __forceinline__ float4 box_corners_f(const Box &a) {
    return make_float4((float)a.lo0, (float)a.lo1, (float)a.hi0, (float)a.hi1);
}

// the same from the boxes' float corners (box_corners_f) and a's lo1
__device__ double box_max_distance_f(const float4 &fa, const float4 &ft, double a_lo1, bool geo) {
    const float ax0 = fa.x, ax1 = fa.z, ay0 = fa.y, ay1 = fa.w;
    const float tx0 = ft.x, tx1 = ft.z, ty0 = ft.y, ty1 = ft.w;
    const float mx = fmaxf(fmaxf(fabsf(__fsub_rn(ax0, tx0)), fabsf(__fsub_rn(ax0, tx1))),
                           fmaxf(fabsf(__fsub_rn(ax1, tx0)), fabsf(__fsub_rn(ax1, tx1))));
    const float my = fmaxf(fmaxf(fabsf(__fsub_rn(ay0, ty0)), fabsf(__fsub_rn(ay0, ty1))),
                           fmaxf(fabsf(__fsub_rn(ay1, ty0)), fabsf(__fsub_rn(ay1, ty1))));
    double dx = mx, dy = my;
    if (geo) {
        dy = dy / DEG_LAT;
        dx = dx / deg_lon(a_lo1);
    }
    return sqrt(dx * dx + dy * dy);
}

__device__ double box_max_distance(const Box &a, const Box &t, bool geo) {
    const float ax0 = (float)a.lo0, ax1 = (float)a.hi0, ay0 = (float)a.lo1, ay1 = (float)a.hi1;
    const float tx0 = (float)t.lo0, tx1 = (float)t.hi0, ty0 = (float)t.lo1, ty1 = (float)t.hi1;
    const float mx = fmaxf(fmaxf(fabsf(__fsub_rn(ax0, tx0)), fabsf(__fsub_rn(ax0, tx1))),
                           fmaxf(fabsf(__fsub_rn(ax1, tx0)), fabsf(__fsub_rn(ax1, tx1))));
    const float my = fmaxf(fmaxf(fabsf(__fsub_rn(ay0, ty0)), fabsf(__fsub_rn(ay0, ty1))),
                           fmaxf(fabsf(__fsub_rn(ay1, ty0)), fabsf(__fsub_rn(ay1, ty1))));
    double dx = mx, dy = my;
    if (geo) {
        dy = dy / DEG_LAT;
        dx = dx / deg_lon(a.lo1);
    }
    return sqrt(dx * dx + dy * dy);
}

// geometry_computation.h:49-89
__device__ double pt_seg_dist(float2 p, float2 p1, float2 p2, bool geo) {
    double A = __fsub_rn(p.x, p1.x), B = __fsub_rn(p.y, p1.y);
    double C = __fsub_rn(p2.x, p1.x), D = __fsub_rn(p2.y, p1.y);
    double dot = A * C + B * D;
    double len_sq = C * C + D * D;
    double param = -1;
    if (len_sq != 0) param = dot / len_sq;
    double xx, yy;
    if (param < 0) {
        xx = p1.x;
        yy = p1.y;
    } else if (param > 1) {
        xx = p2.x;
        yy = p2.y;
    } else {
        xx = p1.x + param * C;
        yy = p1.y + param * D;
    }
    double dx = p.x - xx, dy = p.y - yy;
    if (geo) {
        dx = dx / deg_lon(p.y);
        dy = dy / DEG_LAT;
    }
    return sqrt(dx * dx + dy * dy);
}

// FP32 first pass of pt_seg_dist, with a bound on its distance from the FP64
// value pt_seg_dist returns. It works relative to p1 — the reference's own
// float differences A, B, C, D and the projection parameter clamped to
// [0, 1] — so absolute coordinates never enter its rounding:
//   |d32 - d64| <= 20 u32 (M + L) S + 7 u32 d32 + 8 u64 (|p| + |p1| + M + L) S
// (taken about 3x wider below)
// with M = |A| + |B|, L = |C| + |D|, S the geography scale (1 when planar).
// The first term covers the FP32 dot/length/parameter/projection rounding
// and the float roundings of the differences the reference keeps in double;
// the second the sqrt, scaling and squares; the third the reference's own
// FP64 rounding (its projection is taken in absolute coordinates). The
// distance to a segment is 1-Lipschitz in the clamped parameter times the
// segment length, so branch flips at the clamp stay inside the bound.
__device__ __forceinline__ float pt_seg_dist32(float2 p, float2 p1, float2 p2, bool geo, float &err) {
    const float A = __fsub_rn(p.x, p1.x), B = __fsub_rn(p.y, p1.y);
    const float C = __fsub_rn(p2.x, p1.x), D = __fsub_rn(p2.y, p1.y);
    const float dot = __fadd_rn(__fmul_rn(A, C), __fmul_rn(B, D));
    const float len = __fadd_rn(__fmul_rn(C, C), __fmul_rn(D, D));
    float t = len != 0.f ? __fdiv_rn(dot, len) : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    float dx = __fsub_rn(A, __fmul_rn(t, C)), dy = __fsub_rn(B, __fmul_rn(t, D));
    float S = 1.f;
    if (geo) {
        float a = fabsf(p.y);
        if (a == 90.f) a = 89.9f;
        int idx = (int)(a * 10.f);
        if (idx < 0 || idx >= 900) idx = 899;
        // the table index may differ from the FP64 one at a boundary; taking
        // the larger neighbouring scale keeps the bound valid either way
        const float s0 = c_inv_deg_lon_f[idx];
        const float s1 = c_inv_deg_lon_f[idx + 1 < 900 ? idx + 1 : 899];
        const float s2 = c_inv_deg_lon_f[idx > 0 ? idx - 1 : 0];
        const float sy = (float)(40076.0 / 360.0);
        dx = __fmul_rn(dx, s0);
        dy = __fmul_rn(dy, sy);
        S = fmaxf(fmaxf(fmaxf(s0, s1), s2), sy);
        // a neighbouring table entry changes dx's scale: widen by that difference
        err = fabsf(__fsub_rn(A, __fmul_rn(t, C))) * fmaxf(fabsf(s1 - s0), fabsf(s2 - s0));
    } else {
        err = 0.f;
    }
    const float d = sqrtf(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    const float M = fabsf(A) + fabsf(B), L = fabsf(C) + fabsf(D);
    const float absx = fabsf(p.x) + fabsf(p.y) + fabsf(p1.x) + fabsf(p1.y);
    // the derivation's constants (20 u32, 7 u32, 8 u64), widened about 3x
    err += 4e-6f * (M + L) * S + 1.2e-6f * d + 3e-15f * (absx + M + L) * S;
    return d;
}

struct WCand {
    double apx, lo, hi;
    uint32_t pair;
    int32_t id1, id2;
    uint32_t pad;
};

struct WCandLess {
    __device__ bool operator()(const WCand &a, const WCand &b) const {
        if (a.pair != b.pair) return a.pair < b.pair;
        if (a.apx != b.apx) return a.apx < b.apx;
        if (a.lo != b.lo) return a.lo < b.lo;
        if (a.hi != b.hi) return a.hi < b.hi;
        if (a.id1 != b.id1) return a.id1 < b.id1;
        return a.id2 < b.id2;
    }
};

// out codes of the descent: 0 / 1 decided, 4 refine candidates, 2 polygon
// failed rasterization, 3 did not fit the candidate buffer (retried)
enum : uint8_t { W_FALSE = 0, W_TRUE = 1, W_BADPOLY = 2, W_RETRY = 3, W_REFINE = 4 };

struct WithinArgs {
    const uint32_t *pairs;
    uint64_t n;
    uint64_t tgt_base;
    double thr;
    int geo;
    uint32_t cap_pix;  // per-side pixel capacity of a warp's scratch
    uint32_t *scratch; // per warp: 2 sides x (bitmap words + 2 lists)
    uint64_t scratch_words;
    WCand *cand;
    unsigned long long *ncand;
    uint64_t cand_cap;
    uint8_t *out;
    unsigned long long *next;
    unsigned long long *stats;  // candidates, box pairs
};

struct SideScratch {
    uint32_t *bits;  // cap_pix/32 + 1 words
    uint32_t *q;     // current queued set
    uint32_t *p;     // next level set
    Box *box;        // the boxes of the pixels in p, and their corners as floats
    float4 *fbox;    // (lo0, lo1, hi0, hi1)
};

// u32 words of one warp's scratch: per side the boxes (8 words each) and
// float corners (4) of up to cap pixels, then per side a bitmap and two lists
__host__ __device__ inline uint64_t within_scratch_words(uint32_t cap) {
    const uint64_t w = 24ull * cap + 2 * (((uint64_t)cap >> 5) + 1 + 2ull * cap);
    return (w + 3) & ~3ull;
}

// set bit, return whether newly set
__device__ __forceinline__ void set_bit(uint32_t *bits, uint32_t id) { atomicOr(&bits[id >> 5], 1u << (id & 31)); }

// Compact the set bits of [0, nbits) into list (ascending) and clear them.
__device__ uint32_t compact_bits(uint32_t *bits, uint32_t nbits, uint32_t *list, int lane) {
    uint32_t nw = (nbits + 31) >> 5;
    uint32_t total = 0;
    for (uint32_t w0 = 0; w0 < nw; w0 += 32) {
        uint32_t w = w0 + lane;
        uint32_t word = w < nw ? bits[w] : 0u;
        uint32_t c = __popc(word);
        uint32_t incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t at = total + incl - c;
        while (word) {
            int b = __ffs(word) - 1;
            list[at++] = (w << 5) + b;
            word &= word - 1;
        }
        if (w < nw) bits[w] = 0u;
        total += __shfl_sync(0xffffffffu, incl, 31);
    }
    __syncwarp();
    return total;
}

// Children of the queued pixels at layer `li` (their box at the coarser
// layer, shrunk by 1e-6, then retrieve_pixels' own 1e-6) or the queued pixels
// themselves; BORDER ones only (Ideal.cpp:2513-2551).
__device__ uint32_t next_set(const PolyHdr &h, const uint8_t *status, bool advance, uint32_t li, const uint32_t *q,
                             uint32_t nq, SideScratch &sc, int lane, int cc) {
    LayerGeom g;
    layer_geom(h, li, g);
    LayerGeom pg;
    if (advance) layer_geom(h, li - 1, pg);
    const uint8_t *st = status + h.st + g.offset;
    for (uint32_t k = lane; k < nq; k += 32) {
        uint32_t id = q[k];
        if (advance) {
            Box b = pixel_box(pg, (int)id);
            b.lo0 += 1e-6;
            b.lo1 += 1e-6;
            b.hi0 -= 1e-6;
            b.hi1 -= 1e-6;
            int sx = offset_x(g.mbr, g.step_x, g.dimx, b.lo0 + 1e-6);
            int sy = offset_y(g.mbr, g.step_y, g.dimy, b.lo1 + 1e-6);
            int ex = offset_x(g.mbr, g.step_x, g.dimx, b.hi0 - 1e-6);
            int ey = offset_y(g.mbr, g.step_y, g.dimy, b.hi1 - 1e-6);
            for (int x = sx; x <= ex; x++)
                for (int y = sy; y <= ey; y++) {
                    uint32_t c = (uint32_t)(y * g.dimx + x);
                    if (show_status(st[c], cc) == 1) set_bit(sc.bits, c);
                }
        } else if (show_status(st[id], cc) == 1) {
            set_bit(sc.bits, id);
        }
    }
    __syncwarp();
    return compact_bits(sc.bits, (uint32_t)(g.dimx * g.dimy), sc.p, lane);
}

__global__ void __launch_bounds__(256) k_within_descend(const StoreView sv, WithinArgs a) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int cc = sv.category_count;
    const bool geo = a.geo != 0;
    uint32_t *wbase = a.scratch + warp * a.scratch_words;
    const uint32_t cap = a.cap_pix;
    Box *boxes = reinterpret_cast<Box *>(wbase);
    float4 *fboxes = reinterpret_cast<float4 *>(wbase + 16ull * cap);
    uint32_t *base = wbase + 24ull * cap;
    const uint32_t bw = (cap >> 5) + 1;
    SideScratch ss{base, base + bw, base + bw + cap, boxes, fboxes};
    SideScratch ts{base + bw + 2 * cap, base + 2 * bw + 2 * cap, base + 2 * bw + 3 * cap, boxes + cap, fboxes + cap};
    unsigned long long my_cand = 0, my_box = 0;
    for (;;) {
        unsigned long long pid = 0;
        if (lane == 0) pid = atomicAdd(a.next, 1ull);
        pid = __shfl_sync(0xffffffffu, pid, 0);
        if (pid >= a.n) break;
        const uint32_t s = a.pairs[2 * pid], t = a.pairs[2 * pid + 1];
        const PolyHdr &S = sv.hdr[s];
        const PolyHdr &T = sv.hdr[a.tgt_base + t];
        if (S.err || T.err) {
            if (lane == 0) a.out[pid] = W_BADPOLY;
            continue;
        }
        if (S.num_layers == 0 || T.num_layers == 0) {
            if (lane == 0) a.out[pid] = W_RETRY;
            continue;
        }
        const uint32_t sL = S.num_layers - 1, tL = T.num_layers - 1;
        // initial queue: every layer-0 pixel pair (Ideal.cpp:2483-2488)
        uint32_t nqs, nqt;
        {
            LayerGeom g0;
            layer_geom(S, 0, g0);
            nqs = (uint32_t)(g0.dimx * g0.dimy);
            for (uint32_t k = lane; k < nqs; k += 32) ss.q[k] = k;
            layer_geom(T, 0, g0);
            nqt = (uint32_t)(g0.dimx * g0.dimy);
            for (uint32_t k = lane; k < nqt; k += 32) ts.q[k] = k;
            __syncwarp();
        }
        uint32_t i = 0, j = 0;
        uint8_t result = W_FALSE;
        for (;;) {
            LayerGeom gs, gt;
            layer_geom(S, i, gs);
            layer_geom(T, j, gt);
            const double s_step = gs.step_x, t_step = gt.step_x;
            bool s_next = false, t_next = false;
            if (i < sL && (s_step >= t_step || j >= tL)) {
                i++;
                s_next = true;
            }
            if (j < tL && (s_step <= t_step || i >= sL)) {
                j++;
                t_next = true;
            }
            if (nqs == 0 || nqt == 0) break;  // empty queue
            uint32_t np_s = next_set(S, sv.status, s_next, i, ss.q, nqs, ss, lane, cc);
            uint32_t np_t = next_set(T, sv.status, t_next, j, ts.q, nqt, ts, lane, cc);
            layer_geom(S, i, gs);
            layer_geom(T, j, gt);
            // each pixel's box and float corners once per level, for all the
            // box pairs it is in (the same values as computed per pair)
            for (uint32_t k = lane; k < np_s; k += 32) {
                const Box b = pixel_box(gs, (int)ss.p[k]);
                ss.box[k] = b;
                ss.fbox[k] = box_corners_f(b);
            }
            for (uint32_t k = lane; k < np_t; k += 32) {
                const Box b = pixel_box(gt, (int)ts.p[k]);
                ts.box[k] = b;
                ts.fbox[k] = box_corners_f(b);
            }
            __syncwarp();
            // smallest box max-distance; any <= d decides (Ideal.cpp:2557-2570)
            const uint64_t tot = (uint64_t)np_s * np_t;
            double mbd = 100000.0;
            bool hit = false;
            for (uint64_t k = lane; k < tot; k += 32) {
                const uint32_t k1 = (uint32_t)(k / np_t), k2 = (uint32_t)(k % np_t);
                double md = box_max_distance_f(ss.fbox[k1], ts.fbox[k2], ss.box[k1].lo1, geo);
                if (md <= a.thr) {
                    hit = true;
                    break;
                }
                mbd = mbd < md ? mbd : md;
            }
            if (lane == 0) my_box += tot;
            if (__any_sync(0xffffffffu, hit)) {
                result = W_TRUE;
                break;
            }
            for (int o = 16; o; o >>= 1) {
                double v = __shfl_xor_sync(0xffffffffu, mbd, o);
                mbd = mbd < v ? mbd : v;
            }
            const bool last = !s_next && !t_next;
            // keep pairs with box distance <= d and < the smallest max-distance
            bool overflow = false;
            unsigned long long nc = 0;
            for (uint64_t k0 = 0; k0 < tot; k0 += 32) {
                uint64_t k = k0 + lane;
                bool keep = false;
                uint32_t id1 = 0, id2 = 0;
                Box b1, b2;
                double lo = 0;
                if (k < tot) {
                    const uint32_t k1 = (uint32_t)(k / np_t), k2 = (uint32_t)(k % np_t);
                    id1 = ss.p[k1];
                    id2 = ts.p[k2];
                    b1 = ss.box[k1];
                    b2 = ts.box[k2];
                    lo = box_distance(b1, b2, geo);
                    keep = !(lo > a.thr) && lo < mbd;
                }
                if (!last) {
                    if (keep) {
                        set_bit(ss.bits, id1);
                        set_bit(ts.bits, id2);
                    }
                    continue;
                }
                unsigned m = __ballot_sync(0xffffffffu, keep);
                if (!m) continue;
                unsigned long long at = 0;
                if (lane == 0) at = atomicAdd(a.ncand, (unsigned long long)__popc(m));
                at = __shfl_sync(0xffffffffu, at, 0) + __popc(m & ((1u << lane) - 1));
                nc += __popc(m);
                if (keep) {
                    if (at < a.cand_cap) {
                        // Ideal.cpp:2587-2606
                        double hi = box_max_distance(b1, b2, geo);
                        int pf = classify(sv.areas[S.pix + id1] + sv.areas[T.pix + id2],
                                          S.step_x * S.step_y + T.step_x * T.step_y, 20);
                        WCand c;
                        c.apx = lo + (double)c_mean20[pf] * (hi - lo);
                        c.lo = lo;
                        c.hi = hi;
                        c.pair = (uint32_t)pid;
                        c.id1 = (int32_t)id1;
                        c.id2 = (int32_t)id2;
                        c.pad = 0;
                        a.cand[at] = c;
                    } else {
                        overflow = true;
                    }
                }
            }
            if (last) {
                overflow = __any_sync(0xffffffffu, overflow);
                result = overflow ? W_RETRY : (nc ? W_REFINE : W_FALSE);
                if (lane == 0) my_cand += nc;
                break;
            }
            __syncwarp();
            nqs = compact_bits(ss.bits, (uint32_t)(gs.dimx * gs.dimy), ss.q, lane);
            nqt = compact_bits(ts.bits, (uint32_t)(gt.dimx * gt.dimy), ts.q, lane);
        }
        // leave the scratch bitmaps clean for the next pair
        __syncwarp();
        for (uint32_t w = lane; w < bw; w += 32) {
            ss.bits[w] = 0u;
            ts.bits[w] = 0u;
        }
        __syncwarp();
        if (lane == 0) a.out[pid] = result;
    }
    if (lane == 0) {
        atomicAdd(&a.stats[0], my_cand);
        atomicAdd(&a.stats[1], my_box);
    }
}

// first candidate of each pair (candidates sorted by pair)
__global__ void k_cand_bounds(const WCand *__restrict__ c, uint64_t n, uint64_t *__restrict__ first) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        if (k == 0 || c[k - 1].pair != c[k].pair) first[c[k].pair] = k;
    }
}

// Work order of the refinement: the pairs with the most candidates first
// (longest-first scheduling, so that the pass does not end on a long pair
// that started last). key[p] = ~(candidates of p) at p's last candidate;
// pairs without candidates keep the all-ones key and come last. Results are
// written by pair index, so the order is invisible.
__global__ void k_within_cost(const WCand *__restrict__ c, uint64_t n, const uint64_t *__restrict__ first,
                              uint32_t *__restrict__ key) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        if (k + 1 == n || c[k + 1].pair != c[k].pair) {
            const uint64_t cnt = k + 1 - first[c[k].pair];
            key[c[k].pair] = ~(uint32_t)(cnt < 0xFFFFFFFEull ? cnt : 0xFFFFFFFEull);
        }
    }
}

__global__ void k_iota32(uint32_t *__restrict__ v, uint64_t n) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        v[k] = (uint32_t)k;
}

// FARM_PAIR_ORDER=0 takes the pairs in index order
static bool within_order_on() {
    const char *v = getenv("FARM_PAIR_ORDER");
    return !(v && *v == '0');
}

// suf[k] = the smallest lo of the pair's candidates after k (100000 after the
// last), the bound Ideal.cpp:2615-2621 recomputes for every candidate; one
// warp per refined pair scans its candidates backwards 32 at a time.
__global__ void k_cand_sufmin(const WCand *__restrict__ c, uint64_t ncand, const uint64_t *__restrict__ first,
                              const uint8_t *__restrict__ out, uint64_t n, double *__restrict__ suf) {
    const int lane = threadIdx.x & 31;
    const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t pid = w0; pid < n; pid += nw) {
        if (out[pid] != W_REFINE) continue;
        const uint64_t b = first[pid];
        uint64_t e = b;
        while (e < ncand && c[e].pair == pid) e++;
        double carry = 100000.0;
        for (uint64_t hi = e; hi > b;) {
            const uint64_t cnt = hi - b < 32 ? hi - b : 32;
            const bool v = (uint64_t)lane < cnt;
            const uint64_t k = hi - 1 - lane;
            double incl = v ? c[k].lo : 100000.0;
            // inclusive min over lanes 0..lane (indices hi-1 down to k)
            for (int o = 1; o < 32; o <<= 1) {
                double x = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl = incl < x ? incl : x;
            }
            double before = __shfl_up_sync(0xffffffffu, incl, 1);  // indices after k in this chunk
            double r = lane == 0 ? carry : (carry < before ? carry : before);
            if (v) suf[k] = r;
            double last = __shfl_sync(0xffffffffu, incl, 31);
            carry = carry < last ? carry : last;
            hi -= cnt;
        }
    }
}

struct RefineArgs {
    const uint32_t *pairs;
    uint64_t n;
    uint64_t tgt_base;
    double thr;
    int geo;
    const WCand *cand;
    uint64_t ncand;
    const uint64_t *first;
    const double *suf;  // per candidate: smallest lo of the later candidates
    uint8_t *out;
    unsigned long long *next;
    unsigned long long *stats;  // seq pairs, point-segment tests
    const uint32_t *order;      // pairs taken in this order (most candidates first), or index order
};

// Ideal.cpp:2612-2643 in the candidates' order.
// exclusive warp scan of v; the warp's total in `total`
__device__ __forceinline__ uint32_t warp_scan_excl(uint32_t v, int lane, uint32_t &total) {
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - v;
}

// float <-> int keys whose signed order is the floats' order (no NaNs)
__device__ __forceinline__ int ord_key(float v) {
    const int i = __float_as_int(v);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord_val(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// Sequence pairs of one candidate pixel pair refined together (see below)
// when there are at most this many.
constexpr uint32_t kFlatSP = 64;

__global__ void __launch_bounds__(256) k_within_refine(const StoreView sv, RefineArgs a) {
    const int lane = threadIdx.x & 31;
    const bool geo = a.geo != 0;
    const int cc = sv.category_count;
    unsigned long long my_seq = 0, my_tests = 0, my_rechk = 0;
    __shared__ uint2 s_seq[8][2 * kFlatSP];
    __shared__ uint32_t s_off[8][kFlatSP + 1];
    __shared__ int s_lb[8][kFlatSP];
    const int wib = threadIdx.x >> 5;
    uint2 *sa = s_seq[wib], *sb = s_seq[wib] + kFlatSP;
    uint32_t *off = s_off[wib];
    int *lbk = s_lb[wib];
    for (;;) {
        unsigned long long pid = 0;
        if (lane == 0) {
            pid = atomicAdd(a.next, 1ull);
            if (a.order && pid < a.n) pid = a.order[pid];
        }
        pid = __shfl_sync(0xffffffffu, pid, 0);
        if (pid >= a.n) break;
        if (a.out[pid] != W_REFINE) continue;
        const uint32_t s = a.pairs[2 * pid], t = a.pairs[2 * pid + 1];
        const PolyHdr &S = sv.hdr[s];
        const PolyHdr &T = sv.hdr[a.tgt_base + t];
        const uint64_t b = a.first[pid];
        uint64_t e = b;
        while (e < a.ncand && a.cand[e].pair == pid) e++;
        const uint32_t *so = sv.offset + S.off, *to = sv.offset + T.off;
        const uint2 *sseq = sv.seq + S.seq, *tseq = sv.seq + T.seq;
        const float2 *sr = sv.ring + S.ring, *tr = sv.ring + T.ring;
        double min_dist = 100000.0;
        int decided = -1;
        for (uint64_t k = b; k < e && decided < 0; k++) {
            // lower bound of every later candidate
            const double ref = a.suf[k];
            const int id1 = a.cand[k].id1, id2 = a.cand[k].id2;
            uint32_t a0 = 0, a1 = 0, b0 = 0, b1 = 0;
            if (show_status(sv.status[S.st + id1], cc) == 1) {
                a0 = so[id1];
                a1 = so[id1 + 1];
            }
            if (show_status(sv.status[T.st + id2], cc) == 1) {
                b0 = to[id2];
                b1 = to[id2 + 1];
            }
            const uint32_t na = a1 - a0, nb = b1 - b0;
            if (na * nb <= kFlatSP) {
                // All sequence pairs of the pixel pair at once: the FP32
                // lower bounds of every (point, segment) test of every
                // sequence pair are spread over the lanes, with a minimum per
                // sequence pair; then the reference's sequential rule is
                // replayed on them in its order (source sequence outer,
                // target inner), with the FP64 minimum of a sequence pair
                // computed where its bound may lower the running minimum.
                // The bounds are those of the loop below, so the decisions
                // are the same.
                const uint32_t nsp = na * nb;
                for (uint32_t i = lane; i < na; i += 32) sa[i] = sseq[a0 + i];
                for (uint32_t j = lane; j < nb; j += 32) sb[j] = tseq[b0 + j];
                __syncwarp();
                // tests of sequence pairs lane and lane + 32
                auto sp_tests = [&](uint32_t sp) -> uint32_t {
                    if (sp >= nsp) return 0u;
                    const uint2 e1 = sa[sp / nb], e2 = sb[sp % nb];
                    return (e1.y >= 2 && e2.y >= 2) ? e2.y * (e1.y - 1) + e1.y * (e2.y - 1) : 0u;
                };
                const uint32_t sz0 = sp_tests((uint32_t)lane), sz1 = sp_tests((uint32_t)lane + 32u);
                uint32_t tot0, tot1;
                const uint32_t ex0 = warp_scan_excl(sz0, lane, tot0);
                const uint32_t ex1 = warp_scan_excl(sz1, lane, tot1);
                const uint32_t total = tot0 + tot1;
                if ((uint32_t)lane < nsp) {
                    off[lane] = ex0;
                    lbk[lane] = ord_key(3.4e38f);
                }
                if ((uint32_t)lane + 32u < nsp) {
                    off[lane + 32] = tot0 + ex1;
                    lbk[lane + 32] = ord_key(3.4e38f);
                }
                if (lane == 0) off[nsp] = total;
                __syncwarp();
                for (uint32_t t0 = 0; t0 < total; t0 += 32) {
                    const uint32_t t = t0 + lane;
                    if (t < total) {
                        uint32_t lo = 0, hi = nsp;  // the last sp with off[sp] <= t
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (off[mid] <= t) lo = mid; else hi = mid;
                        }
                        const uint32_t sp = lo, k2 = t - off[sp];
                        const uint2 e1 = sa[sp / nb], e2 = sb[sp % nb];
                        const uint32_t n1 = e2.y * (e1.y - 1);
                        float d, er;
                        if (k2 < n1) {
                            const uint32_t pi = k2 / (e1.y - 1), si = k2 % (e1.y - 1);
                            d = pt_seg_dist32(tr[e2.x + pi], sr[e1.x + si], sr[e1.x + si + 1], geo, er);
                        } else {
                            const uint32_t r = k2 - n1;
                            const uint32_t pi = r / (e2.y - 1), si = r % (e2.y - 1);
                            d = pt_seg_dist32(sr[e1.x + pi], tr[e2.x + si], tr[e2.x + si + 1], geo, er);
                        }
                        atomicMin(&lbk[sp], ord_key(d - er));
                    }
                }
                __syncwarp();
                for (uint32_t sp = 0; sp < nsp && decided < 0; sp++) {
                    const uint32_t nsz = off[sp + 1] - off[sp];
                    if (nsz == 0) continue;  // a sequence of fewer than 2 points
                    const uint2 e1 = sa[sp / nb], e2 = sb[sp % nb];
                    const uint32_t n1 = e2.y * (e1.y - 1), n2 = e1.y * (e2.y - 1);
                    const float lb = ord_val(lbk[sp]);
                    if (lane == 0) {
                        my_seq++;
                        my_tests += nsz;
                    }
                    if ((double)lb < min_dist) {
                        double m = 1.7976931348623157e308;
                        for (uint32_t k2 = lane; k2 < n1 + n2; k2 += 32) {
                            double dd;
                            if (k2 < n1) {
                                uint32_t pi = k2 / (e1.y - 1), si = k2 % (e1.y - 1);
                                dd = pt_seg_dist(tr[e2.x + pi], sr[e1.x + si], sr[e1.x + si + 1], geo);
                            } else {
                                uint32_t r = k2 - n1;
                                uint32_t pi = r / (e2.y - 1), si = r % (e2.y - 1);
                                dd = pt_seg_dist(sr[e1.x + pi], tr[e2.x + si], tr[e2.x + si + 1], geo);
                            }
                            m = m < dd ? m : dd;
                        }
                        for (int o = 16; o; o >>= 1) {
                            double v = __shfl_xor_sync(0xffffffffu, m, o);
                            m = m < v ? m : v;
                        }
                        if (lane == 0) my_rechk++;
                        min_dist = min_dist < m ? min_dist : m;
                    }
                    if (min_dist < a.thr) {
                        decided = 1;
                    } else if (min_dist < ref) {
                        decided = 0;
                    }
                }
                __syncwarp();
                continue;
            }
            for (uint32_t ia = a0; ia < a1 && decided < 0; ia++) {
                uint2 e1 = sseq[ia];
                for (uint32_t jb = b0; jb < b1; jb++) {
                    uint2 e2 = tseq[jb];
                    if (e1.y < 2 || e2.y < 2) continue;
                    // segment_to_segment_within_batch(target seq, source seq):
                    // e2.y target points vs e1.y - 1 source segments, and back
                    const uint32_t n1 = e2.y * (e1.y - 1), n2 = e1.y * (e2.y - 1);
                    // FP32 first: a lower bound on this sequence pair's minimum
                    float lb = 3.4e38f;
                    for (uint32_t k2 = lane; k2 < n1 + n2; k2 += 32) {
                        float d, er;
                        if (k2 < n1) {
                            uint32_t pi = k2 / (e1.y - 1), si = k2 % (e1.y - 1);
                            d = pt_seg_dist32(tr[e2.x + pi], sr[e1.x + si], sr[e1.x + si + 1], geo, er);
                        } else {
                            uint32_t r = k2 - n1;
                            uint32_t pi = r / (e2.y - 1), si = r % (e2.y - 1);
                            d = pt_seg_dist32(sr[e1.x + pi], tr[e2.x + si], tr[e2.x + si + 1], geo, er);
                        }
                        lb = fminf(lb, d - er);
                    }
                    for (int o = 16; o; o >>= 1) lb = fminf(lb, __shfl_xor_sync(0xffffffffu, lb, o));
                    if (lane == 0) {
                        my_seq++;
                        my_tests += n1 + n2;
                    }
                    // FP64 only when this pair may lower the exact running
                    // minimum, so min_dist is always the reference's value
                    if ((double)lb < min_dist) {
                        double m = 1.7976931348623157e308;
                        for (uint32_t k2 = lane; k2 < n1 + n2; k2 += 32) {
                            double d;
                            if (k2 < n1) {
                                uint32_t pi = k2 / (e1.y - 1), si = k2 % (e1.y - 1);
                                d = pt_seg_dist(tr[e2.x + pi], sr[e1.x + si], sr[e1.x + si + 1], geo);
                            } else {
                                uint32_t r = k2 - n1;
                                uint32_t pi = r / (e2.y - 1), si = r % (e2.y - 1);
                                d = pt_seg_dist(sr[e1.x + pi], tr[e2.x + si], tr[e2.x + si + 1], geo);
                            }
                            m = m < d ? m : d;
                        }
                        for (int o = 16; o; o >>= 1) {
                            double v = __shfl_xor_sync(0xffffffffu, m, o);
                            m = m < v ? m : v;
                        }
                        if (lane == 0) my_rechk++;
                        min_dist = min_dist < m ? min_dist : m;
                    }
                    if (min_dist < a.thr) {
                        decided = 1;
                        break;
                    } else if (min_dist < ref) {
                        decided = 0;
                        break;
                    }
                }
            }
        }
        if (lane == 0) a.out[pid] = decided == 1 ? W_TRUE : W_FALSE;
    }
    if (lane == 0) {
        atomicAdd(&a.stats[0], my_seq);
        atomicAdd(&a.stats[1], my_tests);
        atomicAdd(&a.stats[2], my_rechk);
    }
}

__global__ void k_within_count(const uint8_t *__restrict__ out, uint64_t n, unsigned long long *found,
                               unsigned long long *retry) {
    unsigned long long f = 0, r = 0;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        f += out[k] == W_TRUE;
        r += out[k] == W_RETRY;
    }
    for (int o = 16; o; o >>= 1) {
        f += __shfl_xor_sync(0xffffffffu, f, o);
        r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(found, f);
        atomicAdd(retry, r);
    }
}

__global__ void k_gather_retry(const uint32_t *__restrict__ pairs, const uint8_t *__restrict__ out, uint64_t n,
                               uint32_t *__restrict__ rp, uint64_t *__restrict__ ridx,
                               unsigned long long *__restrict__ cnt) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        if (out[k] != W_RETRY) continue;
        unsigned long long at = atomicAdd(cnt, 1ull);
        rp[2 * at] = pairs[2 * k];
        rp[2 * at + 1] = pairs[2 * k + 1];
        ridx[at] = k;
    }
}

__global__ void k_scatter_retry(const uint8_t *__restrict__ rout, const uint64_t *__restrict__ ridx, uint64_t n,
                                uint8_t *__restrict__ out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        out[ridx[k]] = rout[k];
}

// Within "-a" (query_within_polygon.cu:332-375): a pair the descent left
// undecided is within when one of its surviving finest pixel pairs has
// apxDist = minDist + mean (maxDist - minDist) <= the distance, in float.
// mean is (1.0 - pf / category_count) * 0.5 with both operands 8-bit
// integers (:352), so the quotient is 0 and mean is 0.5; 0.5 (max - min) is
// exact in float, so contracting the sum into an FMA rounds the same.
__global__ void k_within_apx(const WCand *__restrict__ c, uint64_t nc, const uint8_t *__restrict__ out, double thr,
                             uint8_t *__restrict__ hit) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = c[k].pair;
        if (out[p] != W_REFINE) continue;
        const float lo = (float)c[k].lo, hi = (float)c[k].hi;
        const float apx = lo + 0.5f * (hi - lo);
        if ((double)apx <= thr) hit[p] = 1;
    }
}

__global__ void k_within_apx_final(const uint8_t *__restrict__ hit, uint64_t n, uint8_t *__restrict__ out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        if (out[k] == W_REFINE) out[k] = hit[k] ? W_TRUE : W_FALSE;
}

static unsigned gbw(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    uint64_t cap = 32ull * sm_count();
    if (g > cap) g = cap;
    return (unsigned)(g ? g : 1);
}

// One descend + sort + refine round over n device pairs with out in device memory.
static int within_round(farm_store *s, const uint32_t *dpairs, uint64_t n, uint8_t *dout, double thr, int geo,
                        int mode, uint64_t tgt_base, uint32_t cap_pix, int nwarps, uint64_t cand_cap,
                        farm_stats *acc, int &launches) {
    cudaStream_t st = s->stream;
    StoreView sv = s->view();
    const uint64_t words = within_scratch_words(cap_pix);
    DevBuf &scr = s->s[Q_SCR0], &cand = s->s[Q_SCR1], &tmp = s->s[Q_SCR2], &first = s->s[Q_SCR3];
    FARM_TRY(scr.ensure(4 * words * (uint64_t)nwarps + 64));
    FARM_CUDA(cudaMemsetAsync(scr.p, 0, 4 * words * (uint64_t)nwarps, st));
    FARM_TRY(cand.ensure(sizeof(WCand) * cand_cap + 64));
    FARM_TRY(s->d_counters.ensure(256));
    unsigned long long *ctr = s->d_counters.as<unsigned long long>();
    FARM_CUDA(cudaMemsetAsync(ctr, 0, 256, st));
    WithinArgs wa;
    wa.pairs = dpairs;
    wa.n = n;
    wa.tgt_base = tgt_base;
    wa.thr = thr;
    wa.geo = geo;
    wa.cap_pix = cap_pix;
    wa.scratch = scr.as<uint32_t>();
    wa.scratch_words = words;
    wa.cand = cand.as<WCand>();
    wa.ncand = ctr + 1;
    wa.cand_cap = cand_cap;
    wa.out = dout;
    wa.next = ctr + 0;
    wa.stats = ctr + 2;
    // device time of the descent and of the ordered refinement (events on the
    // store's stream, read after the synchronisations below)
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    for (auto &e : ev) cudaEventCreate(&e);
    struct EvFree {
        cudaEvent_t *e;
        ~EvFree() {
            for (int k = 0; k < 3; k++)
                if (e[k]) cudaEventDestroy(e[k]);
        }
    } ev_free{ev};
    if (ev[0]) cudaEventRecord(ev[0], st);
    k_within_descend<<<nwarps / 8, 256, 0, st>>>(sv, wa);
    launches++;
    if (ev[1]) cudaEventRecord(ev[1], st);
    unsigned long long hc[4];
    FARM_CUDA(cudaMemcpyAsync(hc, ctr, 32, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    {
        float ms = 0;
        if (ev[0] && ev[1] && cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess) acc->ms_stage[1] += ms;
    }
    uint64_t nc = hc[1] < cand_cap ? hc[1] : cand_cap;
    acc->border_pairs += hc[3];
    acc->in_hits += hc[2];  // candidate pixel pairs
    if (nc && mode == FARM_MODE_APPROX) {
        // no order and no refinement: one pass over the candidates
        FARM_TRY(first.ensure(n + 64));
        uint8_t *hit = first.as<uint8_t>();
        FARM_CUDA(cudaMemsetAsync(hit, 0, n, st));
        k_within_apx<<<gbw(nc), 256, 0, st>>>(cand.as<WCand>(), nc, dout, thr, hit);
        k_within_apx_final<<<gbw(n), 256, 0, st>>>(hit, n, dout);
        launches += 2;
    } else if (nc) {
        // order by pair, then the reference's tuple (Ideal.cpp:2612)
        size_t bytes = 0;
        FARM_CUDA(cub::DeviceMergeSort::SortKeys(nullptr, bytes, cand.as<WCand>(), (int64_t)nc, WCandLess(), st));
        FARM_TRY(tmp.ensure(bytes + 64));
        FARM_CUDA(cub::DeviceMergeSort::SortKeys(tmp.p, bytes, cand.as<WCand>(), (int64_t)nc, WCandLess(), st));
        FARM_TRY(first.ensure(8 * n + 64));
        k_cand_bounds<<<gbw(nc), 256, 0, st>>>(cand.as<WCand>(), nc, first.as<uint64_t>());
        RefineArgs ra;
        ra.pairs = dpairs;
        ra.n = n;
        ra.tgt_base = tgt_base;
        ra.thr = thr;
        ra.geo = geo;
        ra.cand = cand.as<WCand>();
        ra.ncand = nc;
        ra.first = first.as<uint64_t>();
        DevBuf &suf = s->s[Q_WITHIN_SUF];
        FARM_TRY(suf.ensure(8 * nc + 64));
        k_cand_sufmin<<<sm_count() * 8, 256, 0, st>>>(cand.as<WCand>(), nc, first.as<uint64_t>(), dout, n,
                                                      suf.as<double>());
        launches++;
        ra.suf = suf.as<double>();
        ra.out = dout;
        ra.next = ctr + 4;
        ra.stats = ctr + 5;
        ra.order = nullptr;
        if (within_order_on() && n > 1 && n < 0xFFFFFFFFull) {
            FARM_TRY(s->s[Q_PAIR_ORDER].ensure(16 * n + 64));
            uint32_t *key = s->s[Q_PAIR_ORDER].as<uint32_t>(), *key_s = key + n, *idx = key_s + n, *idx_s = idx + n;
            FARM_CUDA(cudaMemsetAsync(key, 0xFF, 4 * n, st));
            k_within_cost<<<gbw(nc), 256, 0, st>>>(cand.as<WCand>(), nc, first.as<uint64_t>(), key);
            k_iota32<<<gbw(n), 256, 0, st>>>(idx, n);
            launches += 2;
            size_t ob = 0;
            FARM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, ob, key, key_s, idx, idx_s, (int64_t)n, 0, 32, st));
            FARM_TRY(s->cub_tmp.ensure(ob + 64));
            FARM_CUDA(cub::DeviceRadixSort::SortPairs(s->cub_tmp.p, ob, key, key_s, idx, idx_s, (int64_t)n, 0, 32,
                                                      st));
            ra.order = idx_s;
        }
        k_within_refine<<<sm_count() * 8, 256, 0, st>>>(sv, ra);
        launches += 2;
        if (ev[2]) cudaEventRecord(ev[2], st);
        unsigned long long hs[3];
        FARM_CUDA(cudaMemcpyAsync(hs, ctr + 5, 24, cudaMemcpyDeviceToHost, st));
        FARM_CUDA(cudaStreamSynchronize(st));
        {
            float ms = 0;
            if (ev[1] && ev[2] && cudaEventElapsedTime(&ms, ev[1], ev[2]) == cudaSuccess) acc->ms_stage[2] += ms;
        }
        acc->sequence_pairs += hs[0];
        acc->segment_tests += hs[1];
        acc->fp64_rechecks += hs[2];
    }
    return FARM_OK;
}

int within(farm_store *s, const uint32_t *pairs, uint64_t n, double distance, int geography, int self, int mode,
           int mem, uint8_t *out, uint64_t *found, farm_stats *st) {
    if (mode != FARM_MODE_EXACT && mode != FARM_MODE_APPROX) {
        set_error("farm_within: mode must be FARM_MODE_EXACT or FARM_MODE_APPROX");
        return FARM_EINVAL;
    }
    if (!s->rasterized || !s->ropts.hierarchy) {
        set_error("farm_within: rasterize with hierarchy first");
        return FARM_EINVAL;
    }
    if (!self && s->n_side[1] == 0) {
        set_error("farm_within: no target side loaded (or pass target_is_source)");
        return FARM_EINVAL;
    }
    FARM_TRY(check_pairs(s, pairs, n, mem, self != 0, "farm_within"));
    FARM_TRY(ensure_tables(s->device));
    cudaStream_t stream = s->stream;
    const uint64_t tgt_base = self ? 0 : s->n_side[0];
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
    // the largest finest raster bounds a warp's pixel sets
    uint32_t cap = 64;
    {
        std::vector<PolyHdr> hh(s->n_poly);
        FARM_CUDA(cudaMemcpyAsync(hh.data(), s->d_hdr.p, sizeof(PolyHdr) * s->n_poly, cudaMemcpyDeviceToHost, stream));
        FARM_CUDA(cudaStreamSynchronize(stream));
        for (auto &h : hh) {
            if (h.err) continue;
            for (uint32_t li = 0; li < h.num_layers; li++) {
                LayerGeom g;
                layer_geom(h, li, g);
                uint32_t np = (uint32_t)(g.dimx * g.dimy);
                if (np > cap) cap = np;
            }
        }
        cap = (cap + 31) & ~31u;
    }
    farm_stats acc;
    memset(&acc, 0, sizeof acc);
    int launches = 0;
    FARM_CUDA(cudaEventRecord(s->ev[6], stream));
    int nwarps = sm_count() * 8 * 2;
    size_t freeb = 0, totb = 0;
    cudaMemGetInfo(&freeb, &totb);
    const uint64_t words = within_scratch_words(cap);
    while (nwarps > 64 && 4ull * words * (uint64_t)nwarps > freeb / 4) nwarps /= 2;
    uint64_t cand_cap = 1ull << 24;
    if (n) FARM_TRY(within_round(s, dpairs, n, dout, distance, geography, mode, tgt_base, cap, nwarps, cand_cap,
                                 &acc, launches));
    // pairs whose candidates did not fit: gather and rerun with a larger buffer
    for (int round = 0; round < 8 && n; round++) {
        FARM_TRY(s->d_counters.ensure(256));
        unsigned long long *ctr = s->d_counters.as<unsigned long long>() + 16;
        FARM_CUDA(cudaMemsetAsync(ctr, 0, 16, stream));
        k_within_count<<<gbw(n), 256, 0, stream>>>(dout, n, ctr, ctr + 1);
        launches++;
        unsigned long long hc[2];
        FARM_CUDA(cudaMemcpyAsync(hc, ctr, 16, cudaMemcpyDeviceToHost, stream));
        FARM_CUDA(cudaStreamSynchronize(stream));
        if (hc[1] == 0) break;
        DevBuf &rp = s->s[Q_SCR4], &ro = s->s[Q_SCR5];
        FARM_TRY(rp.ensure((8 + 8) * hc[1] + 64));
        FARM_TRY(ro.ensure(hc[1] + 64));
        uint32_t *rpairs = rp.as<uint32_t>();
        uint64_t *ridx = reinterpret_cast<uint64_t *>(rpairs + 2 * hc[1] + 2);
        FARM_CUDA(cudaMemsetAsync(ctr, 0, 8, stream));
        k_gather_retry<<<gbw(n), 256, 0, stream>>>(dpairs, dout, n, rpairs, ridx, ctr);
        launches++;
        cand_cap *= 4;
        int rw = nwarps > 256 ? 256 : nwarps;
        FARM_TRY(within_round(s, rpairs, hc[1], ro.as<uint8_t>(), distance, geography, mode, tgt_base, cap, rw,
                              cand_cap, &acc, launches));
        k_scatter_retry<<<gbw(hc[1]), 256, 0, stream>>>(ro.as<uint8_t>(), ridx, hc[1], dout);
        launches++;
    }
    FARM_CUDA(cudaEventRecord(s->ev[7], stream));
    unsigned long long *fc = s->d_counters.as<unsigned long long>() + 20;
    FARM_CUDA(cudaMemsetAsync(fc, 0, 16, stream));
    k_within_count<<<gbw(n), 256, 0, stream>>>(dout, n, fc, fc + 1);
    launches++;
    unsigned long long hf[2] = {0, 0};
    FARM_CUDA(cudaMemcpyAsync(hf, fc, 16, cudaMemcpyDeviceToHost, stream));
    if (mem == FARM_MEM_HOST && out && n) FARM_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, stream));
    FARM_CUDA(cudaStreamSynchronize(stream));
    s->launches += (uint64_t)launches;
    if (hf[1]) {
        set_error("farm_within: some pairs exceeded the candidate buffer after retries");
        return FARM_ENOMEM;
    }
    if (found) *found = hf[0];
    if (st) {
        memset(st, 0, sizeof *st);
        st->pairs = n;
        st->found = hf[0];
        st->border_pairs = acc.border_pairs;
        st->segment_tests = acc.segment_tests;
        st->fp64_rechecks = acc.fp64_rechecks;
        st->sequence_pairs = acc.sequence_pairs;
        st->in_hits = acc.in_hits;
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[6], s->ev[7]);
        st->ms_total = ms;
        st->ms_stage[1] = acc.ms_stage[1];  // the hierarchical descent (filter)
        st->ms_stage[2] = acc.ms_stage[2];  // candidate order and the ordered refinement
        st->kernel_launches = launches;
    }
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_within(farm_store *s, const uint32_t *pairs, uint64_t n, double distance, int geography,
                           int target_is_source, int mem, uint8_t *out, uint64_t *found, farm_stats *st) {
    using namespace farm;
    if (!s || (n && !pairs)) {
        set_error("invalid arguments to farm_within");
        return FARM_EINVAL;
    }
    return within(s, pairs, n, distance, geography, target_is_source, FARM_MODE_EXACT, mem, out, found, st);
}

extern "C" int farm_within_mode(farm_store *s, const uint32_t *pairs, uint64_t n, double distance, int geography,
                                int target_is_source, int mode, int mem, uint8_t *out, uint64_t *found,
                                farm_stats *st) {
    using namespace farm;
    if (!s || (n && !pairs)) {
        set_error("invalid arguments to farm_within_mode");
        return FARM_EINVAL;
    }
    return within(s, pairs, n, distance, geography, target_is_source, mode, mem, out, found, st);
}
