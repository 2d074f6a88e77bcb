// Stage (a): rasterization of every loaded polygon on the GPU, reproducing the
// reference's CPU raster exactly (status bytes, per-pixel edge-sequence CSR,
// sorted grid-line crossing nodes, FP64 fill areas, hierarchy layers).
//
// Reference: preprocessing.cpp:4-29, MyRaster.cpp:8-33 (dims), :444-491
// (grid_align), Ideal.cpp:90-183 (process_crosses), :185-238
// (process_intersection), :252-538 (evaluate_edges), :540-573 (scanline),
// :575-918 (fill), :1008-1099 (layering / merge).
//
// The reference walks each polygon sequentially and accumulates per-pixel
// lists in std::map. Here the same lists come out of a flattened pipeline over
// all polygons at once: per-edge count -> scan -> fill, then stable radix
// sorts by pixel / line / column / cell, which reproduce the map iteration
// order (key order, then insertion order) exactly. The fill clip (strip, then
// cell) is scattered per edge into the columns and cells it touches, so its
// cost is linear in the output, not columns x vertices.
#include <cub/cub.cuh>

#include <algorithm>

#include <cmath>
#include <cstdlib>
#include <cstring>

#include "common.cuh"
#include "dfloat.cuh"

namespace farm {

struct RasterParams {
    int vpr, cc, hier;
    double gstep;           // UniversalGrid step: round_sig(360 / 2^25, 2)
    int pow2_ceil[40];      // ceil(log(2^k) / log(2.0)) as the host's libm evaluates it
};

enum Scratch {
    S_SIZES = 0,  // per-polygon size table [9][npoly+1]
    S_SCAN,       // scanned size table
    S_CNT_E,      // per-edge counts [3][nedges+1]
    S_SCAN_E,
    S_CFROM,      // crossings: from pixel, to pixel, edge
    S_CTO,
    S_CEDGE,
    S_VKEY,       // visits
    S_VVAL,
    S_VKEY2,
    S_VVAL2,
    S_SEQW,       // seq widths / positions
    S_PIXCNT,     // per pixel u32 counts (seqs, then cells)
    S_PIXSCAN,
    S_HKEY,
    S_HVAL,
    S_VNKEY,
    S_VNVAL,
    S_LINECNT,
    S_LINESCAN,
    S_COLX,       // sweep lines
    S_ROWY,
    S_TMP_A,
    S_TMP_B,
    S_CPOLY,  // column polygons of the fill sweep
    S_SMALL,  // small-point flags / scan / index
    S_SMALL_K,  // small-point sort keys and dependency lists
    S_SMALL_V,
    S_SMALL_D,
    S_PERM_K,  // walk / clip order: per-item cost keys / permutation
    S_PERM,
    S_CPCOL,    // column of each column-polygon point
    S_COLPOLY,  // polygon of each fill column
    S_ECNT16,   // per-edge walk counts from phase 1 (u16 x 3), reused by phase 2
    S_COLXF = 40,  // float forms of the sweep lines (LineF); slots 35-39 belong to the queries
    S_ROWYF = 41,
    S_WALKF = 42,  // per-polygon walk constants (WalkF)
    S_LINEBIG = 43, // grid lines too long for the shared-memory node sort
    S_XTILE = 44,   // bucketing (k_bucket): per-polygon tile and counter offsets
    S_XSLOT = 45,   // bucketing: (bucket, tile) counters and their scan
    S_XSTART = 34,  // column clip: first point of each polygon
};

// ------------------------------------------------------------ headers ----

__device__ void init_raster(PolyHdr &h, int num_pixels) {
    const double *m = h.mbr;
    double multi = fabs((m[3] - m[1]) / (m[2] - m[0]));
    // MyRaster.cpp:12 uses pow(x, 0.5); sqrt is the correctly rounded square root
    h.dimx = (int)sqrt(num_pixels / multi);
    h.dimy = (int)(h.dimx * multi);
    if (h.dimx == 0) h.dimx = 1;
    if (h.dimy == 0) h.dimy = 1;
    h.step_x = (m[2] - m[0]) / h.dimx;
    h.step_y = (m[3] - m[1]) / h.dimy;
    if (h.step_x < 0.00001) {
        h.step_x = 0.00001;
        h.dimx = (int)((m[2] - m[0]) / h.step_x + 1);
    }
    if (h.step_y < 0.00001) {
        h.step_y = 0.00001;
        h.dimy = (int)((m[3] - m[1]) / h.step_y + 1);
    }
}

__device__ bool grid_align(PolyHdr &h, double gstep) {
    bool f1 = false, f2 = false;
    double x = gstep, y = gstep;
    if (h.step_x <= x) { h.step_x = x; f1 = true; }
    if (h.step_y <= y) { h.step_y = y; f2 = true; }
    for (int i = 25; i > 0; i--) {
        if (!f1 && h.step_x > x && h.step_x < x * 2) {
            f1 = true;
            h.step_x = fabs(h.step_x - x) < fabs(h.step_x - x * 2) ? x : x * 2;
        }
        if (!f2 && h.step_y > y && h.step_y < y * 2) {
            f2 = true;
            h.step_y = fabs(h.step_y - y) < fabs(h.step_y - y * 2) ? y : y * 2;
        }
        if (f1 && f2) break;
        x *= 2;
        y *= 2;
    }
    if (!(f1 && f2)) return false;
    h.step_x = h.step_x < h.step_y ? h.step_x : h.step_y;
    h.step_y = h.step_x;
    double *m = h.mbr;
    m[0] = floor(m[0] / h.step_x) * h.step_x;
    m[1] = floor(m[1] / h.step_y) * h.step_y;
    m[2] = ceil(m[2] / h.step_x) * h.step_x;
    m[3] = ceil(m[3] / h.step_y) * h.step_y;
    h.dimx = (int)round((m[2] - m[0]) / h.step_x);
    h.dimy = (int)round((m[3] - m[1]) / h.step_y);
    return true;
}

__device__ int log2_ceil(int n, const RasterParams &rp) {
    // ceil(log(n) / log(2.0)): exact for non powers of two (the quotient is
    // then irrational and far from an integer); powers of two use the host
    // library's own rounding.
    if (n <= 1) return 0;
    if ((n & (n - 1)) == 0) return rp.pow2_ceil[__ffs(n) - 1];
    return 32 - __clz(n - 1);
}

__device__ void layering(PolyHdr &h, const RasterParams &rp) {
    int a = log2_ceil(h.dimx, rp), b = log2_ceil(h.dimy, rp);
    int high = a > b ? a : b;
    int low = high;
    double dx = h.dimx, dy = h.dimy;
    for (int i = high - 1; i >= 0; i--) {
        if (dx * dy <= 1) break;
        dx = (int)ceil(dx / 2.0);
        dy = (int)ceil(dy / 2.0);
        low--;
    }
    h.num_layers = (uint32_t)(high - low + 1);
}

// One warp per polygon: MBR (vertex_sequence.cpp:152-168), raster geometry.
__global__ void k_header(const float2 *__restrict__ ring, const uint64_t *__restrict__ off, uint32_t npoly,
                         RasterParams rp, PolyHdr *__restrict__ hdr, uint64_t *__restrict__ sizes) {
    uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = warp; p < npoly; p += nwarps) {
        uint64_t b = off[p], e = off[p + 1];
        const float2 *r = ring + b + 2ull * p;
        uint32_t m = (uint32_t)(e - b);
        double lx = 100000.0, ly = 100000.0, hx = -100000.0, hy = -100000.0;
        for (uint32_t j = lane; j < m; j += 32) {
            float2 q = r[j];
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
            PolyHdr h;
            memset(&h, 0, sizeof h);
            const double bias = (double)1e-9f;
            h.mbr[0] = lx - bias;
            h.mbr[1] = ly - bias;
            h.mbr[2] = hx + bias;
            h.mbr[3] = hy + bias;
            h.nv = m + 1;
            h.ring = b + 2ull * p;
            h.edge = b;
            init_raster(h, (int)(h.nv / (uint32_t)rp.vpr));
            if (rp.hier) {
                if (!grid_align(h, rp.gstep)) h.err = FARM_EASSERT;
                layering(h, rp);
            } else {
                h.num_layers = 0;
            }
            h.P = (uint32_t)h.dimx * (uint32_t)h.dimy;
            uint32_t ss = h.P;
            if (rp.hier && h.num_layers > 1) {
                LayerGeom g;
                layer_geom(h, 0, g);
                ss = g.offset + (uint32_t)(g.dimx * g.dimy);
            }
            h.status_size = ss;
            hdr[p] = h;
            uint64_t n1 = (uint64_t)npoly + 1;
            sizes[0 * n1 + p] = h.P;
            sizes[1 * n1 + p] = h.status_size;
            sizes[2 * n1 + p] = (uint64_t)h.P + 1;
            sizes[3 * n1 + p] = (uint64_t)h.dimy + 2;
            sizes[4 * n1 + p] = (uint64_t)h.dimx + 2;
            sizes[5 * n1 + p] = (uint64_t)h.dimx + 2;  // fill sweep columns
            sizes[6 * n1 + p] = (uint64_t)h.dimy + 2;  // fill sweep rows
            sizes[7 * n1 + p] = (uint64_t)h.dimy;      // scanline rows
        }
    }
}

// Bases from the scanned sizes, and the fill sweep lines (Ideal.cpp:829-851,
// :869-875): Xi accumulates by repeated addition, exactly as the loop does.
// The line after the last column (row) is stored too, with each line's float
// forms (LineF, declared with the fill kernels).
struct LineF;
__device__ inline void put_line(double *lines, LineF *lf, uint64_t at, double v);

__global__ void k_bases(PolyHdr *__restrict__ hdr, uint32_t npoly, const uint64_t *__restrict__ scan,
                        double *__restrict__ colx, double *__restrict__ rowy, LineF *__restrict__ colf,
                        LineF *__restrict__ rowf) {
    uint64_t n1 = (uint64_t)npoly + 1;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npoly; p += gridDim.x * blockDim.x) {
        PolyHdr h = hdr[p];
        h.pix = scan[0 * n1 + p];
        h.st = scan[1 * n1 + p];
        h.off = scan[2 * n1 + p];
        h.hline = scan[3 * n1 + p];
        h.vline = scan[4 * n1 + p];
        h.col = scan[5 * n1 + p];
        h.row = scan[6 * n1 + p];
        double Xi = h.mbr[0];
        double Xi1 = Xi + h.step_x;
        double kx = Xi + h.dimx * h.step_x;
        int c = 0;
        while (Xi1 < kx + 1e-9) {
            if (c > h.dimx) {  // the reference's get_id asserts x < dimx
                h.err = FARM_EASSERT;
                break;
            }
            put_line(colx, colf, h.col + c, Xi);
            Xi += h.step_x;
            Xi1 = Xi + h.step_x;
            c++;
        }
        put_line(colx, colf, h.col + c, Xi);  // c <= dimx + 1 < dimx + 2 entries
        if (c > h.dimx) h.err = FARM_EASSERT;
        h.ncols = c;
        double Yi = h.mbr[1];
        double Yi1 = Yi + h.step_y;
        double ky = h.mbr[1] + h.dimy * h.step_y;
        int r = 0;
        while (Yi1 < ky + 1e-9) {
            if (r > h.dimy) {
                h.err = FARM_EASSERT;
                break;
            }
            put_line(rowy, rowf, h.row + r, Yi);
            Yi += h.step_y;
            Yi1 = Yi + h.step_y;
            r++;
        }
        put_line(rowy, rowf, h.row + r, Yi);
        if (r > h.dimy) h.err = FARM_EASSERT;
        h.nrows = r;
        hdr[p] = h;
    }
}

// ---------------------------------------------------------- edge walk ----
// Ideal.cpp:259-521 for one edge. Sink receives: border(x, y), cross(from,
// to) (a LEAVE/ENTER pair), hnode(line, value), vnode(line, value).
//
// FP64 is GB300's scarcest pipe (2 lanes per clock per SM against 128 for
// FP32), and every quotient of the reference's walk only feeds an integer
// decision: the truncation and 1e-8 snap of double_to_int for the endpoint
// cells, the 1e-9 grid-corner test and the truncation of the x-branch, the
// truncation of the y-branch. Each is evaluated in double-float arithmetic
// on the FP32 pipe with a bound on its distance from the reference's double
// (cval, dfloat.cuh); when no decision threshold lies within that bound the
// decision is the reference's, and otherwise the reference's FP64 expression
// decides. Only the emitted node values (the v-node ordinates and h-node
// abscissae, doubles) are computed in FP64, and only by the fill pass.

// Per polygon: start, step and 1 / step of both axes split into
// double-floats (k_bases), the walk's constants.
struct WalkF {
    dflt sx, sy, tx, ty, ix, iy;
};

__device__ inline dflt split_d(double v) {
    const float hi = __double2float_rn(v);
    return {hi, __double2float_rn(v - (double)hi)};
}

// Where a quotient q (within e of the reference's double Q) sits between
// integers: fi = floor, d0 = q - fi, d1 = fi + 1 - q, each accurate to a
// rounding of itself when small. false when q is out of the float range used.
__device__ inline bool frac_parts(dflt q, float &fi, float &d0, float &d1) {
    if (!(fabsf(q.hi) < 4194304.f)) return false;
    fi = floorf(q.hi);
    if (q.hi == fi) {
        if (q.lo < 0.f) {
            fi = __fsub_rn(fi, 1.f);
            d0 = __fadd_rn(1.f, q.lo);
            d1 = -q.lo;
        } else {
            d0 = q.lo;
            d1 = __fsub_rn(1.f, q.lo);
        }
    } else {
        d0 = __fadd_rn(__fsub_rn(q.hi, fi), q.lo);
        d1 = __fsub_rn(__fsub_rn(__fadd_rn(fi, 1.f), q.hi), q.lo);
    }
    return true;
}

// double_to_int(Q) (util.h:98-106) for the reference's quotient Q within e
// of q, Q >= 0: the integer part, plus one when the next integer is less
// than 1e-8 away. -1 when undecided.
__device__ inline int d2i_cert(const cval &q) {
    float fi, d0, d1;
    if (!frac_parts(q.v, fi, d0, d1) || fi < 0.f) return -1;
    const float m = __fadd_rn(__fadd_rn(q.e, __fmul_rn(2.f * kU, d1)), 1e-15f);
    if (fabsf(__fsub_rn(d1, 1e-8f)) <= m) return -1;
    return (int)fi + (d1 < 1e-8f ? 1 : 0);
}

// The walk's decisions by the reference's FP64 expressions, for the
// undecided cases only (out of line, so that their divisions are never
// evaluated ahead of the test that selects them).
__device__ __noinline__ int cell_fp64(float v, double start, double step) {
    return double_to_int(((double)v - start) / step);
}
__device__ __noinline__ int xstep_fp64(int xl, double start_x, double step_x, double start_y, double step_y, double a,
                                       double b, int *cur_y) {
    const double xval = (double)xl * step_x + start_x;
    const double yval = xval * a + b;
    const double q = (yval - start_y) / step_y;
    *cur_y = (int)q;
    return fabs(q - round(q)) < 1e-9 ? 1 : 0;
}
__device__ __noinline__ int ystep_fp64(int yl, double start_x, double step_x, double start_y, double step_y, double a,
                                       double b) {
    const double yval = (double)yl * step_y + start_y;
    const double xval = (yval - b) / a;
    return (int)((xval - start_x) / step_x);
}
// the h-node abscissa the fill pass emits (Ideal.cpp:476)
__device__ __noinline__ double hnode_fp64(int yl, double start_y, double step_y, double a, double b) {
    return ((double)yl * step_y + start_y - b) / a;
}
// the line of the reference (Ideal.cpp:371-372)
__device__ __noinline__ void line_ab_fp64(float x1, float y1, float x2, float y2, double *a, double *b) {
    *a = ((double)y1 - (double)y2) / ((double)x1 - (double)x2);
    *b = ((double)x1 * (double)y2 - (double)x2 * (double)y1) / ((double)x1 - (double)x2);
}

// double_to_int((v - start) / step) for a vertex coordinate v
__device__ inline int cell_of(float v, const dflt &s, const dflt &is, double start, double step) {
    const cval q = cv_mul(cv_add(cv_f(v), cv_neg(cv_d(s))), cv_d(is));
    const int r = d2i_cert(q);
    return r >= 0 ? r : cell_fp64(v, start, step);
}

template <typename Sink>
__device__ void walk_edge(const PolyHdr &h, const WalkF &g, float2 A, float2 B, Sink &s) {
    const double start_x = h.mbr[0], start_y = h.mbr[1];
    const double step_x = h.step_x, step_y = h.step_y;
    const int dimx = h.dimx, dimy = h.dimy;
    const float x1 = A.x, y1 = A.y, x2 = B.x, y2 = B.y;
    int cur_startx = cell_of(x1, g.sx, g.ix, start_x, step_x);
    int cur_endx = cell_of(x2, g.sx, g.ix, start_x, step_x);
    int cur_starty = cell_of(y1, g.sy, g.iy, start_y, step_y);
    int cur_endy = cell_of(y2, g.sy, g.iy, start_y, step_y);
    if (cur_startx == dimx) cur_startx--;
    if (cur_endx == dimx) cur_endx--;
    if (cur_starty == dimy) cur_starty--;
    if (cur_endy == dimy) cur_endy--;
    if (cur_startx >= dimx || cur_endx >= dimx || cur_starty >= dimy || cur_endy >= dimy) {
        s.fail();
        return;
    }
    s.border(cur_startx, cur_starty);
    s.border(cur_endx, cur_endy);
    if (cur_startx == cur_endx && cur_starty == cur_endy) return;
    if (y1 == y2) {
        if (cur_startx < cur_endx) {
            for (int x = cur_startx; x < cur_endx; x++) {
                s.vnode(x + 1, (double)y1);
                s.cross(x, cur_starty, x + 1, cur_starty);
            }
        } else {
            for (int x = cur_startx; x > cur_endx; x--) {
                s.vnode(x, (double)y1);
                s.cross(x, cur_starty, x - 1, cur_starty);
            }
        }
        return;
    }
    if (x1 == x2) {
        if (cur_starty < cur_endy) {
            for (int y = cur_starty; y < cur_endy; y++) {
                s.hnode(y + 1, (double)x1);
                s.cross(cur_startx, y, cur_startx, y + 1);
            }
        } else {
            for (int y = cur_starty; y > cur_endy; y--) {
                s.hnode(y, (double)x1);
                s.cross(cur_startx, y, cur_startx, y - 1);
            }
        }
        return;
    }
    // the line y = a x + b of the reference (Ideal.cpp:371-372), tracked:
    // a = (y1 - y2) / (x1 - x2), b = (x1 y2 - x2 y1) / (x1 - x2); the
    // products of floats are exact in double, so the numerator of b is the
    // exact difference rounded once
    const cval cdy = cv_add(cv_f(y1), cv_f(-y2));
    const cval cdx = cv_add(cv_f(x1), cv_f(-x2));
    const cval ca = cv_div(cdy, cdx);
    const cval cia = cv_div(cdx, cdy);  // 1 / a: a's own rounding is one more 2^-52 relative
    const cval cia2 = {cia.v, __fadd_rn(cia.e, __fmul_rn(kRef, fabsf(cia.v.hi)))};
    const dflt p1 = two_prod(x1, y2), p2 = two_prod(x2, y1);
    const cval cnum = cv_add({p1, 0.f}, {{-p2.hi, -p2.lo}, 0.f});
    const cval cb = cv_div(cnum, cdx);
    const cval csx = cv_d(g.sx), csy = cv_d(g.sy), ctx = cv_d(g.tx), cty = cv_d(g.ty);
    const cval cix = cv_d(g.ix), ciy = cv_d(g.iy);
    // the reference's doubles, computed on first use (fill pass values and
    // undecided steps only)
    double a = 0.0, b = 0.0;
    bool have_ab = false;
    auto need_ab = [&]() {
        if (!have_ab) {
            line_ab_fp64(x1, y1, x2, y2, &a, &b);
            have_ab = true;
        }
    };
    const int ymax = cur_endy > cur_starty ? cur_endy : cur_starty;
    const int ymin = cur_endy < cur_starty ? cur_endy : cur_starty;
    const int xmax = cur_endx > cur_startx ? cur_endx : cur_startx;
    const int xmin = cur_endx < cur_startx ? cur_endx : cur_startx;
    int x = cur_startx, y = cur_starty;
    long guard = 4L * (labs((long)cur_endx - cur_startx) + labs((long)cur_endy - cur_starty) + 4);
    while (x != cur_endx || y != cur_endy) {
        if (--guard <= 0 || s.failed()) {
            s.fail();
            return;
        }
        bool passed = false;
        if (x != cur_endx) {
            const int xl = cur_startx < cur_endx ? x + 1 : x;  // the vertical line crossed
            // xval = xl * step_x + start_x; Q = (xval * a + b - start_y) / step_y
            const cval cxv = cv_add(cv_mul(cv_f((float)xl), ctx), csx);
            const cval cq = cv_mul(cv_add(cv_add(cv_mul(cxv, ca), cb), cv_neg(csy)), ciy);
            float fi, d0, d1;
            int corner = -1, cur_y = 0;
            if (frac_parts(cq.v, fi, d0, d1)) {
                const float dist = fminf(d0, d1);
                const float m = __fadd_rn(__fadd_rn(cq.e, __fmul_rn(2.f * kU, dist)), 1e-15f);
                if (fabsf(__fsub_rn(dist, 1e-9f)) > m) {
                    corner = dist < 1e-9f ? 1 : 0;
                    cur_y = (int)fi;  // floor; equal to the truncation after the clamp below
                }
            }
            if (corner < 0) {  // undecided: the reference's FP64 expression
                need_ab();
                corner = xstep_fp64(xl, start_x, step_x, start_y, step_y, a, b, &cur_y);
            }
            if (corner) {
                // Ideal.cpp:396-422: through a grid corner
                double yval = 0.0;
                if (Sink::kValues && cur_startx < cur_endx) {
                    need_ab();
                    yval = ((double)xl * step_x + start_x) * a + b;
                }
                if (cur_startx < cur_endx && cur_starty < cur_endy) {
                    s.vnode(x + 1, yval);
                    s.cross(x, y, x + 1, y + 1);
                    x++;
                    y++;
                } else if (cur_startx < cur_endx && cur_starty > cur_endy) {
                    s.vnode(x, yval);
                    s.cross(x, y, x + 1, y - 1);
                    x++;
                    y--;
                } else if (cur_startx > cur_endx && cur_starty < cur_endy) {
                    s.cross(x, y, x - 1, y + 1);
                    x--;
                    y++;
                } else if (cur_startx > cur_endx && cur_starty > cur_endy) {
                    s.cross(x, y, x - 1, y - 1);
                    x--;
                    y--;
                }
                continue;
            }
            if (cur_y > ymax) cur_y = ymax;
            if (cur_y < ymin) cur_y = ymin;
            if (cur_y == y) {
                passed = true;
                double yval = 0.0;
                if (Sink::kValues) {
                    need_ab();
                    yval = ((double)xl * step_x + start_x) * a + b;
                }
                if (cur_startx < cur_endx) {
                    s.vnode(x + 1, yval);
                    s.cross(x, y, x + 1, y);
                    x++;
                } else {
                    s.vnode(x, yval);
                    s.cross(x, y, x - 1, y);
                    x--;
                }
            }
        }
        if (y != cur_endy) {
            const int yl = cur_starty < cur_endy ? y + 1 : y;  // the horizontal line crossed
            // yval = yl * step_y + start_y; xval = (yval - b) / a; Q = (xval - start_x) / step_x
            const cval cyv = cv_add(cv_mul(cv_f((float)yl), cty), csy);
            const cval cxv = cv_mul(cv_add(cyv, cv_neg(cb)), cia2);
            const cval cq = cv_mul(cv_add(cxv, cv_neg(csx)), cix);
            float fi, d0, d1;
            int cur_x = 0;
            bool ok = false;
            if (frac_parts(cq.v, fi, d0, d1)) {
                const float dist = fminf(d0, d1);
                if (dist > __fadd_rn(__fadd_rn(cq.e, __fmul_rn(2.f * kU, dist)), 1e-15f)) {
                    cur_x = (int)fi;
                    ok = true;
                }
            }
            double xval = 0.0;
            if (!ok) {
                need_ab();
                cur_x = ystep_fp64(yl, start_x, step_x, start_y, step_y, a, b);
            }
            if (cur_x > xmax) cur_x = xmax;
            if (cur_x < xmin) cur_x = xmin;
            if (cur_x == x) {
                passed = true;
                if (Sink::kValues) {
                    need_ab();
                    xval = hnode_fp64(yl, start_y, step_y, a, b);
                }
                if (cur_starty < cur_endy) {
                    s.hnode(y + 1, xval);
                    s.cross(x, y, x, y + 1);
                    y++;
                } else {
                    s.hnode(y, xval);
                    s.cross(x, y, x, y - 1);
                    y--;
                }
            }
        }
        if (!passed) {
            s.fail();
            return;
        }
    }
}

__global__ void k_walkf(const PolyHdr *__restrict__ hdr, uint32_t npoly, WalkF *__restrict__ wf) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npoly; p += gridDim.x * blockDim.x) {
        const PolyHdr &h = hdr[p];
        WalkF g;
        g.sx = split_d(h.mbr[0]);
        g.sy = split_d(h.mbr[1]);
        g.tx = split_d(h.step_x);
        g.ty = split_d(h.step_y);
        g.ix = split_d(1.0 / h.step_x);
        g.iy = split_d(1.0 / h.step_y);
        wf[p] = g;
    }
}

struct CountSink {
    static constexpr bool kValues = false;
    uint8_t *status;
    int dimx, dimy;
    uint32_t nc = 0, nh = 0, nv = 0;
    bool bad = false;
    __device__ bool inb(int x, int y) const { return x >= 0 && x < dimx && y >= 0 && y < dimy; }
    __device__ void border(int x, int y) {
        if (!inb(x, y)) {
            bad = true;
            return;
        }
        status[y * dimx + x] = 1;
    }
    __device__ void cross(int fx, int fy, int tx, int ty) {
        if (!inb(fx, fy) || !inb(tx, ty)) {
            bad = true;
            return;
        }
        status[fy * dimx + fx] = 1;
        status[ty * dimx + tx] = 1;
        nc++;
    }
    __device__ void hnode(int line, double) {
        if (line < 0 || line > dimy + 1) { bad = true; return; }
        nh++;
    }
    __device__ void vnode(int line, double) {
        if (line < 0 || line > dimx + 1) { bad = true; return; }
        nv++;
    }
    __device__ void fail() { bad = true; }
    __device__ bool failed() const { return bad; }
};

// Emits exactly what CountSink counted: the walk is deterministic and both
// sinks drop the same out-of-range items.
struct FillSink {
    static constexpr bool kValues = true;
    int dimx, dimy;
    uint32_t edge;
    uint64_t c, hn, vn;           // output cursors
    uint32_t *from, *to, *cedge;  // crossings
    uint64_t *hkey, *vkey;
    double *hval, *vval;
    uint64_t hline, vline;
    bool bad = false;
    __device__ bool inb(int x, int y) const { return x >= 0 && x < dimx && y >= 0 && y < dimy; }
    __device__ void border(int x, int y) {
        if (!inb(x, y)) bad = true;
    }
    __device__ void cross(int fx, int fy, int tx, int ty) {
        if (!inb(fx, fy) || !inb(tx, ty)) {
            bad = true;
            return;
        }
        from[c] = (uint32_t)(fy * dimx + fx);
        to[c] = (uint32_t)(ty * dimx + tx);
        cedge[c] = edge;
        c++;
    }
    __device__ void hnode(int line, double v) {
        if (line < 0 || line > dimy + 1) { bad = true; return; }
        hkey[hn] = hline + (uint64_t)line;
        hval[hn] = v;
        hn++;
    }
    __device__ void vnode(int line, double v) {
        if (line < 0 || line > dimx + 1) { bad = true; return; }
        vkey[vn] = vline + (uint64_t)line;
        vval[vn] = v;
        vn++;
    }
    __device__ void fail() { bad = true; }
    __device__ bool failed() const { return bad; }
};

// ------------------------------------------------------------ fill ----
//
// The fill sweep's column and row lines are doubles built by repeated
// addition (Ideal.cpp:829-851); each is kept with its float forms (LineF):
// rn = the float nearest to it (the clip points' coordinate on that line),
// up / dn = the smallest float >= it and the largest float <= it (so that a
// float v satisfies v >= line iff v >= up, and v <= line iff v <= dn: the
// reference's float-vs-double range tests become float compares), and
// lo = rn(line - rn), with which rn + lo carries the line to ~2^-48.
//
// The clip points' other coordinate is an FP64 expression of the reference
// rounded to float. It is evaluated in double-float arithmetic on the FP32
// pipe with an error bound that covers both this evaluation and the
// reference's own FP64 roundings (dfloat.cuh); only when a float rounding
// midpoint lies inside that bound is the reference's FP64 expression itself
// evaluated. Both paths give the reference's float, so the clip is
// bit-identical either way; FARM_RASTER_EXACT=1 forces the FP64 path.

struct LineF {
    float rn, up, dn, lo;
};

__device__ inline LineF line_f(double L) {
    LineF f;
    f.rn = __double2float_rn(L);
    const double r = (double)f.rn;
    if (r == L) {
        f.up = f.dn = f.rn;
    } else if (r > L) {
        f.up = f.rn;
        f.dn = nextafterf(f.rn, -INFINITY);
    } else {
        f.dn = f.rn;
        f.up = nextafterf(f.rn, INFINITY);
    }
    f.lo = __double2float_rn(L - r);
    return f;
}

__device__ inline void put_line(double *lines, LineF *lf, uint64_t at, double v) {
    lines[at] = v;
    lf[at] = line_f(v);
}

__device__ inline float2 mk(double x, double y) { return make_float2((float)x, (float)y); }

// range test on floats: the reference compares these promoted to double, and
// the promotion is exact, so comparing in float gives the same answer without
// the FP64 pipe
__device__ inline bool in_rngf(float lo, float hi, float v) { return !(v < lo || v > hi); }

// !(v < L0 || v > L1) for a float v and double lines L0, L1 (in_rng of the reference)
__device__ inline bool in_lines(const LineF &L0, const LineF &L1, float v) { return v >= L0.up && v <= L1.dn; }

// Points one edge contributes to column c's clip (Ideal.cpp:575-678), in order.
// pi, pi1 are the float points (Xi, yi), (Xi1, yi1) on the column lines, yi and
// yi1 the edge's ordinates there (ClipXEdge).
// Returns the count; writes up to 4 points when out != nullptr.
// emitA: false for every edge but the ring's first. Edge i's A is edge
// i-1's B (the same vertex), which edge i-1 emits last into the same column
// under the same range test, so A would follow its own bit-identical copy in
// the column's stream — a point the dedup rule always drops (a later copy of
// a kept point, or of a point dropped for equalling a kept one).
__device__ inline int clip_x_points(float2 A, float2 B, const LineF &X0, const LineF &X1, float2 pi, float2 pi1,
                                    bool emitA, float2 *out) {
    int n = 0;
    const float mny = A.y < B.y ? A.y : B.y, mxy = A.y < B.y ? B.y : A.y;
    const float mnx = A.x < B.x ? A.x : B.x, mxx = A.x < B.x ? B.x : A.x;
    if (emitA && in_lines(X0, X1, A.x)) {
        if (out) out[n] = A;
        n++;
    }
    bool c0 = in_rngf(mny, mxy, pi.y) && in_rngf(mnx, mxx, pi.x);
    bool c1 = in_rngf(mny, mxy, pi1.y) && in_rngf(mnx, mxx, pi1.x);
    if (A.x < B.x) {
        if (c0) { if (out) out[n] = pi; n++; }
        if (c1) { if (out) out[n] = pi1; n++; }
    } else {
        if (c1) { if (out) out[n] = pi1; n++; }
        if (c0) { if (out) out[n] = pi; n++; }
    }
    if (in_lines(X0, X1, B.x)) {
        if (out) out[n] = B;
        n++;
    }
    return n;
}

// The reference's FP64 expressions, evaluated only where the certified
// double-float value is undecided. Kept out of line: inlined, the compiler
// may evaluate them ahead of the test that selects them, which would issue
// their FP64 divisions for every point.
__device__ __noinline__ float clip_ord_fp64(float2 A, float2 B, double X) {
    const double sl = ((double)B.y - A.y) / (double)(B.x - A.x);
    return (float)(sl * (X - B.x) + B.y);
}
__device__ __noinline__ float clip_absc_fp64(float2 A, float2 B, double Y) {
    const double sl = ((double)B.y - A.y) / (double)(B.x - A.x);
    return (float)(((Y - B.y) / sl) + B.x);
}

// The edge's ordinate at column line X (Ideal.cpp:575-600): the reference
// computes slope = ((double)B.y - A.y) / (double)(B.x - A.x) (the x difference
// taken in float) and ord = slope * (X - B.x) + B.y in FP64, then stores it as
// a float. ordf(X) returns that float.
struct ClipXEdge {
    float2 A, B;
    bool vert;
    float ymin, dxf;
    dflt slope;      // double-float slope
    float slope_err; // bound on |slope - the reference's double slope|
    __device__ ClipXEdge(float2 a, float2 b) : A(a), B(b) {
        vert = A.x == B.x;
        ymin = A.y < B.y ? A.y : B.y;
        dxf = __fsub_rn(B.x, A.x);
        slope = {0.f, 0.f};
        slope_err = 0.f;
        if (!vert) {
            const dflt dy = two_sum(B.y, -A.y);  // exact
            slope = df_div_f(dy, dxf, &slope_err);
            // the reference rounds dy and the quotient to double: 2 x 2^-53 relative
            slope_err = __fadd_rn(slope_err, __fmul_rn(kU2 * 0.125f, fabsf(slope.hi)));
        }
    }
    __device__ float ord_exact(double X) const { return vert ? ymin : clip_ord_fp64(A, B, X); }
    __device__ float ordf(double X, const LineF &L, bool cert) const {
        if (vert) return ymin;
        if (cert) {
            float err = __fmul_rn(kU2, fabsf(L.rn));  // the line's own split (rn + lo)
            const dflt d = df_add({L.rn, L.lo}, {-B.x, 0.f}, &err);
            const float ed = err;  // |d - exact X - B.x|
            float em = 0.f;
            const dflt p = df_mul(slope, d, &em);
            float e = __fadd_rn(__fadd_rn(__fmul_rn(fabsf(slope.hi), ed), __fmul_rn(fabsf(d.hi), slope_err)), em);
            const dflt o = df_add(p, {B.y, 0.f}, &e);
            // the reference's own roundings of X - B.x, the product and the sum
            e = __fadd_rn(e, __fmul_rn(kU2 * 0.125f, __fadd_rn(__fadd_rn(__fmul_rn(fabsf(slope.hi), fabsf(d.hi)),
                                                                           fabsf(p.hi)), fabsf(o.hi))) * 2.f);
            float y;
            if (round_certified(o, e, &y)) return y;
        }
        return ord_exact(X);
    }
};

// Points one column-polygon edge contributes to row r's clip (Ideal.cpp:680-818),
// given the float points (xi, Yi), (xi1, Yi1) on the row lines and the
// parallel flag (ClipYEdge).
__device__ inline int clip_y_points(float2 A, float2 B, const LineF &Y0, const LineF &Y1, float2 pi, float2 pi1,
                                    bool parallels, float2 *out) {
    int n = 0;
    if (in_lines(Y0, Y1, A.y)) {
        if (out) out[n] = A;
        n++;
    }
    if (!parallels) {
        const float mny = A.y < B.y ? A.y : B.y, mxy = A.y < B.y ? B.y : A.y;
        const float mnx = A.x < B.x ? A.x : B.x, mxx = A.x < B.x ? B.x : A.x;
        bool c0 = in_rngf(mnx, mxx, pi.x) && in_rngf(mny, mxy, pi.y);
        bool c1 = in_rngf(mnx, mxx, pi1.x) && in_rngf(mny, mxy, pi1.y);
        if (A.y < B.y) {
            if (c0) { if (out) out[n] = pi; n++; }
            if (c1) { if (out) out[n] = pi1; n++; }
        } else {
            if (c1) { if (out) out[n] = pi1; n++; }
            if (c0) { if (out) out[n] = pi; n++; }
        }
    }
    return n;
}

// Ideal.cpp:680-730 per edge: vertical edges cut every row line at A.x;
// horizontal edges touch only a row line they lie on (the other abscissa is
// -DBL_MAX, which converts to -inf in float) and are otherwise parallel; the
// rest cut at ((Y - B.y) / slope) + B.x with the slope of ClipXEdge, and the
// abscissa is used only rounded to float (abscf).
struct ClipYEdge {
    float2 A, B;
    bool vert, horiz;
    dflt inv;      // double-float dxf / dy, the reciprocal of the reference's slope
    float inv_err; // bound on |inv - 1 / the reference's double slope|
    __device__ ClipYEdge(float2 a, float2 b) : A(a), B(b) {
        vert = A.x == B.x;
        horiz = !vert && A.y == B.y;
        inv = {0.f, 0.f};
        inv_err = 0.f;
        if (!vert && !horiz) {
            const dflt dy = two_sum(B.y, -A.y);  // exact
            inv = df_rdiv(__fsub_rn(B.x, A.x), dy, &inv_err);
            // the reference's slope carries two double roundings: 2 x 2^-53 relative
            inv_err = __fadd_rn(inv_err, __fmul_rn(kU2 * 0.125f, fabsf(inv.hi)));
        }
    }
    __device__ bool general() const { return !vert && !horiz; }
    __device__ float absc_exact(double Y) const { return clip_absc_fp64(A, B, Y); }
    __device__ float abscf(double Y, const LineF &L, bool cert) const {
        if (cert) {
            float et = __fmul_rn(kU2, fabsf(L.rn));  // the line's own split
            const dflt t = df_add({L.rn, L.lo}, {-B.y, 0.f}, &et);
            float e = 0.f;
            const dflt q = df_mul(t, inv, &e);
            e = __fadd_rn(e, __fadd_rn(__fmul_rn(fabsf(inv.hi), et), __fmul_rn(fabsf(t.hi), inv_err)));
            const dflt x = df_add(q, {B.x, 0.f}, &e);
            // the reference's own roundings of Y - B.y, the quotient and the sum
            e = __fadd_rn(e, __fmul_rn(kU2 * 0.125f,
                                       __fadd_rn(__fadd_rn(__fmul_rn(fabsf(t.hi), fabsf(inv.hi)), fabsf(q.hi)),
                                                 fabsf(x.hi))) * 2.f);
            float v;
            if (round_certified(x, e, &v)) return v;
        }
        return absc_exact(Y);
    }
};

// first index i in [0, n) whose far line lines[i + 1] could reach v, on the
// lines' float forms: up(lines[i + 1]) >= vf with vf <= v. It never lies past
// the reference's first line (lines[i] + step >= v); the lines skipped before
// that one contribute no point.
__device__ int first_line_f(const LineF *lines, int n, float vf) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (lines[mid + 1].up < vf)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// float margin covering the float rounding of a clip line coordinate: at least
// twice the reference's (|a| + |b|) * 1.2e-7 after its own rounding
__device__ inline float fmargin_f(float a, float b) { return (fabsf(a) + fabsf(b)) * 2.5e-7f + 1e-30f; }

// "Small" points: a coordinate below 2^-5 in magnitude, where two distinct
// floats can be closer than the 1e-9 of Point::operator==. Elsewhere that
// equality is bit equality (float spacing there exceeds 1e-9).
__device__ inline bool small_pt(float2 q) { return fabsf(q.x) < 0.03125f || fabsf(q.y) < 0.03125f; }

__device__ inline uint64_t pt_bits(float2 q) {
    return ((uint64_t)__float_as_uint(q.x) << 32) | (uint64_t)__float_as_uint(q.y);
}

// ======================================================= chunked pipeline ==
// Phase 1 covers every polygon at once and only accumulates per-polygon
// totals (crossings, grid-line nodes), which size the persistent outputs.
// Phase 2 runs the full pipeline over chunks of polygons whose scratch fits a
// fixed budget, writing into those outputs at each polygon's base.

struct Chunk {
    uint32_t p0, np;  // polygons
    uint64_t e0, ne;  // edges
    uint64_t pix0, npix;
    uint64_t h0, nh;     // horizontal grid lines
    uint64_t v0, nvl;    // vertical grid lines
    uint64_t col0, ncol; // fill sweep columns
    uint64_t row0, nrow; // scanline rows
    uint64_t hn0, vn0;   // global node bases of the chunk's first polygon
};

// Walk order: an FP32 estimate of the pixels an edge crosses, so that the
// lanes of a warp walk edges of similar length (the walk's trip count varies
// from 0 to dozens of steps, and a warp pays for its longest lane). The order
// only schedules the walks; every walk itself is exact.
__global__ void k_edge_cost(const StoreView sv, const PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ off,
                            uint32_t p0, uint32_t np, uint64_t e0, uint64_t ne, int x_only, uint8_t *__restrict__ key,
                            uint32_t *__restrict__ idx) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ne; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t e = e0 + k;
        uint32_t p = p0 + find_segment(off + p0, np, e);
        const PolyHdr &h = hdr[p];
        float c = 0.f;
        if (h.err == 0) {
            uint32_t i = (uint32_t)(e - h.edge);
            const float2 *r = sv.ring + h.ring;
            float2 A = r[i], B = r[i + 1];
            c = fabsf(B.x - A.x) / (float)h.step_x + (x_only ? 0.f : fabsf(B.y - A.y) / (float)h.step_y);
        }
        key[k] = (uint8_t)(c < 255.f ? c : 255.f);
        if (idx) idx[k] = (uint32_t)k;
    }
}

// Phase 1's walk: per-polygon totals, and each edge's counts kept (u16, for
// phase 2's chunks, which would otherwise walk every edge a second time only
// to count); a count above 65535 sets *ovf and phase 2 counts by walking.
__global__ void k_walk_tot(const StoreView sv, PolyHdr *__restrict__ hdr, const WalkF *__restrict__ wf,
                           const uint64_t *__restrict__ off, uint32_t npoly, uint64_t e0, uint64_t nedges, const uint32_t *__restrict__ perm,
                           unsigned long long *__restrict__ tot, uint16_t *__restrict__ c16, uint64_t ne_all,
                           int *__restrict__ ovf) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nedges;
         k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t e = e0 + perm[k];
        uint32_t p = find_segment(off, npoly, e);
        const PolyHdr &h = hdr[p];
        if (h.err) continue;  // phase 2 zeroes the counts of failed polygons
        uint32_t i = (uint32_t)(e - h.edge);
        const float2 *r = sv.ring + h.ring;
        CountSink s;
        s.status = sv.status + h.st;
        s.dimx = h.dimx;
        s.dimy = h.dimy;
        walk_edge(h, wf[p], r[i], r[i + 1], s);
        if (s.bad) atomicMin(&hdr[p].err, FARM_EASSERT);
        if (s.nc > 0xFFFFu || s.nh > 0xFFFFu || s.nv > 0xFFFFu) atomicOr(ovf, 1);
        c16[e] = (uint16_t)s.nc;
        c16[ne_all + e] = (uint16_t)s.nh;
        c16[2 * ne_all + e] = (uint16_t)s.nv;
        if (s.nc) atomicAdd(&tot[3ull * p], (unsigned long long)s.nc);
        if (s.nh) atomicAdd(&tot[3ull * p + 1], (unsigned long long)s.nh);
        if (s.nv) atomicAdd(&tot[3ull * p + 2], (unsigned long long)s.nv);
    }
}

__global__ void k_tot_sizes(const unsigned long long *__restrict__ tot, const PolyHdr *__restrict__ hdr,
                            uint32_t npoly, uint64_t *__restrict__ sz) {
    uint64_t n1 = (uint64_t)npoly + 1;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= npoly; p += gridDim.x * blockDim.x) {
        if (p == npoly) {
            sz[p] = sz[n1 + p] = sz[2 * n1 + p] = 0;
            continue;
        }
        uint64_t c = tot[3ull * p];
        sz[p] = hdr[p].err ? 0 : (c ? c + 1 : 1);
        sz[n1 + p] = hdr[p].err ? 0 : tot[3ull * p + 1];
        sz[2 * n1 + p] = hdr[p].err ? 0 : tot[3ull * p + 2];
    }
}

__global__ void k_set_node_bases(PolyHdr *__restrict__ hdr, uint32_t npoly, const uint64_t *__restrict__ sz,
                                 const uint64_t *__restrict__ sc) {
    uint64_t n1 = (uint64_t)npoly + 1;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npoly; p += gridDim.x * blockDim.x) {
        PolyHdr &h = hdr[p];
        h.seq = sc[p];
        h.n_seq = (uint32_t)sz[p];
        h.hnode = sc[n1 + p];
        h.n_hnodes = (uint32_t)sz[n1 + p];
        h.vnode = sc[2 * n1 + p];
        h.n_vnodes = (uint32_t)sz[2 * n1 + p];
    }
}

__global__ void k_walk_count(const StoreView sv, PolyHdr *__restrict__ hdr, const WalkF *__restrict__ wf,
                             const uint64_t *__restrict__ off, Chunk ch, const uint32_t *__restrict__ perm, uint32_t *__restrict__ cnt) {
    uint64_t n1 = ch.ne + 1;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ch.ne;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = perm[j];
        uint64_t e = ch.e0 + k;
        uint32_t p = ch.p0 + find_segment(off + ch.p0, ch.np, e);
        const PolyHdr &h = hdr[p];
        CountSink s;
        s.status = sv.status + h.st;
        s.dimx = h.dimx;
        s.dimy = h.dimy;
        if (h.err == 0) {
            uint32_t i = (uint32_t)(e - h.edge);
            const float2 *r = sv.ring + h.ring;
            walk_edge(h, wf[p], r[i], r[i + 1], s);
        }
        if (s.bad) atomicMin(&hdr[p].err, FARM_EASSERT);
        cnt[k] = s.nc;
        cnt[n1 + k] = s.nh;
        cnt[2 * n1 + k] = s.nv;
    }
}

// Phase 2's counts from phase 1's (the same walk, the same sink), zero for
// polygons whose rasterization failed — what k_walk_count would produce.
__global__ void k_load_counts(const PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ off, Chunk ch,
                              const uint16_t *__restrict__ c16, uint64_t ne_all, uint32_t *__restrict__ cnt) {
    uint64_t n1 = ch.ne + 1;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ch.ne;
         k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t e = ch.e0 + k;
        uint32_t p = ch.p0 + find_segment(off + ch.p0, ch.np, e);
        const bool ok = hdr[p].err == 0;
        cnt[k] = ok ? c16[e] : 0u;
        cnt[n1 + k] = ok ? c16[ne_all + e] : 0u;
        cnt[2 * n1 + k] = ok ? c16[2 * ne_all + e] : 0u;
    }
}

__global__ void k_walk_fill(const StoreView sv, const PolyHdr *__restrict__ hdr, const WalkF *__restrict__ wf,
                            const uint64_t *__restrict__ off, Chunk ch, const uint32_t *__restrict__ perm, const uint64_t *__restrict__ scan,
                            uint32_t *from, uint32_t *to, uint32_t *cedge, uint64_t *hkey, double *hval,
                            uint64_t *vkey, double *vval) {
    uint64_t n1 = ch.ne + 1;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ch.ne;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = perm[j];
        // walk exactly the edges the count pass walked (those with output)
        if (scan[k + 1] == scan[k] && scan[n1 + k + 1] == scan[n1 + k] && scan[2 * n1 + k + 1] == scan[2 * n1 + k])
            continue;
        uint64_t e = ch.e0 + k;
        uint32_t p = ch.p0 + find_segment(off + ch.p0, ch.np, e);
        const PolyHdr &h = hdr[p];
        uint32_t i = (uint32_t)(e - h.edge);
        const float2 *r = sv.ring + h.ring;
        FillSink s;
        s.dimx = h.dimx;
        s.dimy = h.dimy;
        s.edge = i;
        s.c = scan[k];
        s.hn = scan[n1 + k];
        s.vn = scan[2 * n1 + k];
        s.from = from;
        s.to = to;
        s.cedge = cedge;
        s.hkey = hkey;
        s.hval = hval;
        s.vkey = vkey;
        s.vval = vval;
        s.hline = h.hline - ch.h0;
        s.vline = h.vline - ch.v0;
        walk_edge(h, wf[p], r[i], r[i + 1], s);
    }
}

// per polygon (chunk-local) crossing base
__global__ void k_cross_base(const uint64_t *__restrict__ off, Chunk ch, const uint64_t *__restrict__ escan,
                             uint64_t *__restrict__ cbase) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q <= ch.np; q += gridDim.x * blockDim.x)
        cbase[q] = escan[off[ch.p0 + q] - ch.e0];
}

// Visits: crossing c enters pixel to[c]; the visit ends at the next crossing
// (which must leave that pixel). The ring's last crossing closes the visit to
// the start pixel that the first crossing left; it is placed first so that,
// after a stable sort by pixel, its two sequences lead that pixel's list, as
// the LEAVE-first case of Ideal.cpp:158-165 orders them.
__global__ void k_visits(PolyHdr *__restrict__ hdr, Chunk ch, const uint64_t *__restrict__ cbase, uint64_t ncross,
                         const uint32_t *__restrict__ from, const uint32_t *__restrict__ to,
                         const uint32_t *__restrict__ cedge, uint64_t *__restrict__ vkey,
                         uint64_t *__restrict__ vval) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncross;
         c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t q = find_segment(cbase, ch.np, c);
        uint64_t cb = cbase[q], ce = cbase[q + 1];
        const PolyHdr &h = hdr[ch.p0 + q];
        bool wrap = (c == ce - 1);
        uint64_t nxt = wrap ? cb : c + 1;
        if (from[nxt] != to[c]) atomicMin(&hdr[ch.p0 + q].err, FARM_EASSERT);
        uint64_t pos = wrap ? cb : c + 1;
        vkey[pos] = (h.pix - ch.pix0) + to[c];
        vval[pos] = ((uint64_t)cedge[c] << 32) | (uint64_t)cedge[nxt] | (wrap ? (1ull << 63) : 0ull);
    }
}

__global__ void k_seq_width(const uint64_t *__restrict__ vkey, const uint64_t *__restrict__ vval, uint64_t n,
                            uint64_t *__restrict__ w, uint32_t *__restrict__ pixcnt) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t wd = (vval[k] >> 63) ? 2u : 1u;
        w[k] = wd;
        atomicAdd(&pixcnt[vkey[k]], wd);
    }
}

__global__ void k_seq_fill(PolyHdr *__restrict__ hdr, Chunk ch, const uint64_t *__restrict__ cbase,
                           const uint64_t *__restrict__ vval, const uint64_t *__restrict__ wscan, uint64_t n,
                           uint2 *__restrict__ seq) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t q = find_segment(cbase, ch.np, k);
        PolyHdr &h = hdr[ch.p0 + q];
        uint64_t rel = wscan[k] - wscan[cbase[q]];
        uint64_t v = vval[k];
        uint32_t ein = (uint32_t)((v >> 32) & 0x7FFFFFFFu), eout = (uint32_t)(v & 0xFFFFFFFFu);
        uint32_t wd = (v >> 63) ? 2u : 1u;
        if (rel + wd > h.n_seq) {  // sizes disagree with the first pass
            atomicMin(&h.err, FARM_EINTERNAL);
            continue;
        }
        uint64_t at = h.seq + rel;
        if (v >> 63) {
            // add_edge(0, first leave) and add_edge(last enter, nv - 2)
            seq[at] = make_uint2(0u, eout + 1u);
            seq[at + 1] = make_uint2(ein, h.nv - 2u - ein + 1u);
        } else {
            if (eout < ein) atomicMin(&h.err, FARM_EASSERT);
            seq[at] = make_uint2(ein, eout - ein + 1u);
        }
    }
}

// Polygons without crossings: one sequence covering the ring (Ideal.cpp:523-529).
__global__ void k_seq_single(const PolyHdr *__restrict__ hdr, Chunk ch, const uint64_t *__restrict__ cbase,
                             uint2 *__restrict__ seq, uint32_t *__restrict__ pixcnt) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ch.np; q += gridDim.x * blockDim.x) {
        const PolyHdr &h = hdr[ch.p0 + q];
        if (h.err == 0 && cbase[q + 1] == cbase[q]) {
            seq[h.seq] = make_uint2(0u, h.nv);
            pixcnt[h.pix - ch.pix0] += 1;
        }
    }
}

// CSR offsets: offset[i] = sequences in pixels before i (Ideal.cpp:35-45 makes
// non-BORDER pixels repeat the next start, which is the same prefix).
__global__ void k_offsets(const PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ pixbase, Chunk ch,
                          const uint64_t *__restrict__ pscan, uint32_t *__restrict__ offset) {
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ch.npix;
         g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t p = ch.p0 + find_segment(pixbase + ch.p0, ch.np, g + ch.pix0);
        const PolyHdr &h = hdr[p];
        uint64_t lb = h.pix - ch.pix0;
        uint32_t i = (uint32_t)(g - lb);
        offset[h.off + i] = (uint32_t)(pscan[g] - pscan[lb]);
        if (i == 0) offset[h.off + h.P] = h.n_seq;
    }
}

__global__ void k_line_count(const uint64_t *__restrict__ key, uint64_t n, uint32_t *__restrict__ cnt) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[key[k]], 1u);
}

__global__ void k_line_scatter(const uint64_t *__restrict__ key, const double *__restrict__ val, uint64_t n,
                               const uint64_t *__restrict__ start, uint32_t *__restrict__ fillc,
                               double *__restrict__ out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t l = key[k];
        uint32_t r = atomicAdd(&fillc[l], 1u);
        out[start[l] + r] = val[k];
    }
}

// Grid-line node values sorted per line (Grid_line sorts each line's
// crossings, Ideal.cpp:185-238). Each line's values are a few to a few
// thousand doubles: one block sorts one line in shared memory by a bitonic
// network on order-preserving 64-bit integer keys (the integer pipe, not
// FP64 compares). Equal keys are equal doubles, so the network's lack of
// stability is invisible; -0.0 sorts before +0.0. Lines longer than
// kLineSortMax are listed for a library segmented sort.
constexpr int kLineSortMax = 4096;

__device__ inline uint64_t dkey(double v) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ inline double dval(uint64_t k) {
    const uint64_t b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}

// Lines of at most 32 nodes, most of them: one warp per line, a bitonic
// network across the lanes (shuffles, no block barrier).
__global__ void k_line_sort_warp(const double *__restrict__ in, double *__restrict__ out,
                                 const uint64_t *__restrict__ start, uint64_t nseg) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t l = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; l < nseg; l += nw) {
        const uint64_t b = start[l], n = start[l + 1] - b;
        if (n == 0 || n > 32) continue;
        uint64_t k = (uint64_t)lane < n ? dkey(in[b + lane]) : ~0ull;
        for (int size = 2; size <= 32; size <<= 1)
            for (int j = size >> 1; j > 0; j >>= 1) {
                const uint64_t o = __shfl_xor_sync(full, k, j);
                const bool up = (lane & size) == 0, lower = (lane & j) == 0;
                k = (lower == up) ? (k < o ? k : o) : (k < o ? o : k);
            }
        if ((uint64_t)lane < n) out[b + lane] = dval(k);
    }
}

// Lines of 33 to 256 nodes: one warp per line, a bitonic network over the
// line in the warp's slice of shared memory (warp barriers only).
constexpr int kLineMid = 256;
__global__ void __launch_bounds__(256) k_line_sort_mid(const double *__restrict__ in, double *__restrict__ out,
                                                       const uint64_t *__restrict__ start, uint64_t nseg) {
    __shared__ uint64_t sks[8][kLineMid];
    const int lane = threadIdx.x & 31;
    uint64_t *sk = sks[threadIdx.x >> 5];
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t l = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; l < nseg; l += nw) {
        const uint64_t b = start[l], n = start[l + 1] - b;
        if (n <= 32 || n > (uint64_t)kLineMid) continue;
        uint32_t N = 64;
        while (N < n) N <<= 1;
        for (uint32_t i = lane; i < N; i += 32) sk[i] = i < n ? dkey(in[b + i]) : ~0ull;
        __syncwarp();
        for (uint32_t k = 2; k <= N; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = lane; i < N; i += 32) {
                    const uint32_t ixj = i ^ j;
                    if (ixj > i) {
                        const uint64_t x = sk[i], y = sk[ixj];
                        if ((x > y) == ((i & k) == 0)) {
                            sk[i] = y;
                            sk[ixj] = x;
                        }
                    }
                }
                __syncwarp();
            }
        for (uint32_t i = lane; i < n; i += 32) out[b + i] = dval(sk[i]);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(256) k_line_sort(const double *__restrict__ in, double *__restrict__ out,
                                                   const uint64_t *__restrict__ start, uint64_t nseg,
                                                   uint64_t *__restrict__ big_b, uint64_t *__restrict__ big_e,
                                                   unsigned long long *__restrict__ nbig) {
    __shared__ uint64_t sk[kLineSortMax];
    for (uint64_t l = blockIdx.x; l < nseg; l += gridDim.x) {
        const uint64_t b = start[l], n = start[l + 1] - b;
        if (n <= (uint64_t)kLineMid) continue;  // k_line_sort_warp, k_line_sort_mid
        if (n > (uint64_t)kLineSortMax) {
            if (threadIdx.x == 0) {
                const unsigned long long at = atomicAdd(nbig, 1ull);
                big_b[at] = b;
                big_e[at] = b + n;
            }
            continue;
        }
        uint32_t N = 1;
        while (N < n) N <<= 1;
        for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) sk[i] = i < n ? dkey(in[b + i]) : ~0ull;
        __syncthreads();
        for (uint32_t k = 2; k <= N; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
                    const uint32_t ixj = i ^ j;
                    if (ixj > i) {
                        const uint64_t x = sk[i], y = sk[ixj];
                        if ((x > y) == ((i & k) == 0)) {
                            sk[i] = y;
                            sk[ixj] = x;
                        }
                    }
                }
                __syncthreads();
            }
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) out[b + i] = dval(sk[i]);
        __syncthreads();
    }
}

// Grid-line offsets (Ideal.cpp:185-238): lines with nodes get their start,
// others keep 0; the end entries get the node count.
__global__ void k_line_offsets(PolyHdr *__restrict__ hdr, Chunk ch, int vertical, const uint32_t *__restrict__ cnt,
                               const uint64_t *__restrict__ start, uint32_t *__restrict__ loff) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ch.np; q += gridDim.x * blockDim.x) {
        PolyHdr &h = hdr[ch.p0 + q];
        uint64_t gl = vertical ? h.vline : h.hline;
        uint64_t lb = gl - (vertical ? ch.v0 : ch.h0);
        int dim = vertical ? h.dimx : h.dimy;
        uint64_t nb = start[lb];
        uint32_t total = (uint32_t)(start[lb + dim + 2] - nb);
        uint64_t gnode = (vertical ? ch.vn0 : ch.hn0) + nb;
        if (total != (vertical ? h.n_vnodes : h.n_hnodes) || gnode != (vertical ? h.vnode : h.hnode))
            atomicMin(&h.err, FARM_EINTERNAL);
        for (int l = 0; l < dim + 2; l++) loff[gl + l] = cnt[lb + l] ? (uint32_t)(start[lb + l] - nb) : 0u;
        loff[gl + dim] = total;
        if (vertical) loff[gl + dim + 1] = total;
    }
}

// Ideal.cpp:540-573: the scanline fill of the non-BORDER pixels.
__global__ void k_scanline(const PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ rowbase, Chunk ch,
                           uint8_t *__restrict__ status, const uint32_t *__restrict__ hoff,
                           const double *__restrict__ hnodes, int cc) {
    // One warp per row, 32 pixels at a time. The reference's sweep consumes,
    // at each BORDER pixel x, the row's nodes up to its right border
    // start_x + step_x * (x + 1), and sets every other pixel from the parity
    // of the nodes consumed so far. The nodes are sorted, so the nodes
    // consumed before pixel x are those <= the right border of the last
    // BORDER pixel left of x: each pixel finds that pixel by a warp max-scan
    // and counts the nodes by binary search.
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t g = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ch.nrow; g += nw) {
        const uint32_t p = ch.p0 + find_segment(rowbase + ch.p0, ch.np, g + ch.row0);
        const PolyHdr &h = hdr[p];
        const int y = (int)(g + ch.row0 - rowbase[p]);
        if (y < 1 || y >= h.dimy || h.err) continue;
        const double start_x = h.mbr[0];
        const uint32_t i0 = hoff[h.hline + y], j0 = hoff[h.hline + y + 1];
        const double *nodes = hnodes + h.hnode;
        uint8_t *st = status + h.st + (uint64_t)y * h.dimx;
        int carry = -1;  // last BORDER pixel of the earlier batches
        for (int x0 = 0; x0 < h.dimx; x0 += 32) {
            const int x = x0 + lane;
            const bool v = x < h.dimx;
            const uint8_t sx = v ? st[x] : 0;
            const bool border = v && show_status(sx, cc) == 1;
            int last = border ? x : -1;  // inclusive max-scan of BORDER positions
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(full, last, o);
                if (lane >= o && t > last) last = t;
            }
            int before = __shfl_up_sync(full, last, 1);  // last BORDER pixel strictly left of x
            if (lane == 0) before = -1;
            if (before < carry) before = carry;
            if (v && !border) {
                bool isin = false;
                if (before >= 0) {
                    const double rb = start_x + h.step_x * (before + 1);
                    uint32_t lo = i0, hi = j0;  // first node > rb
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (nodes[mid] <= rb) lo = mid + 1;
                        else hi = mid;
                    }
                    isin = ((lo - i0) & 1u) != 0;
                }
                st[x] = isin ? 2 : 0;
            }
            const int tail = __shfl_sync(full, last, 31);
            if (tail > carry) carry = tail;
        }
    }
}

// Per edge: points contributed to every column (count pass or emit pass).
// Both passes run the same arithmetic, so they agree point for point.
__global__ void __launch_bounds__(256, 4) k_clipx(const StoreView sv, const PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ off,
                        Chunk ch, const uint32_t *__restrict__ perm, const double *__restrict__ colx,
                        const LineF *__restrict__ colf, int cert, uint32_t *__restrict__ cnt,
                        const uint64_t *__restrict__ scan, uint64_t *__restrict__ okey, float2 *__restrict__ opt) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ch.ne;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = perm[j];
        uint64_t e = ch.e0 + k;
        uint32_t p = ch.p0 + find_segment(off + ch.p0, ch.np, e);
        const PolyHdr &h = hdr[p];
        if (h.err) {
            if (cnt) cnt[k] = 0;
            continue;
        }
        uint32_t i = (uint32_t)(e - h.edge);
        const float2 *r = sv.ring + h.ring;
        float2 A = r[i], B = r[i + 1];
        const float mnx = A.x < B.x ? A.x : B.x, mxx = A.x < B.x ? B.x : A.x;
        const float mg = fmargin_f(mnx, mxx);
        const float vstart = __fsub_rn(mnx, mg), vend = __fadd_rn(mxx, mg);
        const double *lines = colx + h.col;
        const LineF *lf = colf + h.col;
        int c = first_line_f(lf, h.ncols, vstart);
        uint32_t total = 0;
        uint64_t at = scan ? scan[k] : 0;
        float2 buf[4];
        const ClipXEdge E(A, B);
        LineF L0 = lf[c];
        float2 pi = make_float2(L0.rn, c < h.ncols ? E.ordf(lines[c], L0, cert) : 0.f);
        for (; c < h.ncols && L0.dn <= vend; c++) {
            const LineF L1 = lf[c + 1];  // the line Xi + step_x
            const float2 pi1 = make_float2(L1.rn, E.ordf(lines[c + 1], L1, cert));
            int m = clip_x_points(A, B, L0, L1, pi, pi1, i == 0, okey ? buf : nullptr);
            if (okey) {
                for (int q = 0; q < m; q++) {
                    okey[at] = (h.col - ch.col0) + (uint64_t)c;
                    opt[at] = buf[q];
                    at++;
                }
            }
            total += (uint32_t)m;
            L0 = L1;
            pi = pi1;
        }
        if (cnt) cnt[k] = total;
    }
}

// Stable per-polygon bucketing, in place of global radix sorts whose keys
// are (polygon-local bucket + the polygon's base): the column clip's points
// by column (B_COL), the walk's visits by pixel (B_PIX). Items of polygon q
// of the chunk are [pstart[q], pstart[q + 1]), in the order the reference
// adds them (clip order, crossing order), each tagged with its key; a
// bucket's items must keep that order. The polygon's items are cut into
// tiles of kTile items; one warp per tile counts its items per bucket (lanes
// with equal buckets found by __match_any_sync), the counters laid out per
// polygon as [bucket][tile] are scanned once, and the same warps scatter
// their items to the scanned positions, ranked by lane within each 32-item
// batch. Polygons are contiguous in the chunk and their buckets ascend with
// the polygon, so the positions are the chunk's global sorted ones: the
// result of a stable sort by key. A key outside its polygon's buckets (which
// a correct walk never writes) is clamped there and the polygon is marked
// FARM_EINTERNAL.
constexpr uint32_t kTile = 4096;
enum BucketKind { B_COL = 0, B_PIX = 1 };

template <int kKind>
__device__ __forceinline__ void bucket_geom(const PolyHdr &h, const Chunk &ch, uint64_t &base, uint64_t &nb) {
    if (kKind == B_COL) {
        base = h.col - ch.col0;
        nb = h.ncols > 0 ? (uint64_t)h.ncols : 0;
    } else {
        base = h.pix - ch.pix0;
        nb = h.P;
    }
}

// per polygon of the chunk: the first item of its points (column clip)
__global__ void k_xstarts(const uint64_t *__restrict__ off, Chunk ch, const uint64_t *__restrict__ xscan,
                          uint64_t *__restrict__ pstart) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q <= ch.np; q += gridDim.x * blockDim.x)
        pstart[q] = xscan[off[ch.p0 + q] - ch.e0];
}

template <int kKind>
__global__ void k_btiles(const PolyHdr *__restrict__ hdr, Chunk ch, const uint64_t *__restrict__ pstart,
                         uint64_t *__restrict__ ntile, uint64_t *__restrict__ nslot) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q <= ch.np; q += gridDim.x * blockDim.x) {
        if (q == ch.np) {
            ntile[q] = 0;
            nslot[q] = 0;
            continue;
        }
        const uint64_t n = pstart[q + 1] - pstart[q];
        uint64_t base, nb;
        bucket_geom<kKind>(hdr[ch.p0 + q], ch, base, nb);
        if (n && nb == 0) nb = 1;  // clamped keys (k_bucket)
        const uint64_t t = (n + kTile - 1) / kTile;
        ntile[q] = t;
        nslot[q] = t * nb;
    }
}

template <int kKind, bool kScatter>
__global__ void k_bucket(PolyHdr *__restrict__ hdr, Chunk ch, const uint64_t *__restrict__ pstart,
                         const uint64_t *__restrict__ tileoff, uint64_t ntiles, const uint64_t *__restrict__ slotoff,
                         uint64_t *__restrict__ slot, const uint64_t *__restrict__ key,
                         const uint64_t *__restrict__ val, uint64_t *__restrict__ key_out,
                         uint64_t *__restrict__ val_out) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nw) {
        const uint32_t q = find_segment(tileoff, ch.np, t);
        const uint64_t lt = t - tileoff[q], nt = tileoff[q + 1] - tileoff[q];
        const uint64_t pb = pstart[q], pe = pstart[q + 1];
        const uint64_t i0 = pb + lt * kTile, i1 = min(i0 + kTile, pe);
        uint64_t base, nb;
        bucket_geom<kKind>(hdr[ch.p0 + q], ch, base, nb);
        if (nb == 0) nb = 1;
        uint64_t *S = slot + slotoff[q] + lt;  // bucket b's counter: S[b * nt]
        for (uint64_t ib = i0; ib < i1; ib += 32) {
            const uint64_t i = ib + lane;
            const bool v = i < i1;
            const unsigned act = __ballot_sync(full, v);
            if (v) {
                const uint64_t k = key[i];
                uint64_t b = k - base;
                if (b >= nb) {  // never for a correct walk or clip
                    b = nb - 1;
                    if (kScatter) atomicMin(&hdr[ch.p0 + q].err, FARM_EINTERNAL);
                }
                const unsigned grp = __match_any_sync(act, (uint32_t)b);
                const bool leader = lane == __ffs(grp) - 1;
                if (kScatter) {
                    const uint64_t at = S[b * nt] + (uint64_t)__popc(grp & ((1u << lane) - 1u));
                    key_out[at] = k;
                    val_out[at] = val[i];
                    __syncwarp(act);  // every lane has read its bucket's position
                }
                if (leader) S[b * nt] += (uint64_t)__popc(grp);
            }
            __syncwarp();
        }
    }
}

// Dedup key of clip point k: (column, 16-bit hash of its bits). After a
// stable sort by it, bit-identical points of a column share a run, in clip
// order; hash collisions only lengthen runs.
__global__ void k_ptbits(const float2 *__restrict__ pt, const uint64_t *__restrict__ col, uint64_t n,
                         uint64_t *__restrict__ key, uint32_t *__restrict__ idx) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = pt_bits(pt[k]);
        b ^= b >> 33;
        b *= 0xff51afd7ed558ccdull;
        b ^= b >> 29;
        key[k] = (col[k] << 16) | (b & 0xFFFFull);
        idx[k] = (uint32_t)k;
    }
}

// A point with an earlier bit-identical point in its (column, hash) run is a
// later copy, which MyPolygon.h:49-58 drops (it keeps a point only if no
// earlier kept point equals it). This holds for small points too: a later
// bitwise copy equals the earlier copy, and if that copy was itself dropped,
// the kept point that equalled it equals the later copy as well.
__global__ void k_dup_hash(const uint64_t *__restrict__ key, const uint32_t *__restrict__ pos,
                           const float2 *__restrict__ pt, uint64_t n, uint8_t *__restrict__ drop) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t me = pt_bits(pt[pos[i]]), kk = key[i];
        for (uint64_t j = i; j > 0 && key[j - 1] == kk; j--) {
            if (pt_bits(pt[pos[j - 1]]) == me) {
                drop[pos[i]] = 1;
                break;
            }
        }
    }
}

// Segment starts of sorted keys: starts[c] = first index k with key[k] >= c,
// for c in [0, nseg] (keys < nseg). Thread k fills the segments that begin at k.
__global__ void k_seg_starts(const uint64_t *__restrict__ key, uint64_t n, uint64_t nseg,
                             uint64_t *__restrict__ starts) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= n; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t lo = k == 0 ? 0 : key[k - 1] + 1;
        uint64_t hi = k == n ? nseg : key[k];
        for (uint64_t c = lo; c <= hi; c++) starts[c] = k;
    }
}

// Small points that are the first copy of their bit pattern in their column
// are the only ones whose fate depends on the 1e-9 tolerance of
// Point::operator== (Point.h:32). They are sorted by (column, x, y) and each
// finds the earlier (in clip order) points it equals inside its tolerance
// window; the reference's sequential rule is then resolved on that small
// dependency graph: a point is kept iff none of its earlier equal points is.
__global__ void k_small_flags(const float2 *__restrict__ pt, const uint8_t *__restrict__ drop, uint64_t n,
                              uint64_t *__restrict__ flag) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        flag[k] = (small_pt(pt[k]) && !drop[k]) ? 1 : 0;
}

__global__ void k_small_compact(const uint64_t *__restrict__ sscan, uint64_t n, uint32_t *__restrict__ sidx) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        if (sscan[k + 1] != sscan[k]) sidx[sscan[k]] = (uint32_t)k;
}

// float bits mapped so that unsigned order is numeric order (-0 just before +0)
__device__ inline uint32_t ord_f(float v) {
    uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_small_ykey(const float2 *__restrict__ pt, const uint32_t *__restrict__ sidx, uint64_t ns,
                             uint32_t *__restrict__ ky) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x)
        ky[i] = ord_f(pt[sidx[i]].y);
}

__global__ void k_small_xkey(const float2 *__restrict__ pt, const uint64_t *__restrict__ colkey,
                             const uint32_t *__restrict__ sidx, uint64_t ns, uint64_t *__restrict__ kx) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t k = sidx[i];
        kx[i] = (colkey[k] << 32) | ord_f(pt[k].x);
    }
}

__device__ inline uint64_t lower_key(const uint64_t *kx, uint64_t lo, uint64_t hi, uint64_t key) {
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (kx[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__device__ inline uint64_t upper_key(const uint64_t *kx, uint64_t lo, uint64_t hi, uint64_t key) {
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (kx[mid] <= key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// For sorted small point i: the earlier points (clip order) it equals. Runs
// of one x value are sorted by y; the x values within 1e-9 form a contiguous
// band of runs, and inside each run the y values within 1e-9 form a
// contiguous range (float subtraction is monotone), found by binary search.
template <bool kFill>
__global__ void k_small_deps(const uint64_t *__restrict__ kx, const uint32_t *__restrict__ ps, uint64_t ns,
                             const float2 *__restrict__ pt, uint32_t *__restrict__ cnt,
                             const uint64_t *__restrict__ dscan, uint32_t *__restrict__ deps) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = ps[i];
        const float2 q = pt[k];
        const uint64_t key = kx[i], col = key >> 32;
        uint32_t c = 0;
        uint64_t at = kFill ? dscan[i] : 0;
        auto visit = [&](uint64_t j) {
            uint32_t kj = ps[j];
            if (kj < k && pt_eq(pt[kj], q)) {
                if (kFill) deps[at++] = kj;
                c++;
            }
        };
        // y range [first j with y_j - q.y > -1e-9, first with >= 1e-9) of run [b, e)
        auto run = [&](uint64_t b, uint64_t e) {
            uint64_t lo = b, hi = e;
            while (lo < hi) {
                uint64_t mid = (lo + hi) >> 1;
                if (pt[ps[mid]].y - q.y > -1e-9)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            for (uint64_t j = lo; j < e && pt[ps[j]].y - q.y < 1e-9; j++)
                if (j != i) visit(j);
        };
        const uint64_t rb = lower_key(kx, 0, i, key), re = upper_key(kx, i + 1, ns, key);
        run(rb, re);
        for (uint64_t r = re; r < ns && (kx[r] >> 32) == col && pt[ps[r]].x - q.x < 1e-9;) {
            uint64_t e = upper_key(kx, r + 1, ns, kx[r]);
            run(r, e);
            r = e;
        }
        for (uint64_t r1 = rb; r1 > 0 && (kx[r1 - 1] >> 32) == col && q.x - pt[ps[r1 - 1]].x < 1e-9;) {
            uint64_t b = lower_key(kx, 0, r1 - 1, kx[r1 - 1]);
            run(b, r1);
            r1 = b;
        }
        if (!kFill) cnt[i] = c;
    }
}

// One round of the sequential rule on the dependency graph (a DAG: every
// edge points to an earlier point). Rounds repeat until nothing changes; the
// graph's unique fixed point is the reference's result.
__global__ void k_small_resolve(const uint32_t *__restrict__ ps, uint64_t ns, const uint64_t *__restrict__ dscan,
                                const uint32_t *__restrict__ deps, uint8_t *__restrict__ drop,
                                int *__restrict__ changed) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = dscan[i], e = dscan[i + 1];
        if (b == e) continue;
        bool d = false;
        for (uint64_t j = b; j < e && !d; j++) d = !((volatile uint8_t *)drop)[deps[j]];
        uint32_t k = ps[i];
        if ((uint8_t)d != ((volatile uint8_t *)drop)[k]) {
            ((volatile uint8_t *)drop)[k] = (uint8_t)d;
            *changed = 1;
        }
    }
}

__global__ void k_cp_sizes(const uint64_t *__restrict__ colstart, const uint64_t *__restrict__ keptscan, uint64_t ncol,
                           uint64_t *__restrict__ cpsize) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncol; c += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t nk = keptscan[colstart[c + 1]] - keptscan[colstart[c]];
        cpsize[c] = nk ? nk + 1 : 0;
    }
}

// Column polygons: kept points in order plus the closing copy of the first.
__global__ void k_col_polys(const uint64_t *__restrict__ colkey, const float2 *__restrict__ pt,
                            const uint8_t *__restrict__ drop, const uint64_t *__restrict__ keptscan, uint64_t n,
                            const uint64_t *__restrict__ colstart, const uint64_t *__restrict__ cpstart,
                            float2 *__restrict__ cpoly, uint32_t *__restrict__ cpcol) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        if (drop[k]) continue;
        uint64_t c = colkey[k];
        uint64_t rank = keptscan[k] - keptscan[colstart[c]];
        cpoly[cpstart[c] + rank] = pt[k];
        cpcol[cpstart[c] + rank] = (uint32_t)c;
        if (rank == 0) {
            uint64_t nk = keptscan[colstart[c + 1]] - keptscan[colstart[c]];
            cpoly[cpstart[c] + nk] = pt[k];
            cpcol[cpstart[c] + nk] = (uint32_t)c;
        }
    }
}

// polygon owning each fill column of the chunk
__global__ void k_col_owner(const PolyHdr *__restrict__ hdr, Chunk ch, uint32_t *__restrict__ colpoly) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ch.np; q += gridDim.x * blockDim.x) {
        const PolyHdr &h = hdr[ch.p0 + q];
        const uint64_t c0 = h.col - ch.col0;
        for (int32_t c = 0; c < h.ncols; c++) colpoly[c0 + c] = ch.p0 + q;
    }
}

// cell-clip order: rows an edge of a column polygon spans (FP32 estimate)
__global__ void k_cp_cost(const PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ cpstart,
                          const float2 *__restrict__ cpoly, const uint32_t *__restrict__ cpcol,
                          const uint32_t *__restrict__ colpoly, uint64_t ncp, uint8_t *__restrict__ key,
                          uint32_t *__restrict__ idx) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ncp; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = cpcol[j];
        float cost = 0.f;
        if (j + 1 < cpstart[c + 1]) {
            float2 A = cpoly[j], B = cpoly[j + 1];
            cost = fabsf(B.y - A.y) / (float)hdr[colpoly[c]].step_y;
        }
        key[j] = (uint8_t)(cost < 255.f ? cost : 255.f);
        if (idx) idx[j] = (uint32_t)j;
    }
}

// Per column-polygon edge: points contributed to each row (count or emit).
// Both passes run the same arithmetic, so they agree point for point.
__global__ void __launch_bounds__(256, 4) k_clipy(const PolyHdr *__restrict__ hdr, Chunk ch, const uint32_t *__restrict__ perm,
                        const uint64_t *__restrict__ cpstart, const float2 *__restrict__ cpoly,
                        const uint32_t *__restrict__ cpcol, const uint32_t *__restrict__ colpoly, uint64_t ncp,
                        const double *__restrict__ rowy, const LineF *__restrict__ rowf, int cert,
                        uint32_t *__restrict__ cnt, const uint64_t *__restrict__ scan, uint32_t *__restrict__ okey,
                        float2 *__restrict__ opt) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncp; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t j = perm[t];
        const uint64_t c = cpcol[j];
        uint32_t total = 0;
        if (j + 1 < cpstart[c + 1]) {
            const PolyHdr &h = hdr[colpoly[c]];
            float2 A = cpoly[j], B = cpoly[j + 1];
            const float mny = A.y < B.y ? A.y : B.y, mxy = A.y < B.y ? B.y : A.y;
            const float mg = fmargin_f(mny, mxy);
            const float vstart = __fsub_rn(mny, mg), vend = __fadd_rn(mxy, mg);
            const double *lines = rowy + h.row;
            const LineF *lf = rowf + h.row;
            int r = first_line_f(lf, h.nrows, vstart);
            uint64_t at = scan ? scan[j] : 0;
            float2 buf[4];
            const ClipYEdge E(A, B);
            LineF L0 = lf[r];
            // the point on line Yi, carried from the previous row's Yi1
            // (horizontal edges take per-row abscissae instead)
            float2 pc = make_float2(E.vert ? A.x : (E.general() && r < h.nrows ? E.abscf(lines[r], L0, cert) : 0.f),
                                    L0.rn);
            for (; r < h.nrows && L0.dn <= vend; r++) {
                const LineF L1 = lf[r + 1];  // the line Yi + step_y
                float2 pi, pi1;
                bool par = false;
                if (E.horiz) {
                    // the edge lies on a row line only if A.y equals that double exactly
                    const bool on0 = L0.up == L0.dn && A.y == L0.rn, on1 = L1.up == L1.dn && A.y == L1.rn;
                    pi = make_float2(on0 ? A.x : (on1 ? -INFINITY : 0.f), L0.rn);
                    pi1 = make_float2(on0 ? -INFINITY : (on1 ? A.x : 0.f), L1.rn);
                    par = !on0 && !on1;
                } else {
                    pi = pc;
                    pi1 = make_float2(E.vert ? A.x : E.abscf(lines[r + 1], L1, cert), L1.rn);
                    pc = pi1;
                }
                int k = clip_y_points(A, B, L0, L1, pi, pi1, par, okey ? buf : nullptr);
                if (okey && k) {
                    for (int q = 0; q < k; q++) {  // the row within the column; the column is the edge's
                        okey[at] = (uint32_t)r;
                        opt[at] = buf[q];
                        at++;
                    }
                }
                total += (uint32_t)k;
                L0 = L1;
            }
        }
        if (cnt) cnt[j] = total;
    }
}

// The exact double value of the product of two finite floats, built on the
// integer pipe: a 24 x 24-bit significand product fits a double's 53 bits, so
// (double)a * (double)b is this value with no rounding, and it is assembled
// from the significand product and the exponents instead of two conversions
// and an FP64 multiply (GB300's FP64 pipe issues 2 lanes per clock per SM, its
// integer pipe 64). Subnormal floats (exponent field 0) carry no implicit bit
// and the exponent of 1; the result is always a normal double.
__device__ __forceinline__ double exact_fmul(float a, float b) {
    const uint32_t ua = __float_as_uint(a), ub = __float_as_uint(b);
    uint32_t ea = (ua >> 23) & 0xFFu, eb = (ub >> 23) & 0xFFu;
    if (ea == 0xFFu || eb == 0xFFu) return (double)a * (double)b;  // inf / nan: the FP64 rules
    uint32_t ma = ua & 0x7FFFFFu, mb = ub & 0x7FFFFFu;
    if (ea) ma |= 0x800000u; else ea = 1;
    if (eb) mb |= 0x800000u; else eb = 1;
    const uint64_t sign = (uint64_t)((ua ^ ub) & 0x80000000u) << 32;
    const uint64_t m = (uint64_t)ma * mb;  // value = m * 2^(ea + eb - 300)
    if (m == 0) return __longlong_as_double((long long)sign);
    const int top = 63 - __clzll((long long)m);  // m in [2^top, 2^(top + 1)), top <= 47
    const uint64_t frac = (m << (52 - top)) & 0xFFFFFFFFFFFFFull;
    const uint64_t ex = (uint64_t)(top + (int)ea + (int)eb - 300 + 1023);
    return __longlong_as_double((long long)(sign | (ex << 52) | frac));
}

// The cell clip's points grouped by cell. k_clipy writes each column's
// points contiguously, edge after edge of the column polygon, each tagged
// with its row; a cell's points are the column's points of its row, in that
// order. One warp per column buckets them stably by row, 32 points at a time
// (lanes with equal rows found by __match_any_sync, ranked by lane): a count
// pass, a scan over the column's rows, a scatter pass. This replaces a
// global radix sort of every point by cell: two reads and one write of the
// points instead of three sorting passes over 16-byte keys and values.
// Afterwards cnt[g] holds the end of cell g's points within its column (its
// start is the end of the cell above), and ckey[g] the cell's cost key for
// the area schedule (cells of empty columns keep their preset key).
__global__ void k_cell_bucket(const PolyHdr *__restrict__ hdr, Chunk ch, const uint64_t *__restrict__ cpstart,
                              const uint64_t *__restrict__ yscan, const uint32_t *__restrict__ colpoly, uint64_t ncol,
                              const uint32_t *__restrict__ rowkey, const uint64_t *__restrict__ pin,
                              uint64_t *__restrict__ pout, uint32_t *__restrict__ cnt, uint8_t *__restrict__ ckey) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncol; c += nw) {
        const uint64_t j0 = cpstart[c], j1 = cpstart[c + 1];
        if (j0 == j1) continue;
        const PolyHdr &h = hdr[colpoly[c]];
        const uint64_t ib = yscan[j0], ie = yscan[j1];
        const uint64_t dimx = (uint64_t)h.dimx;
        const int nrows = h.nrows;
        const uint64_t cell0 = (h.pix - ch.pix0) + (c + ch.col0 - h.col);  // the column's cell in row 0
        uint32_t *C = cnt + cell0;
        for (uint64_t base = ib; base < ie; base += 32) {  // points per row
            const uint64_t i = base + lane;
            const bool v = i < ie;
            const unsigned act = __ballot_sync(full, v);
            if (v) {
                const uint32_t r = rowkey[i];
                const unsigned grp = __match_any_sync(act, r);
                if (lane == __ffs(grp) - 1) C[r * dimx] += (uint32_t)__popc(grp);
            }
            __syncwarp();
        }
        uint32_t run = 0;
        for (int r0 = 0; r0 < nrows; r0 += 32) {  // rows -> starts, and the cells' cost keys
            const int r = r0 + lane;
            const uint32_t v = r < nrows ? C[(uint64_t)r * dimx] : 0u;
            uint32_t inc = v;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(full, inc, o);
                if (lane >= o) inc += t;
            }
            if (r < nrows) {
                C[(uint64_t)r * dimx] = run + inc - v;
                const uint32_t k = v < 64u ? v : 64u + (v - 64u) / 16u;
                ckey[cell0 + (uint64_t)r * dimx] = (uint8_t)(255u - (k < 255u ? k : 255u));
            }
            run += __shfl_sync(full, inc, 31);
        }
        __syncwarp();
        for (uint64_t base = ib; base < ie; base += 32) {  // stable scatter
            const uint64_t i = base + lane;
            const bool v = i < ie;
            const unsigned act = __ballot_sync(full, v);
            if (v) {
                const uint32_t r = rowkey[i];
                const unsigned grp = __match_any_sync(act, r);
                const uint32_t at = C[r * dimx] + (uint32_t)__popc(grp & ((1u << lane) - 1u));
                pout[ib + at] = pin[i];
                __syncwarp(act);  // every lane has read its row's start
                if (lane == __ffs(grp) - 1) C[r * dimx] += (uint32_t)__popc(grp);
            }
            __syncwarp();
        }
    }
}

// Work order by an 8-bit cost key, sorted within tiles of kOrderTile items
// (a counting sort in shared memory per block): perm[t0 + j] lists the tile's
// items by ascending key. The order only schedules the work (every output
// position comes from a scan), and what it is for is that the 32 lanes of a
// warp carry similar trip counts, which a sort within the tile gives as well
// as a global one, in one read of the keys and one write of the permutation.
constexpr uint32_t kOrderTile = 4096;
__global__ void __launch_bounds__(256) k_local_order(const uint8_t *__restrict__ key, uint64_t n,
                                                     uint32_t *__restrict__ perm) {
    __shared__ uint32_t cnt[256];
    const int tid = threadIdx.x, lane = tid & 31;
    const uint64_t t0 = (uint64_t)blockIdx.x * kOrderTile;
    if (t0 >= n) return;
    const uint32_t m = (uint32_t)min((uint64_t)kOrderTile, n - t0);
    cnt[tid] = 0;
    __syncthreads();
    uint32_t kk[kOrderTile / 256];
#pragma unroll
    for (int j = 0; j < (int)(kOrderTile / 256); j++) {
        const uint32_t i = (uint32_t)j * 256u + (uint32_t)tid;
        kk[j] = i < m ? key[t0 + i] : 256u;  // 256: no item
        const unsigned peers = __match_any_sync(0xffffffffu, kk[j]);
        if (kk[j] < 256u && lane == __ffs(peers) - 1) atomicAdd(&cnt[kk[j]], (uint32_t)__popc(peers));
    }
    __syncthreads();
    // exclusive scan of the 256 counts by the first warp (8 per lane)
    if (tid < 32) {
        uint32_t v[8], sum = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            v[q] = cnt[tid * 8 + q];
            sum += v[q];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            cnt[tid * 8 + q] = run;
            run += v[q];
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < (int)(kOrderTile / 256); j++) {
        const uint32_t i = (uint32_t)j * 256u + (uint32_t)tid;
        const unsigned peers = __match_any_sync(0xffffffffu, kk[j]);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (kk[j] < 256u && lane == leader) b = atomicAdd(&cnt[kk[j]], (uint32_t)__popc(peers));
        b = __shfl_sync(0xffffffffu, b, leader);
        if (kk[j] < 256u) perm[t0 + b + (uint32_t)__popc(peers & ((1u << lane) - 1u))] = (uint32_t)(t0 + i);
    }
}

__global__ void k_iota_u32(uint32_t *__restrict__ a, uint64_t n) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        a[k] = (uint32_t)k;
}

// Per pixel: cell area (geometry_computation.h:275-297 over the cell's clip,
// closed as Ideal.cpp:805-808 does) and the fill class (Ideal.cpp:880-914).
// Each term is (double)p1.x * p2.y - (double)p2.x * p1.y: the two exact
// products come from exact_fmul, so the FP64 pipe only takes the difference and
// the running sum, in the reference's order.
__global__ void k_cells(PolyHdr *__restrict__ hdr, const uint64_t *__restrict__ pixbase, Chunk ch,
                        const uint32_t *__restrict__ order, const uint32_t *__restrict__ cellend,
                        const uint64_t *__restrict__ yscan, const float2 *__restrict__ cpt,
                        const uint64_t *__restrict__ cpstart, uint8_t *__restrict__ status,
                        double *__restrict__ areas, int cc) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ch.npix;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t g = order ? order[t] : t;
        uint32_t p = ch.p0 + find_segment(pixbase + ch.p0, ch.np, g + ch.pix0);
        const PolyHdr &h = hdr[p];
        if (h.err) continue;
        uint32_t id = (uint32_t)(g + ch.pix0 - h.pix);
        int x = (int)(id % (uint32_t)h.dimx), y = (int)(id / (uint32_t)h.dimx);
        if (x >= h.ncols || y >= h.nrows) continue;
        uint64_t cidx = h.col - ch.col0 + (uint64_t)x;
        if (cpstart[cidx + 1] == cpstart[cidx]) continue;  // empty column: not visited
        const uint64_t colbase = yscan[cpstart[cidx]];  // the column's points (k_cell_bucket)
        const uint64_t b = colbase + (y ? cellend[g - (uint64_t)h.dimx] : 0u), e = colbase + cellend[g];
        uint64_t n = e - b;
        bool close = n > 0 && pt_ne(cpt[b], cpt[e - 1]);
        uint64_t m = n + (close ? 1 : 0);
        double area = 0.0;
        if (m >= 3) {
            float2 p1 = cpt[b];
            for (uint64_t k = 0; k + 1 < m; k++) {
                const float2 p2 = (k + 1 < n) ? cpt[b + k + 1] : cpt[b];
                area += exact_fmul(p1.x, p2.y) - exact_fmul(p2.x, p1.y);
                p1 = p2;
            }
            area = fabs(area) / 2.0;
        }
        double pa = h.step_x * h.step_y;
        int type = classify(area, pa, cc);
        uint8_t *st = status + h.st + id;
        uint8_t raw = *st;
        if (raw == 1) {
            int t2 = type < cc - 2 ? type : cc - 2;
            *st = (uint8_t)(t2 > 1 ? t2 : 1);
            areas[h.pix + id] = area;
        } else if (raw == 2) {
            *st = (uint8_t)(cc - 1);
            areas[h.pix + id] = pa;
        } else {
            *st = 0;
            areas[h.pix + id] = 0.0;
        }
    }
}

// ---------------------------------------------------------- hierarchy --
// Ideal.cpp:1008-1059: each coarse pixel sums the finest areas under it. The
// reference leaves merge_area's status argument uninitialised; compiled, it
// carries over from the previous coarse pixel (x outer, y inner), so once a
// BORDER is seen the rest of the layer is classified as BORDER. Pass 0 finds
// the first such pixel per layer; pass 1 classifies.
__global__ void k_merge(const PolyHdr *__restrict__ hdr, Chunk ch, uint8_t *__restrict__ status,
                        const double *__restrict__ areas, int cc, int pass, uint32_t *__restrict__ firstb) {
    uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = warp; q < ch.np; q += nw) {
        const PolyHdr &h = hdr[ch.p0 + q];
        if (h.err || h.num_layers < 2) continue;
        for (int li = (int)h.num_layers - 2; li >= 0; li--) {
            LayerGeom g;
            layer_geom(h, (uint32_t)li, g);
            uint32_t *fb = firstb + 32ull * q + li;
            uint32_t np = (uint32_t)(g.dimx * g.dimy);
            for (uint32_t k = lane; k < np; k += 32) {
                int x = (int)(k / (uint32_t)g.dimy), y = (int)(k % (uint32_t)g.dimy);  // x outer
                double lowx = g.mbr[0] + x * g.step_x, lowy = g.mbr[1] + y * g.step_y;
                double highx = g.mbr[0] + (x + 1) * g.step_x, highy = g.mbr[1] + (y + 1) * g.step_y;
                int sx = offset_x(h.mbr, h.step_x, h.dimx, lowx);
                int sy = offset_y(h.mbr, h.step_y, h.dimy, lowy);
                int ex = offset_x(h.mbr, h.step_x, h.dimx, highx) - 1;
                int ey = offset_y(h.mbr, h.step_y, h.dimy, highy) - 1;
                if (ey < sy) ey = sy;
                if (ex < sx) ex = sx;
                const uint8_t *fs = status + h.st;
                bool border = false;
                double area = 0.0;
                for (int i = sx; i <= ex; i++)
                    for (int j = sy; j <= ey; j++) {
                        uint32_t id = (uint32_t)(j * h.dimx + i);
                        if (show_status(fs[id], cc) == 1) border = true;
                        if (pass == 1) area += areas[h.pix + id];
                    }
                if (pass == 0) {
                    if (border) atomicMin(fb, k);
                } else {
                    int st = (k >= *fb) ? 1 : show_status(fs[sy * h.dimx + sx], cc);
                    uint8_t full = st == 1 ? (uint8_t)classify(area, g.step_x * g.step_y, cc)
                                           : (st == 2 ? (uint8_t)(cc - 1) : 0);
                    status[h.st + g.offset + (uint32_t)(y * g.dimx + x)] = full;
                }
            }
        }
    }
}

__global__ void k_fill_u32(uint32_t *a, uint64_t n, uint32_t v) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        a[k] = v;
}

__global__ void k_u32_to_u64(const uint32_t *__restrict__ a, uint64_t n, uint64_t *__restrict__ b) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        b[k] = a[k];
}

__global__ void k_not_u8(const uint8_t *__restrict__ a, uint64_t n, uint64_t *__restrict__ b) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        b[k] = a[k] ? 0 : 1;
}

__global__ void k_err_reduce(const PolyHdr *__restrict__ hdr, uint32_t npoly, int *__restrict__ out) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npoly; p += gridDim.x * blockDim.x)
        if (hdr[p].err) atomicMin(out, hdr[p].err);
}

// ------------------------------------------------------------ host ----

template <typename F>
static int cub_call(farm_store *s, F f) {
    size_t bytes = 0;
    FARM_CUDA(f(nullptr, bytes));
    FARM_TRY(s->cub_tmp.ensure(bytes + 16));
    FARM_CUDA(f(s->cub_tmp.p, bytes));
    return FARM_OK;
}

static int excl_scan(farm_store *s, const uint64_t *in, uint64_t *out, uint64_t n) {
    if (n == 0) return FARM_OK;
    return cub_call(s, [&](void *t, size_t &b) {
        return cub::DeviceScan::ExclusiveSum(t, b, in, out, (int64_t)n, s->stream);
    });
}

static int d2h(farm_store *s, void *h, const void *d, size_t bytes) {
    FARM_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s->stream));
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    return FARM_OK;
}

static int key_bits(uint64_t maxkey) {
    int b = 1;
    while (b < 64 && (maxkey >> b)) b++;
    return b;
}

template <typename K, typename V>
static int sort_pairs(farm_store *s, const K *kin, K *kout, const V *vin, V *vout, uint64_t n, int bits) {
    if (n == 0) return FARM_OK;
    return cub_call(s, [&](void *t, size_t &b) {
        return cub::DeviceRadixSort::SortPairs(t, b, kin, kout, vin, vout, (int64_t)n, 0, bits, s->stream);
    });
}

static unsigned gb(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    uint64_t cap = 64ull * sm_count();
    if (g > cap) g = cap;
    return (unsigned)(g ? g : 1);
}

// blocks for a warp-per-item grid-stride kernel of `warps` warps per block
static unsigned warp_blocks(uint64_t items, int warps = 8) {
    uint64_t g = (items + warps - 1) / warps;
    uint64_t cap = (uint64_t)(256 / warps) * 8ull * sm_count();
    if (g > cap) g = cap;
    return (unsigned)(g ? g : 1);
}

// scratch budget per chunk (crossings and edges bound the sizes of every
// intermediate array)
// (FARM_CHUNK_EDGES / FARM_CHUNK_CROSS / FARM_CHUNK_PIX override them, e.g. to
// exercise many small chunks in tests)
static uint64_t env_u64(const char *name, uint64_t dflt) {
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    unsigned long long x = strtoull(v, nullptr, 10);
    return x ? (uint64_t)x : dflt;
}

// Device time of the rasterizer's heavy kernels: an event pair around each
// launch, summed per stage once the call has finished (no synchronisation in
// between).
enum { T_WALK, T_CLIPX, T_CLIPY, T_CELLS, T_N };
struct KTimer {
    std::vector<cudaEvent_t> ev;
    std::vector<int> stage;  // per pair
    cudaEvent_t next() {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ev.push_back(e);
        return e;
    }
    template <typename F>
    void time(int stg, cudaStream_t st, F launch) {
        cudaEvent_t a = next(), b = next();
        if (a) cudaEventRecord(a, st);
        launch();
        if (b) cudaEventRecord(b, st);
        stage.push_back(a && b ? stg : -1);
    }
    void sum(double *ms) {
        for (size_t k = 0; k < stage.size(); k++) {
            float t = 0;
            if (stage[k] >= 0 && cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]) == cudaSuccess) ms[stage[k]] += t;
        }
    }
    ~KTimer() {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};

struct RasterCtx {
    farm_store *s;
    uint32_t np;
    uint64_t n1;
    PolyHdr *hdr;
    const uint64_t *doff;
    const uint64_t *scan;  // per polygon bases (pix, st, off, hline, vline, col, row, scanrow)
    double *colx, *rowy;
    LineF *colf, *rowf;
    WalkF *wf;  // per polygon: the walk's constants as double-floats
    int cert = 1;  // clip points by certified double-float (0: FP64 throughout)
    int cc;
    int launches = 0;
    KTimer timer;
    std::vector<uint64_t> hoff;  // per-polygon first edge (host copy of doff)
    bool counts_kept = false;    // phase 1's per-edge counts are valid for phase 2
};

// perm = items [0, n) ordered by key within tiles (k_local_order)
static int local_order(RasterCtx &R, const uint8_t *key, uint64_t n, uint32_t *perm) {
    if (!n) return FARM_OK;
    const uint64_t tiles = (n + kOrderTile - 1) / kOrderTile;
    k_local_order<<<(unsigned)tiles, 256, 0, R.s->stream>>>(key, n, perm);
    R.launches++;
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

// Edges [e0, e0 + ne) of polygons [p0, p0 + np) in walk order (k_edge_cost).
static int edge_order(RasterCtx &R, uint32_t p0, uint32_t np, uint64_t e0, uint64_t ne, const uint32_t **perm,
                      int x_only = 0) {
    farm_store *s = R.s;
    cudaStream_t st = s->stream;
    FARM_TRY(s->s[S_PERM_K].ensure(2 * ne + 16));
    FARM_TRY(s->s[S_PERM].ensure(8 * ne + 16));
    uint8_t *key = s->s[S_PERM_K].as<uint8_t>(), *key_s = key + ne;
    uint32_t *idx = s->s[S_PERM].as<uint32_t>(), *idx_s = idx + ne;
    k_edge_cost<<<gb(ne), 256, 0, st>>>(s->view(), R.hdr, R.doff, p0, np, e0, ne, x_only, key, nullptr);
    R.launches++;
    (void)key_s;
    (void)idx;
    FARM_TRY(local_order(R, key, ne, idx_s));
    *perm = idx_s;
    return FARM_OK;
}

// Items [pstart[q], pstart[q + 1]) of each polygon q of the chunk, keyed by
// key (its base + a bucket), into key_out / val_out stably by key (k_bucket).
template <int kKind>
static int bucket_sort(RasterCtx &R, const Chunk &ch, const uint64_t *pstart, const uint64_t *key,
                       const uint64_t *val, uint64_t *key_out, uint64_t *val_out, uint64_t n) {
    if (!n) return FARM_OK;
    farm_store *s = R.s;
    cudaStream_t st = s->stream;
    const uint64_t np1 = (uint64_t)ch.np + 1;
    FARM_TRY(s->s[S_XTILE].ensure(8 * 4 * np1 + 64));
    uint64_t *ntile = s->s[S_XTILE].as<uint64_t>(), *nslot = ntile + np1, *tileoff = nslot + np1,
             *slotoff = tileoff + np1;
    k_btiles<kKind><<<gb(np1), 256, 0, st>>>(R.hdr, ch, pstart, ntile, nslot);
    FARM_TRY(excl_scan(s, ntile, tileoff, np1));
    FARM_TRY(excl_scan(s, nslot, slotoff, np1));
    uint64_t ntiles = 0, nslots = 0;
    FARM_TRY(d2h(s, &ntiles, tileoff + ch.np, 8));
    FARM_TRY(d2h(s, &nslots, slotoff + ch.np, 8));
    FARM_TRY(s->s[S_XSLOT].ensure(16 * (nslots + 1) + 64));
    uint64_t *cnt = s->s[S_XSLOT].as<uint64_t>(), *pos = cnt + (nslots + 1);
    FARM_CUDA(cudaMemsetAsync(cnt, 0, 8 * (nslots + 1), st));
    const unsigned tb = warp_blocks(ntiles);
    k_bucket<kKind, false><<<tb, 256, 0, st>>>(R.hdr, ch, pstart, tileoff, ntiles, slotoff, cnt, key, val, nullptr,
                                               nullptr);
    FARM_TRY(excl_scan(s, cnt, pos, nslots + 1));
    k_bucket<kKind, true><<<tb, 256, 0, st>>>(R.hdr, ch, pstart, tileoff, ntiles, slotoff, pos, key, val, key_out,
                                              val_out);
    R.launches += 3;
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

static int raster_chunk(RasterCtx &R, const Chunk &ch) {
    farm_store *s = R.s;
    cudaStream_t st = s->stream;
    int &L = R.launches;
    StoreView sv = s->view();
    sv.category_count = R.cc;
    const uint64_t *pixbase = R.scan + 0 * R.n1, *rowbase = R.scan + 7 * R.n1;
    const uint64_t ne = ch.ne, ne1 = ne + 1;

    // ---- edge walk: count, scan, fill
    FARM_TRY(s->s[S_CNT_E].ensure(3 * ne1 * 4 + 16));
    FARM_TRY(s->s[S_TMP_A].ensure(3 * ne1 * 8 + 16));
    FARM_TRY(s->s[S_SCAN_E].ensure(3 * ne1 * 8 + 16));
    uint32_t *ecnt = s->s[S_CNT_E].as<uint32_t>();
    FARM_CUDA(cudaMemsetAsync(ecnt, 0, 3 * ne1 * 4, st));
    const uint32_t *perm = nullptr;
    FARM_TRY(edge_order(R, ch.p0, ch.np, ch.e0, ne, &perm));
    if (R.counts_kept) {
        k_load_counts<<<gb(ne), 256, 0, st>>>(R.hdr, R.doff, ch, s->s[S_ECNT16].as<uint16_t>(), s->n_edges, ecnt);
    } else {
        R.timer.time(T_WALK, st, [&] { k_walk_count<<<gb(ne), 256, 0, st>>>(sv, R.hdr, R.wf, R.doff, ch, perm, ecnt); });
    }
    uint64_t *ecnt64 = s->s[S_TMP_A].as<uint64_t>(), *escan = s->s[S_SCAN_E].as<uint64_t>();
    k_u32_to_u64<<<gb(3 * ne1), 256, 0, st>>>(ecnt, 3 * ne1, ecnt64);
    L += 2;
    for (int t = 0; t < 3; t++) FARM_TRY(excl_scan(s, ecnt64 + t * ne1, escan + t * ne1, ne1));
    uint64_t nC, nH, nV;
    FARM_TRY(d2h(s, &nC, escan + ne, 8));
    FARM_TRY(d2h(s, &nH, escan + ne1 + ne, 8));
    FARM_TRY(d2h(s, &nV, escan + 2 * ne1 + ne, 8));
    s->rtot.crossings += nC;
    s->rtot.chunks++;
    FARM_TRY(s->s[S_CFROM].ensure(4 * nC + 16));
    FARM_TRY(s->s[S_CTO].ensure(4 * nC + 16));
    FARM_TRY(s->s[S_CEDGE].ensure(4 * nC + 16));
    FARM_TRY(s->s[S_HKEY].ensure(8 * nH + 16));
    FARM_TRY(s->s[S_HVAL].ensure(8 * nH + 16));
    FARM_TRY(s->s[S_VNKEY].ensure(8 * nV + 16));
    FARM_TRY(s->s[S_VNVAL].ensure(8 * nV + 16));
    uint32_t *cfrom = s->s[S_CFROM].as<uint32_t>(), *cto = s->s[S_CTO].as<uint32_t>(),
             *cedge = s->s[S_CEDGE].as<uint32_t>();
    R.timer.time(T_WALK, st, [&] { k_walk_fill<<<gb(ne), 256, 0, st>>>(sv, R.hdr, R.wf, R.doff, ch, perm, escan, cfrom, cto, cedge, s->s[S_HKEY].as<uint64_t>(),
                                        s->s[S_HVAL].as<double>(), s->s[S_VNKEY].as<uint64_t>(),
                                        s->s[S_VNVAL].as<double>()); });
    L++;

    // ---- visits -> edge sequences (process_crosses)
    const uint64_t cn1 = (uint64_t)ch.np + 1;
    FARM_TRY(s->s[S_TMP_B].ensure(cn1 * 8 + 16));
    uint64_t *cbase = s->s[S_TMP_B].as<uint64_t>();
    k_cross_base<<<gb(cn1), 256, 0, st>>>(R.doff, ch, escan, cbase);
    L++;
    FARM_TRY(s->s[S_VKEY].ensure(8 * nC + 16));
    FARM_TRY(s->s[S_VVAL].ensure(8 * nC + 16));
    FARM_TRY(s->s[S_VKEY2].ensure(8 * nC + 16));
    FARM_TRY(s->s[S_VVAL2].ensure(8 * nC + 16));
    uint64_t *vkey = s->s[S_VKEY].as<uint64_t>(), *vval = s->s[S_VVAL].as<uint64_t>();
    uint64_t *vkey2 = s->s[S_VKEY2].as<uint64_t>(), *vval2 = s->s[S_VVAL2].as<uint64_t>();
    if (nC) {
        k_visits<<<gb(nC), 256, 0, st>>>(R.hdr, ch, cbase, nC, cfrom, cto, cedge, vkey, vval);
        L++;
        FARM_TRY(bucket_sort<B_PIX>(R, ch, cbase, vkey, vval, vkey2, vval2, nC));
    }
    FARM_TRY(s->s[S_PIXCNT].ensure(4 * (ch.npix + 1) + 16));
    uint32_t *pixcnt = s->s[S_PIXCNT].as<uint32_t>();
    FARM_CUDA(cudaMemsetAsync(pixcnt, 0, 4 * (ch.npix + 1), st));
    FARM_TRY(s->s[S_SEQW].ensure(2 * 8 * (nC + 1) + 16));
    uint64_t *w = s->s[S_SEQW].as<uint64_t>(), *wscan = w + nC + 1;
    uint2 *seq = s->d_seq.as<uint2>();
    if (nC) {
        k_seq_width<<<gb(nC), 256, 0, st>>>(vkey2, vval2, nC, w, pixcnt);
        FARM_TRY(excl_scan(s, w, wscan, nC + 1));
        k_seq_fill<<<gb(nC), 256, 0, st>>>(R.hdr, ch, cbase, vval2, wscan, nC, seq);
        L += 2;
    }
    k_seq_single<<<gb(ch.np), 256, 0, st>>>(R.hdr, ch, cbase, seq, pixcnt);
    L++;
    {
        FARM_TRY(s->s[S_TMP_A].ensure(8 * (ch.npix + 1) + 16));
        uint64_t *p64 = s->s[S_TMP_A].as<uint64_t>();
        k_u32_to_u64<<<gb(ch.npix + 1), 256, 0, st>>>(pixcnt, ch.npix + 1, p64);
        FARM_TRY(s->s[S_PIXSCAN].ensure(8 * (ch.npix + 1) + 16));
        uint64_t *pscan = s->s[S_PIXSCAN].as<uint64_t>();
        FARM_TRY(excl_scan(s, p64, pscan, ch.npix + 1));
        k_offsets<<<gb(ch.npix), 256, 0, st>>>(R.hdr, pixbase, ch, pscan, s->d_offset.as<uint32_t>());
        L += 2;
    }

    // ---- grid lines (process_intersection)
    for (int vert = 0; vert < 2; vert++) {
        uint64_t nn = vert ? nV : nH;
        uint64_t nl = vert ? ch.nvl : ch.nh;
        const uint64_t *key = vert ? s->s[S_VNKEY].as<uint64_t>() : s->s[S_HKEY].as<uint64_t>();
        const double *val = vert ? s->s[S_VNVAL].as<double>() : s->s[S_HVAL].as<double>();
        double *nodes_out = (vert ? s->d_vnodes.as<double>() : s->d_hnodes.as<double>()) + (vert ? ch.vn0 : ch.hn0);
        FARM_TRY(s->s[S_LINECNT].ensure(2 * 4 * (nl + 1) + 16));
        FARM_TRY(s->s[S_LINESCAN].ensure(2 * 8 * (nl + 1) + 16));
        uint32_t *lcnt = s->s[S_LINECNT].as<uint32_t>(), *lfill = lcnt + (nl + 1);
        uint64_t *lc64 = s->s[S_LINESCAN].as<uint64_t>(), *lstart = lc64 + (nl + 1);
        FARM_CUDA(cudaMemsetAsync(lcnt, 0, 2 * 4 * (nl + 1), st));
        if (nn) {
            k_line_count<<<gb(nn), 256, 0, st>>>(key, nn, lcnt);
            L++;
        }
        k_u32_to_u64<<<gb(nl + 1), 256, 0, st>>>(lcnt, nl + 1, lc64);
        L++;
        FARM_TRY(excl_scan(s, lc64, lstart, nl + 1));
        FARM_TRY(s->s[S_TMP_B].ensure(8 * nn + 16));
        double *unsorted = s->s[S_TMP_B].as<double>();
        if (nn) {
            k_line_scatter<<<gb(nn), 256, 0, st>>>(key, val, nn, lstart, lfill, unsorted);
            L++;
            FARM_TRY(s->s[S_LINEBIG].ensure(16 * (nl + 1) + 64));
            uint64_t *big_b = s->s[S_LINEBIG].as<uint64_t>(), *big_e = big_b + (nl + 1);
            unsigned long long *nbig = reinterpret_cast<unsigned long long *>(big_e + (nl + 1));
            FARM_CUDA(cudaMemsetAsync(nbig, 0, 8, st));
            unsigned lb = (unsigned)std::min<uint64_t>(nl, 8ull * sm_count());
            k_line_sort_warp<<<warp_blocks(nl), 256, 0, st>>>(unsorted, nodes_out, lstart, nl);
            k_line_sort_mid<<<warp_blocks(nl), 256, 0, st>>>(unsorted, nodes_out, lstart, nl);
            k_line_sort<<<lb ? lb : 1, 256, 0, st>>>(unsorted, nodes_out, lstart, nl, big_b, big_e, nbig);
            L += 3;
            unsigned long long hbig = 0;
            FARM_TRY(d2h(s, &hbig, nbig, 8));
            if (hbig) {  // lines beyond the shared-memory sort: the library's segmented sort
                FARM_TRY(cub_call(s, [&](void *t, size_t &b) {
                    return cub::DeviceSegmentedSort::SortKeys(t, b, unsorted, nodes_out, (int64_t)nn, (int64_t)hbig,
                                                              big_b, big_e, st);
                }));
            }
        }
        k_line_offsets<<<gb(ch.np), 256, 0, st>>>(R.hdr, ch, vert, lcnt, lstart,
                                                  vert ? s->d_voff.as<uint32_t>() : s->d_hoff.as<uint32_t>());
        L++;
    }

    // ---- scanline
    k_scanline<<<warp_blocks(ch.nrow), 256, 0, st>>>(R.hdr, rowbase, ch, s->d_status.as<uint8_t>(),
                                                     s->d_hoff.as<uint32_t>(), s->d_hnodes.as<double>(), R.cc);
    L++;

    // ---- fill: strip clip per column
    FARM_TRY(s->s[S_CNT_E].ensure(4 * ne1 + 16));
    uint32_t *xcnt = s->s[S_CNT_E].as<uint32_t>();
    FARM_CUDA(cudaMemsetAsync(xcnt, 0, 4 * ne1, st));
    const uint32_t *xperm = nullptr;
    FARM_TRY(edge_order(R, ch.p0, ch.np, ch.e0, ne, &xperm, 1));
    R.timer.time(T_CLIPX, st, [&] { k_clipx<<<gb(ne), 256, 0, st>>>(sv, R.hdr, R.doff, ch, xperm, R.colx, R.colf, R.cert, xcnt, nullptr, nullptr, nullptr); });
    FARM_TRY(s->s[S_TMP_A].ensure(8 * ne1 + 16));
    uint64_t *x64 = s->s[S_TMP_A].as<uint64_t>();
    k_u32_to_u64<<<gb(ne1), 256, 0, st>>>(xcnt, ne1, x64);
    L += 2;
    FARM_TRY(s->s[S_SCAN_E].ensure(8 * ne1 + 16));
    uint64_t *xscan = s->s[S_SCAN_E].as<uint64_t>();
    FARM_TRY(excl_scan(s, x64, xscan, ne1));
    uint64_t nX;
    FARM_TRY(d2h(s, &nX, xscan + ne, 8));
    s->rtot.clip_x_points += nX;
    FARM_TRY(s->s[S_VKEY].ensure(8 * nX + 16));
    FARM_TRY(s->s[S_VVAL].ensure(8 * nX + 16));
    FARM_TRY(s->s[S_VKEY2].ensure(8 * nX + 16));
    FARM_TRY(s->s[S_VVAL2].ensure(8 * nX + 16));
    uint64_t *xkey = s->s[S_VKEY].as<uint64_t>(), *xkey_s = s->s[S_VKEY2].as<uint64_t>();
    float2 *xpt = s->s[S_VVAL].as<float2>(), *xpt_s = s->s[S_VVAL2].as<float2>();
    if (nX) {
        R.timer.time(T_CLIPX, st, [&] { k_clipx<<<gb(ne), 256, 0, st>>>(sv, R.hdr, R.doff, ch, xperm, R.colx, R.colf, R.cert, nullptr, xscan, xkey, xpt); });
        L++;
        // group the points by column (k_bucket), in clip order within each
        FARM_TRY(s->s[S_XSTART].ensure(8 * ((uint64_t)ch.np + 1) + 64));
        uint64_t *pstart = s->s[S_XSTART].as<uint64_t>();
        k_xstarts<<<gb((uint64_t)ch.np + 1), 256, 0, st>>>(R.doff, ch, xscan, pstart);
        L++;
        FARM_TRY(bucket_sort<B_COL>(R, ch, pstart, xkey, reinterpret_cast<const uint64_t *>(xpt), xkey_s,
                                    reinterpret_cast<uint64_t *>(xpt_s), nX));
    }
    // column starts (the points are grouped by column)
    const uint64_t ncol = ch.ncol;
    FARM_TRY(s->s[S_LINESCAN].ensure(8 * (ncol + 1) + 16));
    uint64_t *colstart = s->s[S_LINESCAN].as<uint64_t>();
    k_seg_starts<<<gb(nX + 1), 256, 0, st>>>(xkey_s, nX, ncol, colstart);
    L++;
    // duplicates: one stable sort by (column, 16-bit hash of the bits), then
    // a backward scan of each run
    FARM_TRY(s->s[S_HKEY].ensure(8 * nX + 16));
    FARM_TRY(s->s[S_HVAL].ensure(8 * nX + 16));
    FARM_TRY(s->s[S_CFROM].ensure(4 * nX + 16));
    FARM_TRY(s->s[S_CTO].ensure(4 * nX + 16));
    FARM_TRY(s->s[S_SEQW].ensure(nX + 32 + 8 * (nX + 1) * 2));
    uint64_t *bits = s->s[S_HKEY].as<uint64_t>(), *bits_s = s->s[S_HVAL].as<uint64_t>();
    uint32_t *pos = s->s[S_CFROM].as<uint32_t>(), *pos_s = s->s[S_CTO].as<uint32_t>();
    uint8_t *drop = s->s[S_SEQW].as<uint8_t>();
    uint64_t *keptscan = reinterpret_cast<uint64_t *>(drop + ((nX + 16 + 7) & ~7ull));
    uint64_t *kept64 = keptscan + (nX + 1);
    FARM_CUDA(cudaMemsetAsync(drop, 0, nX + 1, st));
    if (nX) {
        k_ptbits<<<gb(nX), 256, 0, st>>>(xpt_s, xkey_s, nX, bits, pos);
        L++;
        FARM_TRY(sort_pairs(s, bits, bits_s, pos, pos_s, nX, key_bits(ch.ncol) + 16));
        k_dup_hash<<<gb(nX), 256, 0, st>>>(bits_s, pos_s, xpt_s, nX, drop);
        L++;
    }
    if (nX) {
        // small first copies: tolerance-equality dependencies, then the
        // sequential rule on them
        FARM_TRY(s->s[S_SMALL].ensure(8 * (nX + 1) * 2 + 4 * nX + 32));
        uint64_t *sflag = s->s[S_SMALL].as<uint64_t>(), *sscan = sflag + (nX + 1);
        uint32_t *sidx = reinterpret_cast<uint32_t *>(sscan + (nX + 1));
        FARM_CUDA(cudaMemsetAsync(sflag + nX, 0, 8, st));
        k_small_flags<<<gb(nX), 256, 0, st>>>(xpt_s, drop, nX, sflag);
        L++;
        FARM_TRY(excl_scan(s, sflag, sscan, nX + 1));
        uint64_t ns = 0;
        FARM_TRY(d2h(s, &ns, sscan + nX, 8));
        if (ns > 1) {
            k_small_compact<<<gb(nX), 256, 0, st>>>(sscan, nX, sidx);
            L++;
            // 4 B y keys, y-sorted keys, y-sorted indices, final indices; 8 B x keys, sorted x keys
            const uint64_t ns2 = (ns + 1) & ~1ull;
            FARM_TRY(s->s[S_SMALL_K].ensure(16 * ns2 + 16 * ns + 64));
            unsigned char *kb = s->s[S_SMALL_K].as<unsigned char>();
            uint32_t *ky = reinterpret_cast<uint32_t *>(kb), *ky_s = ky + ns;
            uint32_t *sidx_y = ky_s + ns, *ps = sidx_y + ns;
            uint64_t *kx = reinterpret_cast<uint64_t *>(kb + 16 * ns2), *kx_s = kx + ns;
            k_small_ykey<<<gb(ns), 256, 0, st>>>(xpt_s, sidx, ns, ky);
            L++;
            FARM_TRY(sort_pairs(s, ky, ky_s, sidx, sidx_y, ns, 32));
            k_small_xkey<<<gb(ns), 256, 0, st>>>(xpt_s, xkey_s, sidx_y, ns, kx);
            L++;
            FARM_TRY(sort_pairs(s, kx, kx_s, sidx_y, ps, ns, 32 + key_bits(ncol)));
            // dependency counts -> scan -> lists (counts reuse the flag buffer)
            uint32_t *dcnt = reinterpret_cast<uint32_t *>(sflag);
            k_small_deps<false><<<gb(ns), 256, 0, st>>>(kx_s, ps, ns, xpt_s, dcnt, nullptr, nullptr);
            L++;
            FARM_TRY(s->s[S_SMALL_V].ensure(8 * (ns + 1) * 2 + 16));
            uint64_t *d64 = s->s[S_SMALL_V].as<uint64_t>(), *dscan = d64 + (ns + 1);
            FARM_CUDA(cudaMemsetAsync(dcnt + ns, 0, 4, st));
            k_u32_to_u64<<<gb(ns + 1), 256, 0, st>>>(dcnt, ns + 1, d64);
            L++;
            FARM_TRY(excl_scan(s, d64, dscan, ns + 1));
            uint64_t nd = 0;
            FARM_TRY(d2h(s, &nd, dscan + ns, 8));
            if (nd) {
                FARM_TRY(s->s[S_SMALL_D].ensure(4 * nd + 64));
                uint32_t *deps = s->s[S_SMALL_D].as<uint32_t>();
                int *changed = reinterpret_cast<int *>(deps + ((nd + 3) & ~3ull));
                k_small_deps<true><<<gb(ns), 256, 0, st>>>(kx_s, ps, ns, xpt_s, nullptr, dscan, deps);
                L++;
                for (uint64_t round = 0; round <= ns; round++) {
                    FARM_CUDA(cudaMemsetAsync(changed, 0, 4, st));
                    k_small_resolve<<<gb(ns), 256, 0, st>>>(ps, ns, dscan, deps, drop, changed);
                    L++;
                    int h = 0;
                    FARM_TRY(d2h(s, &h, changed, 4));
                    if (!h) break;
                }
            }
        }
    }
    k_not_u8<<<gb(nX + 1), 256, 0, st>>>(drop, nX + 1, kept64);
    L++;
    FARM_TRY(excl_scan(s, kept64, keptscan, nX + 1));
    FARM_TRY(s->s[S_PIXSCAN].ensure(8 * (ncol + 1) * 2 + 16));
    uint64_t *cpsize = s->s[S_PIXSCAN].as<uint64_t>(), *cpstart = cpsize + (ncol + 1);
    FARM_CUDA(cudaMemsetAsync(cpsize, 0, 8 * (ncol + 1), st));
    k_cp_sizes<<<gb(ncol), 256, 0, st>>>(colstart, keptscan, ncol, cpsize);
    L++;
    FARM_TRY(excl_scan(s, cpsize, cpstart, ncol + 1));
    uint64_t nCP;
    FARM_TRY(d2h(s, &nCP, cpstart + ncol, 8));
    FARM_TRY(s->s[S_CPOLY].ensure(8 * nCP + 16));
    FARM_TRY(s->s[S_CPCOL].ensure(4 * nCP + 16));
    FARM_TRY(s->s[S_COLPOLY].ensure(4 * ncol + 16));
    float2 *cpoly = s->s[S_CPOLY].as<float2>();
    uint32_t *cpcol = s->s[S_CPCOL].as<uint32_t>(), *colpoly = s->s[S_COLPOLY].as<uint32_t>();
    if (nX) {
        k_col_polys<<<gb(nX), 256, 0, st>>>(xkey_s, xpt_s, drop, keptscan, nX, colstart, cpstart, cpoly, cpcol);
        L++;
    }
    k_col_owner<<<gb(ch.np), 256, 0, st>>>(R.hdr, ch, colpoly);
    L++;
    // cell-clip order: edges by the rows they span
    const uint32_t *yperm = nullptr;
    if (nCP) {
        FARM_TRY(s->s[S_PERM_K].ensure(2 * nCP + 16));
        FARM_TRY(s->s[S_PERM].ensure(8 * nCP + 16));
        uint8_t *key = s->s[S_PERM_K].as<uint8_t>(), *key_s = key + nCP;
        uint32_t *idx = s->s[S_PERM].as<uint32_t>(), *idx_s = idx + nCP;
        k_cp_cost<<<gb(nCP), 256, 0, st>>>(R.hdr, cpstart, cpoly, cpcol, colpoly, nCP, key, nullptr);
        L++;
        (void)key_s;
        (void)idx;
        FARM_TRY(local_order(R, key, nCP, idx_s));
        yperm = idx_s;
    }

    // ---- fill: cell clip per row
    FARM_TRY(s->s[S_CNT_E].ensure(4 * (nCP + 1) + 16));
    uint32_t *ycnt = s->s[S_CNT_E].as<uint32_t>();
    FARM_CUDA(cudaMemsetAsync(ycnt, 0, 4 * (nCP + 1), st));
    if (nCP) {
        R.timer.time(T_CLIPY, st, [&] { k_clipy<<<gb(nCP), 256, 0, st>>>(R.hdr, ch, yperm, cpstart, cpoly, cpcol, colpoly, nCP, R.rowy, R.rowf, R.cert, ycnt,
                                         nullptr, nullptr, nullptr); });
        L++;
    }
    FARM_TRY(s->s[S_TMP_A].ensure(8 * (nCP + 1) + 16));
    uint64_t *y64 = s->s[S_TMP_A].as<uint64_t>();
    k_u32_to_u64<<<gb(nCP + 1), 256, 0, st>>>(ycnt, nCP + 1, y64);
    L++;
    FARM_TRY(s->s[S_SCAN_E].ensure(8 * (nCP + 1) + 16));
    uint64_t *yscan = s->s[S_SCAN_E].as<uint64_t>();
    FARM_TRY(excl_scan(s, y64, yscan, nCP + 1));
    uint64_t nY;
    FARM_TRY(d2h(s, &nY, yscan + nCP, 8));
    s->rtot.clip_y_points += nY;
    FARM_TRY(s->s[S_VKEY].ensure(8 * nY + 16));
    FARM_TRY(s->s[S_VVAL].ensure(8 * nY + 16));
    FARM_TRY(s->s[S_HKEY].ensure(8 * nY + 16));
    FARM_TRY(s->s[S_HVAL].ensure(8 * nY + 16));
    uint32_t *ykb = s->s[S_VKEY].as<uint32_t>();
    float2 *ypb = s->s[S_VVAL].as<float2>(), *yps = s->s[S_HVAL].as<float2>();
    // per cell: the end of its points within its column, and its cost key
    // (the cell order's buffers are free again after the cell-clip order)
    FARM_TRY(s->s[S_TMP_A].ensure(4 * (ch.npix + 1) + 16));
    uint32_t *cellend = s->s[S_TMP_A].as<uint32_t>();
    FARM_CUDA(cudaMemsetAsync(cellend, 0, 4 * (ch.npix + 1), st));
    if (nY) {
        R.timer.time(T_CLIPY, st, [&] { k_clipy<<<gb(nCP), 256, 0, st>>>(R.hdr, ch, yperm, cpstart, cpoly, cpcol, colpoly, nCP, R.rowy, R.rowf,
                                         R.cert, nullptr, yscan, ykb, ypb); });
        L++;
    }
    // (yperm lives in S_PERM: the emit pass above is done with it before these
    // buffers are regrown or rewritten, stream-ordered)
    FARM_TRY(s->s[S_PERM_K].ensure(2 * ch.npix + 16));
    FARM_TRY(s->s[S_PERM].ensure(8 * ch.npix + 16));
    uint8_t *ckey = s->s[S_PERM_K].as<uint8_t>(), *ckey_s = ckey + ch.npix;
    uint32_t *cidx = s->s[S_PERM].as<uint32_t>(), *cidx_s = cidx + ch.npix;
    FARM_CUDA(cudaMemsetAsync(ckey, 0xFF, ch.npix, st));
    if (nY) {
        unsigned cb = (unsigned)std::min<uint64_t>((ncol + 7) / 8, 64ull * sm_count());
        k_cell_bucket<<<cb ? cb : 1, 256, 0, st>>>(R.hdr, ch, cpstart, yscan, colpoly, ncol, ykb,
                                                  reinterpret_cast<const uint64_t *>(ypb),
                                                  reinterpret_cast<uint64_t *>(yps), cellend, ckey);
        L++;
    }
    // cells heaviest first
    uint32_t *corder = nullptr;
    if (ch.npix) {
        k_iota_u32<<<gb(ch.npix), 256, 0, st>>>(cidx, ch.npix);
        L++;
        FARM_TRY(sort_pairs(s, ckey, ckey_s, cidx, cidx_s, ch.npix, 8));
        corder = cidx_s;
    }
    R.timer.time(T_CELLS, st, [&] { k_cells<<<gb(ch.npix), 256, 0, st>>>(R.hdr, pixbase, ch, corder, cellend, yscan, yps,
                                         cpstart, s->d_status.as<uint8_t>(), s->d_areas.as<double>(), R.cc); });
    L++;

    // ---- hierarchy
    if (s->ropts.hierarchy) {
        FARM_TRY(s->s[S_TMP_B].ensure(4ull * 32 * ch.np + 16));
        uint32_t *fb = s->s[S_TMP_B].as<uint32_t>();
        k_fill_u32<<<gb(32ull * ch.np), 256, 0, st>>>(fb, 32ull * ch.np, 0xFFFFFFFFu);
        k_merge<<<gb(32ull * ch.np), 256, 0, st>>>(R.hdr, ch, s->d_status.as<uint8_t>(), s->d_areas.as<double>(), R.cc,
                                                  0, fb);
        k_merge<<<gb(32ull * ch.np), 256, 0, st>>>(R.hdr, ch, s->d_status.as<uint8_t>(), s->d_areas.as<double>(), R.cc,
                                                  1, fb);
        L += 3;
    }
    FARM_CUDA(cudaGetLastError());
    return FARM_OK;
}

int rasterize(farm_store *s, const farm_raster_opts *o, int *launches) {
    uint32_t np = (uint32_t)s->n_poly;
    uint64_t ne = s->n_edges;
    if (np == 0) {
        set_error("no polygons loaded");
        return FARM_EINVAL;
    }
    RasterParams rp;
    memset(&rp, 0, sizeof rp);
    rp.vpr = o->vpr;
    rp.cc = o->category_count;
    rp.hier = o->hierarchy;
    {
        // UniversalGrid::configure(25) (UniversalGrid.h:29-35) with util.h:53-66
        double num = (o->grid_extent > 0 ? o->grid_extent : 360.0) / pow(2, 25);
        double d = ceil(log10(num < 0 ? -num : num));
        int power = 2 - (int)d;
        double magnitude = pow(10.0, power);
        rp.gstep = round(num * magnitude) / magnitude;
        for (int k = 0; k < 40; k++) rp.pow2_ceil[k] = (int)ceil(log((double)(1ull << k)) / log(2.0));
    }
    cudaStream_t st = s->stream;
    RasterCtx R;
    cudaEvent_t t_begin = R.timer.next(), t_end = R.timer.next();
    R.timer.stage.push_back(-1);  // the pair (t_begin, t_end) is read separately
    if (t_begin) cudaEventRecord(t_begin, st);
    R.s = s;
    R.np = np;
    R.n1 = (uint64_t)np + 1;
    R.cc = o->category_count;
    R.doff = s->d_off.as<uint64_t>();
    R.hoff.resize((size_t)np + 1);
    FARM_CUDA(cudaMemcpyAsync(R.hoff.data(), R.doff, 8 * ((size_t)np + 1), cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    const uint64_t n1 = R.n1;
    FARM_TRY(s->d_hdr.ensure(sizeof(PolyHdr) * np));
    FARM_TRY(s->s[S_SIZES].ensure(9 * n1 * 8));
    FARM_TRY(s->s[S_SCAN].ensure(9 * n1 * 8));
    FARM_CUDA(cudaMemsetAsync(s->s[S_SIZES].p, 0, 9 * n1 * 8, st));
    R.hdr = s->d_hdr.as<PolyHdr>();
    uint64_t *sizes = s->s[S_SIZES].as<uint64_t>(), *scan = s->s[S_SCAN].as<uint64_t>();
    R.scan = scan;
    k_header<<<gb(32ull * np), 256, 0, st>>>(s->d_ring.as<float2>(), R.doff, np, rp, R.hdr, sizes);
    R.launches++;
    for (int t = 0; t < 8; t++) FARM_TRY(excl_scan(s, sizes + t * n1, scan + t * n1, n1));
    uint64_t tot[8];
    for (int t = 0; t < 8; t++) FARM_CUDA(cudaMemcpyAsync(&tot[t], scan + t * n1 + np, 8, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    const uint64_t totP = tot[0], totStatus = tot[1], totOff = tot[2], totH = tot[3], totV = tot[4], totCol = tot[5],
                   totRow = tot[6];
    FARM_TRY(s->d_status.ensure(totStatus + 16));
    FARM_TRY(s->d_offset.ensure(4 * totOff + 16));
    FARM_TRY(s->d_areas.ensure(8 * totP + 16));
    FARM_TRY(s->d_hoff.ensure(4 * totH + 16));
    FARM_TRY(s->d_voff.ensure(4 * totV + 16));
    FARM_TRY(s->s[S_COLX].ensure(8 * totCol + 16));
    FARM_TRY(s->s[S_ROWY].ensure(8 * totRow + 16));
    FARM_TRY(s->s[S_COLXF].ensure(16 * totCol + 16));
    FARM_TRY(s->s[S_ROWYF].ensure(16 * totRow + 16));
    FARM_CUDA(cudaMemsetAsync(s->d_status.p, 0, totStatus + 16, st));
    FARM_CUDA(cudaMemsetAsync(s->d_areas.p, 0, 8 * totP + 16, st));
    FARM_CUDA(cudaMemsetAsync(s->d_offset.p, 0, 4 * totOff + 16, st));
    FARM_CUDA(cudaMemsetAsync(s->d_hoff.p, 0, 4 * totH + 16, st));
    FARM_CUDA(cudaMemsetAsync(s->d_voff.p, 0, 4 * totV + 16, st));
    R.colx = s->s[S_COLX].as<double>();
    R.rowy = s->s[S_ROWY].as<double>();
    R.colf = s->s[S_COLXF].as<LineF>();
    R.rowf = s->s[S_ROWYF].as<LineF>();
    {
        const char *ex = getenv("FARM_RASTER_EXACT");
        R.cert = (ex && *ex && *ex != '0') ? 0 : 1;
    }
    k_bases<<<gb(np), 256, 0, st>>>(R.hdr, np, scan, R.colx, R.rowy, R.colf, R.rowf);
    FARM_TRY(s->s[S_WALKF].ensure(sizeof(WalkF) * (uint64_t)np + 16));
    R.wf = s->s[S_WALKF].as<WalkF>();
    k_walkf<<<gb(np), 256, 0, st>>>(R.hdr, np, R.wf);
    R.launches++;
    R.launches++;

    memset(&s->rtot, 0, sizeof s->rtot);
    s->rtot.polygons = np;
    s->rtot.vertices = ne;
    s->rtot.pixels = totP;
    s->rtot.status_bytes = totStatus;

    // ---- phase 1: per-polygon totals size the sequence and node arrays
    {
        StoreView sv = s->view();
        FARM_TRY(s->s[S_TMP_B].ensure(3 * 8 * n1 + 16));
        unsigned long long *tot3 = s->s[S_TMP_B].as<unsigned long long>();
        FARM_CUDA(cudaMemsetAsync(tot3, 0, 3 * 8 * n1, st));
        FARM_TRY(s->s[S_ECNT16].ensure(3 * 2 * ne + 64));
        uint16_t *c16 = s->s[S_ECNT16].as<uint16_t>();
        FARM_TRY(s->d_counters.ensure(256));
        int *ovf = reinterpret_cast<int *>(s->d_counters.as<unsigned long long>() + 30);
        FARM_CUDA(cudaMemsetAsync(ovf, 0, 4, st));
        for (uint64_t e0 = 0; e0 < ne; e0 += 1ull << 27) {
            const uint64_t n = ne - e0 < (1ull << 27) ? ne - e0 : 1ull << 27;
            // polygons whose edges meet [e0, e0 + n)
            uint32_t pa = 0, pb = np;
            {
                const std::vector<uint64_t> &ho = R.hoff;
                pa = (uint32_t)(std::upper_bound(ho.begin(), ho.end(), e0) - ho.begin() - 1);
                pb = (uint32_t)(std::lower_bound(ho.begin(), ho.end(), e0 + n) - ho.begin());
                if (pb > np) pb = np;
            }
            const uint32_t *perm = nullptr;
            FARM_TRY(edge_order(R, pa, pb - pa, e0, n, &perm));
            R.timer.time(T_WALK, st,
                         [&] { k_walk_tot<<<gb(n), 256, 0, st>>>(sv, R.hdr, R.wf, R.doff, np, e0, n, perm, tot3,
                                                                   c16, ne, ovf); });
            R.launches++;
        }
        int h_ovf = 1;
        FARM_TRY(d2h(s, &h_ovf, ovf, 4));
        R.counts_kept = h_ovf == 0;
        FARM_TRY(s->s[S_TMP_A].ensure(2 * 3 * 8 * n1 + 16));
        uint64_t *sz = s->s[S_TMP_A].as<uint64_t>(), *sc = sz + 3 * n1;
        k_tot_sizes<<<gb(n1), 256, 0, st>>>(tot3, R.hdr, np, sz);
        R.launches++;
        for (int t = 0; t < 3; t++) FARM_TRY(excl_scan(s, sz + t * n1, sc + t * n1, n1));
        k_set_node_bases<<<gb(np), 256, 0, st>>>(R.hdr, np, sz, sc);
        R.launches++;
        uint64_t tseq, th, tv;
        FARM_TRY(d2h(s, &tseq, sc + np, 8));
        FARM_TRY(d2h(s, &th, sc + n1 + np, 8));
        FARM_TRY(d2h(s, &tv, sc + 2 * n1 + np, 8));
        FARM_TRY(s->d_seq.ensure(8 * tseq + 16));
        FARM_TRY(s->d_hnodes.ensure(8 * th + 16));
        FARM_TRY(s->d_vnodes.ensure(8 * tv + 16));
        s->tot_seq = tseq;
        s->rtot.sequences = tseq;
        s->rtot.hnodes = th;
        s->rtot.vnodes = tv;
    }

    // ---- phase 2: chunks
    std::vector<uint64_t> hscan(8 * n1);
    std::vector<PolyHdr> hh(np);
    FARM_CUDA(cudaMemcpyAsync(hscan.data(), scan, 8 * 8 * n1, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaMemcpyAsync(hh.data(), R.hdr, sizeof(PolyHdr) * np, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    const std::vector<uint64_t> &hoff = R.hoff;
    const uint64_t kChunkEdges = env_u64("FARM_CHUNK_EDGES", 1ull << 27);
    const uint64_t kChunkCross = env_u64("FARM_CHUNK_CROSS", 1ull << 27);
    const uint64_t kChunkPix = env_u64("FARM_CHUNK_PIX", 1ull << 27);
    uint32_t p = 0;
    while (p < np) {
        uint32_t q = p;
        uint64_t ce = 0, cc = 0, cp = 0;
        do {
            ce += hoff[q + 1] - hoff[q];
            cc += hh[q].n_seq;
            cp += hh[q].P;
            q++;
        } while (q < np && ce + (hoff[q + 1] - hoff[q]) <= kChunkEdges && cc + hh[q].n_seq <= kChunkCross &&
                 cp + hh[q].P <= kChunkPix);
        Chunk ch;
        ch.p0 = p;
        ch.np = q - p;
        ch.e0 = hoff[p];
        ch.ne = hoff[q] - hoff[p];
        ch.pix0 = hscan[0 * n1 + p];
        ch.npix = hscan[0 * n1 + q] - ch.pix0;
        ch.h0 = hscan[3 * n1 + p];
        ch.nh = hscan[3 * n1 + q] - ch.h0;
        ch.v0 = hscan[4 * n1 + p];
        ch.nvl = hscan[4 * n1 + q] - ch.v0;
        ch.col0 = hscan[5 * n1 + p];
        ch.ncol = hscan[5 * n1 + q] - ch.col0;
        ch.row0 = hscan[7 * n1 + p];
        ch.nrow = hscan[7 * n1 + q] - ch.row0;
        ch.hn0 = hh[p].hnode;
        ch.vn0 = hh[p].vnode;
        FARM_TRY(raster_chunk(R, ch));
        p = q;
    }
    (void)totRow;

    if (t_end) cudaEventRecord(t_end, st);

    // errors
    FARM_TRY(s->d_counters.ensure(64));
    int *derr = s->d_counters.as<int>();
    FARM_CUDA(cudaMemsetAsync(derr, 0, 4, st));
    k_err_reduce<<<gb(np), 256, 0, st>>>(R.hdr, np, derr);
    R.launches++;
    int herr = 0;
    FARM_CUDA(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st));
    FARM_CUDA(cudaStreamSynchronize(st));
    s->tot_P = totP;
    s->tot_status = totStatus;
    {
        double ms[T_N] = {0, 0, 0, 0};
        R.timer.sum(ms);
        s->rtot.ms_walk = ms[T_WALK];
        s->rtot.ms_clip_x = ms[T_CLIPX];
        s->rtot.ms_clip_y = ms[T_CLIPY];
        s->rtot.ms_cells = ms[T_CELLS];
        float t = 0;
        if (t_begin && t_end && cudaEventElapsedTime(&t, t_begin, t_end) == cudaSuccess) s->rtot.ms_total = t;
    }
    if (launches) *launches = R.launches;
    if (herr) {
        set_error(herr == FARM_EASSERT
                      ? "a polygon violated a condition the reference asserts on (see farm_raster_fetch err)"
                      : "internal inconsistency between the rasterizer's passes");
        return herr;
    }
    return FARM_OK;
}

}  // namespace farm

extern "C" int farm_raster_get_totals(farm_store *s, farm_raster_totals *out) {
    using namespace farm;
    if (!s || !out) {
        set_error("invalid arguments to farm_raster_get_totals");
        return FARM_EINVAL;
    }
    *out = s->rtot;
    return FARM_OK;
}

extern "C" int farm_rasterize(farm_store *s, const farm_raster_opts *o) {
    using namespace farm;
    if (!s || !o || o->vpr <= 0) {
        set_error("invalid arguments to farm_rasterize");
        return FARM_EINVAL;
    }
    if (!(o->category_count == 4 || o->category_count == 16 || o->category_count == 256)) {
        set_error("category_count must be 4, 16 or 256");
        return FARM_EINVAL;
    }
    s->rasterized = false;
    s->ropts = *o;
    int launches = 0;
    int rc = rasterize(s, o, &launches);
    s->launches += (uint64_t)launches;
    // with FARM_EASSERT the other polygons' rasters stay valid and inspectable;
    // queries refuse to run on such a store
    s->raster_epoch++;
    if (rc == FARM_OK || rc == FARM_EASSERT) s->rasterized = true;
    s->raster_err = rc == FARM_EASSERT ? rc : 0;
    return rc;
}
