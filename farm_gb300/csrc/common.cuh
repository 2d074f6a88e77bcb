// Shared device-side definitions of the GB300 polygon-join engine.
//
// Numerics: every translation unit is compiled with -fmad=false. The
// reference's CPU build (x86-64, no -march) never fuses a multiply with an
// add, and the pair sets must be bit-identical to it, so no kernel may either.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "farm_gpu.h"

namespace farm {

// ---------------------------------------------------------------- errors --
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define FARM_CUDA(call)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

#define FARM_TRY(expr)          \
    do {                        \
        int rc_ = (expr);       \
        if (rc_ != FARM_OK) return rc_; \
    } while (0)

// ------------------------------------------------------------ buffers --
// Grow-only device buffer; contents are not preserved across growth.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

// ---------------------------------------------------------- raster data --
// Per polygon header, written by the rasterizer. Bases index the store's
// flattened per-pixel / per-sequence / per-node arrays.
struct PolyHdr {
    double mbr[4];  // lowx lowy highx highy (grid-aligned with the hierarchy)
    double step_x, step_y;
    int32_t dimx, dimy;
    uint32_t nv;           // in-memory ring length (stored vertices + 1)
    uint32_t P;            // dimx * dimy
    uint32_t status_size;  // P + coarser layers
    uint32_t num_layers;
    uint32_t n_seq, n_hnodes, n_vnodes;
    int32_t ncols, nrows;  // columns / rows the fill sweep visits
    int32_t err;
    uint64_t ring;         // first vertex in the padded ring array
    uint64_t edge;         // first edge (global edge id)
    uint64_t pix;          // base of status-free per-pixel arrays (areas, seq counts)
    uint64_t st;           // base into status (status_size bytes)
    uint64_t off;          // base into offset (P + 1 entries)
    uint64_t seq;          // base into seq (n_seq entries of 2 x u32)
    uint64_t hline, vline; // bases into hoff (dimy + 2) / voff (dimx + 2)
    uint64_t hnode, vnode; // bases into hnodes / vnodes
    uint64_t col, row;     // bases into the fill sweep's column / row lines
    uint64_t cross;        // first crossing record
};

struct LayerGeom {
    double mbr[4];
    double step_x, step_y;
    int32_t dimx, dimy;
    uint32_t offset;  // into the polygon's status block
};

// Device-side view of a store (passed by value to kernels).
struct StoreView {
    const float2 *ring;     // padded rings: stored vertices, closing copy, pad copy
    const PolyHdr *hdr;
    uint8_t *status;
    const uint32_t *offset;
    const uint2 *seq;       // (start edge, length)
    const uint32_t *hoff;
    const double *hnodes;
    const uint32_t *voff;
    const double *vnodes;
    const double *areas;
    int32_t category_count;
};

// ------------------------------------------------------- shared math ----
// util.h:98-106
__host__ __device__ inline int double_to_int(double val) {
    int vi = (int)val;
    if (fabs(1.0 * (vi + 1) - val) < 0.00000001) vi++;
    return vi;
}

// MyRaster.cpp:188-200
__host__ __device__ inline int offset_x(const double *mbr, double step, int dim, double v) {
    int x = double_to_int((v - mbr[0]) / step);
    x = x < 0 ? 0 : x;
    return x > dim - 1 ? dim - 1 : x;
}
__host__ __device__ inline int offset_y(const double *mbr, double step, int dim, double v) {
    int y = double_to_int((v - mbr[1]) / step);
    y = y < 0 ? 0 : y;
    return y > dim - 1 ? dim - 1 : y;
}

// MyRaster.cpp:228-239: 0 OUT, 1 BORDER, 2 IN
__host__ __device__ inline int show_status(uint8_t s, int cc) {
    return s == 0 ? 0 : (s == cc - 1 ? 2 : 1);
}

// geometry_computation.h:299-321
__host__ __device__ inline int classify(double area, double pixelArea, int count) {
    double ratio = area / pixelArea;
    if (fabs(ratio - 1.0) < 1e-9) return count - 1;
    if (fabs(ratio) < 1e-9) return 0;
    int idx = (int)ceil(ratio * (count - 2));
    if (idx >= count) idx = count - 1;
    return idx;
}

// Point.h:402-403 (float subtraction, compared with a double constant)
__host__ __device__ inline bool pt_eq(float2 a, float2 b) {
    return fabsf(a.x - b.x) < 1e-9 && fabsf(a.y - b.y) < 1e-9;
}
__host__ __device__ inline bool pt_ne(float2 a, float2 b) {
    return fabsf(a.x - b.x) >= 1e-9 || fabsf(a.y - b.y) >= 1e-9;
}

// Geometry of hierarchy layer li of a polygon (Ideal.cpp:1061-1099,
// Hraster.cpp:3-25): layers are recomputed from the finest raster on demand.
__host__ __device__ inline void layer_geom(const PolyHdr &h, uint32_t li, LayerGeom &g) {
    uint32_t L = h.num_layers;
    for (int k = 0; k < 4; k++) g.mbr[k] = h.mbr[k];
    g.step_x = h.step_x;
    g.step_y = h.step_y;
    g.dimx = h.dimx;
    g.dimy = h.dimy;
    g.offset = 0;
    uint32_t status_size = h.P;
    for (int i = (int)L - 2; i >= (int)li; i--) {
        double sx = g.step_x * 2, sy = g.step_y * 2;
        g.step_x = sx;
        g.step_y = sy;
        g.mbr[0] = floor(h.mbr[0] / sx) * sx;
        g.mbr[1] = floor(h.mbr[1] / sy) * sy;
        g.mbr[2] = ceil(h.mbr[2] / sx) * sx;
        g.mbr[3] = ceil(h.mbr[3] / sy) * sy;
        g.dimx = (int)round((g.mbr[2] - g.mbr[0]) / sx);
        g.dimy = (int)round((g.mbr[3] - g.mbr[1]) / sy);
        g.offset = status_size;
        status_size += (uint32_t)(g.dimx * g.dimy);
    }
}

// upper_bound over a sorted u64 array: index of the segment containing x
__device__ inline uint32_t find_segment(const uint64_t *starts, uint32_t n, uint64_t x) {
    uint32_t lo = 0, hi = n;  // starts[0] <= x
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (starts[mid] <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

inline unsigned grid_for(uint64_t n, unsigned block) {
    uint64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7FFFFFFFull) g = 0x7FFFFFFFull;
    return (unsigned)g;
}

int sm_count();

}  // namespace farm

struct farm_store;
namespace farm {
// FARM_EINVAL unless every pair's source index is below the source count and
// its target index below the target count (the source count when self).
// Device pairs are checked by a kernel (one synchronisation).
int check_pairs(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, bool self, const char *who);
// Book a loaded side's offsets (h from 0, n + 1 entries) and room for its
// padded rings; *ring_first: the float2 index of the side's first ring.
int stage_side(farm_store *s, int side, std::vector<uint64_t> h, uint64_t *ring_first);
// The same with explicit bounds: first index below n_first, second below
// n_second; the names label the two counts in the message.
int check_pair_limits(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint64_t n_first,
                      uint64_t n_second, const char *who, const char *first_name, const char *second_name);
}  // namespace farm

// The store object behind the C ABI.
namespace farm {
// Scratch slots of farm_store::s. The rasterizer's pipeline uses slots 0-34
// and 40-47 (raster.cu) only while farm_rasterize runs; the queries reuse Q_SCR0-5
// within one call; Q_WITHIN_SUF and Q_AREA_ORIENT are theirs alone (the
// area orientations stay valid across calls and a captured area plan holds
// their address).
enum ScratchSlot : int {
    Q_SCR0 = 26,
    Q_SCR1 = 27,
    Q_SCR2 = 28,
    Q_SCR3 = 29,
    Q_SCR4 = 30,
    Q_SCR5 = 31,
    Q_WITHIN_SUF = 35,
    Q_AREA_ORIENT = 36,
    Q_AREA_EPOFF = 37,  // area: edge -> pixel index offsets (per ring position)
    Q_AREA_EPPIX = 38,  // area: edge -> pixel index entries
    Q_PAIR_ORDER = 39,  // intersect: the longest-first pair order
};
}  // namespace farm

struct farm_store {
    cudaStream_t stream = nullptr;
    int device = 0;
    // input rings per side (host layout offsets on device, padded rings)
    uint64_t n_side[2] = {0, 0};
    std::vector<uint64_t> h_off[2];  // host copies of the offsets
    std::vector<uint64_t> h_cat;     // both sides' offsets, concatenated (the source of d_off)
    farm::DevBuf d_xy_in;            // staging for host rings
    farm::DevBuf d_off;              // offsets of both sides, concatenated (n0+n1+1)
    farm::DevBuf d_ring;             // padded rings of both sides
    uint64_t n_poly = 0;             // n_side[0] + n_side[1]
    uint64_t n_edges = 0;            // total stored vertices == edges
    // raster
    bool rasterized = false;
    int raster_err = 0;  // FARM_EASSERT when some polygon hit a reference assert
    farm_raster_opts ropts{};
    farm::DevBuf d_hdr, d_status, d_offset, d_seq, d_hoff, d_hnodes, d_voff, d_vnodes, d_areas;
    uint64_t tot_P = 0, tot_status = 0, tot_seq = 0;
    farm_raster_totals rtot = {};
    // scratch for the rasterizer and the queries
    farm::DevBuf s[48];
    farm::DevBuf cub_tmp;
    farm::DevBuf d_pairs, d_out, d_counters;
    farm::DevBuf d_check;  // pair-index validation counter
    farm::DevBuf d_points; // staged query points (farm_contain_points)
    void *h_stage[2] = {nullptr, nullptr};  // pinned staging of the .dt loader (farm_store_load_dt)
    size_t h_stage_cap = 0;
    cudaEvent_t ev_stage[2] = {};
    cudaEvent_t ev[8] = {};
    uint64_t launches = 0;  // engine kernels launched through this store
    void *mlp = nullptr;    // learned scorer state (mlp.cu)
    uint64_t raster_epoch = 0;     // bumped by every rasterization (plans check it)
    uint64_t orient_epoch = ~0ull;  // raster_epoch the cached orientations belong to
    uint64_t edgepix_epoch = ~0ull; // raster_epoch the area's edge -> pixel index belongs to
    int32_t area_chunk[32] = {};   // edges per area item by size bucket (0: the default 16)
    int32_t area_wide[32] = {};    // area: warp-shared windows above this many pixels, by bucket (0: 200)
    farm::StoreView view() const;
};
