/*
 * farm_gpu.h — C ABI of the GB300 (sm_103a) engine for FARM's polygon-join
 * hot path. No CUDA or torch types: plain pointers, sizes and status codes.
 *
 * It replaces the reference's GPU offload entry points (src/include/Ideal.h:205-213):
 *   cuda_create_buffer / preprocess_for_gpu  -> farm_store_create + farm_store_load + farm_rasterize
 *   cuda_intersect                           -> farm_intersect
 *   cuda_within_polygon                      -> farm_within (farm_within_mode for -a)
 *   cuda_intersection                        -> farm_intersection_area
 *   ResetDevice                              -> (none: results are written to caller buffers)
 * and, for the CPU path it must agree with, Ideal::rasterization / Ideal::intersect /
 * Ideal::within (src/geometry/Ideal.cpp:936, 1329, 2475).
 *
 * Semantics differ from the reference's god-object API in three deliberate ways:
 * pair ids are (source index, target index) into two separate polygon tables
 * (as intersect_cpu.cpp:45-50 uses them); results are written to a caller
 * buffer (one byte per pair) besides the count; errors are returned, never
 * exit()ed. Every call is thread-compatible per store (one store per host thread).
 */
#ifndef FARM_GPU_H
#define FARM_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (shared with farm_host.h). */
#ifndef FARM_OK
#define FARM_OK 0
#define FARM_EINVAL (-1)
#define FARM_EIO (-2)
#define FARM_ENOMEM (-3)
#define FARM_EOVERFLOW (-4)
#define FARM_ECUDA (-5)
#define FARM_ETIMEOUT (-6)
#define FARM_EFORMAT (-7)
#define FARM_EINTERNAL (-8)
#endif
/* a condition the reference asserts on (and aborts) was met while rasterizing */
#define FARM_EASSERT (-10)

typedef struct farm_store farm_store;

/* Query modes for farm_intersect. */
#define FARM_MODE_EXACT 0   /* the reference's decision procedure, bit-exact */
#define FARM_MODE_APPROX 1  /* the reference's -a fill-ratio heuristic (query_intersect.cu:100-134), no refinement */
#define FARM_MODE_LEARNED 2 /* MLP scorer; abstentions refined exactly */
#define FARM_MODE_FILTER 3  /* the exact filter alone (device memory only): 1 = an IN overlap decides true,
                               0 = no non-OUT pixel pair (false), 3 = BORDER x BORDER pixel pairs to refine */

/* Pointer locations for pair lists and result buffers. */
#define FARM_MEM_HOST 0
#define FARM_MEM_DEVICE 1

typedef struct farm_raster_opts {
    int32_t vpr;            /* -v: vertices per pixel (reference default 10) */
    int32_t category_count; /* -w: fill classes 4/16/256 (reference fixes 16) */
    int32_t hierarchy;      /* -h: layered rasters (needed by within) */
    int32_t reserved;
    /* Extent of the hierarchy's global grid in coordinate units: its base step
     * is that extent / 2^25 rounded to 2 significant digits. 0 means 360 (the
     * reference's degrees, UniversalGrid.h:29-35); projected coordinates need
     * a larger extent (e.g. 1e7 for metres up to 5e6). */
    double grid_extent;
} farm_raster_opts;

typedef struct farm_stats {
    uint64_t pairs;          /* pairs decided */
    uint64_t found;          /* pairs whose result is true */
    uint64_t in_hits;        /* decided by an IN pixel overlap (intersect) */
    uint64_t border_pairs;   /* BORDER x BORDER pixel pairs examined (area: crossings counted) */
    uint64_t segment_tests;  /* segment-pair (or point-segment) evaluations (area: FP64 crossing tests) */
    uint64_t fp64_rechecks;  /* within: edge-sequence pairs re-evaluated in FP64 after the FP32 pass;
                                learned intersect: pairs refined exactly */
    double ms_total;         /* device time of the call (CUDA events) */
    double ms_stage[4];      /* raster, filter, refine, other */
    int32_t kernel_launches; /* engine kernels launched by the call */
    int32_t reserved;
    uint64_t src_window_pixels; /* source pixels in the target-MBR windows */
    uint64_t tgt_window_pixels; /* target pixels visited under non-OUT source pixels */
    uint64_t sequence_pairs;    /* within: edge-sequence pairs evaluated (FP32 pass) */
} farm_stats;

const char *farm_last_error(void);
/* Device ordinal and name the library runs on; returns FARM_ECUDA without a GPU. */
int farm_device_info(int *ordinal, char *name, size_t name_len);

int farm_store_create(farm_store **out);
void farm_store_destroy(farm_store *s);

/* Load one side's rings (side 0 = source, 1 = target). Rings in the host
 * layout of farm_host.h: off[n+1] (vertex offsets), xy float32 pairs with the
 * closing copy included, exactly as a .dt record stores them. mem says where
 * off/xy live (FARM_MEM_HOST or FARM_MEM_DEVICE). Replaces both sides' data.
 * xy holds the off[n] - off[0] vertices that the offsets describe. Host
 * vertices in pinned (page-locked) memory at an 8-byte boundary are read by
 * the device over the host link with no staging copy; others are staged
 * through a device buffer. Device vertices must start on an 8-byte boundary
 * (FARM_EINVAL otherwise). Either way the call returns once the rings are in
 * place.
 * For a self-join load side 0 only and pass target_is_source to the queries. */
int farm_store_load(farm_store *s, int side, uint64_t n, const uint64_t *off, const float *xy, int mem);

/* Load one side straight from a .dt file (storage.cpp format), replacing
 * the reference's pthread loader (storage.cpp:320-449) and its per-polygon
 * device copies: the file is mapped, all `threads` host threads (0 = every
 * core) decode its records into two pinned staging buffers of 256 MiB in the
 * store's ring layout, and each buffer is copied to HBM asynchronously while
 * the threads fill the other. Holes are dropped and rings with fewer than 3
 * in-memory vertices skipped, as the reference's loader does. *n_out (may be
 * NULL) gets the polygons kept. The same side rules as farm_store_load. */
int farm_store_load_dt(farm_store *s, int side, const char *path, int threads, uint64_t *n_out);

/* Rasterize every loaded polygon (reference: preprocessing.cpp:4-29,
 * Ideal.cpp:920-955). Must precede the queries. */
int farm_rasterize(farm_store *s, const farm_raster_opts *o);

/* Candidate pairs on the GPU, from the loaded rings (no rasterization
 * needed): every (source, target) whose closed MBRs overlap, the target's box
 * widened by `expand` (the within distance; in degrees by the reference's
 * longitude table when geography is set, Box.cpp:200-214), in ascending
 * (source, target) order: the set and order farm_mbr_join (farm_host.h)
 * returns, i.e. what the reference's R-tree search per target yields
 * (RTree.h:581-600, intersect_cpu.cpp:18-36). target_is_source: a self-join
 * of side 0 without (i, i). pairs: room for cap pairs (2 x uint32 each) in
 * memory `mem`; *n gets the count, and FARM_EOVERFLOW is returned (pairs
 * untouched) when it exceeds cap. */
int farm_mbr_join_gpu(farm_store *s, double expand, int geography, int target_is_source, uint32_t *pairs,
                      uint64_t cap, int mem, uint64_t *n);

/* Decide Ideal::intersect(source[p.s], target[p.t]) for n pairs. pairs: 2n
 * uint32 (s, t). out: n bytes, may be NULL: 0 / 1, or 2 when either polygon
 * failed rasterization (farm_raster_errors: the reference aborts on it).
 * found: count of 1s. */
int farm_intersect(farm_store *s, const uint32_t *pairs, uint64_t n, int mode, int mem, uint8_t *out,
                   uint64_t *found, farm_stats *st);

/* The exact filter alone on n device pairs (the learned mode's first stage):
 * d_code[k] as FARM_MODE_FILTER, d_cost[k] = pair k's refinement cost proxy
 * (float): the BORDER x BORDER pixel pairs it found x both polygons' edges per
 * pixel. No counterpart in the reference. */
int farm_intersect_filter(farm_store *s, const uint32_t *d_pairs, uint64_t n, uint8_t *d_code, float *d_cost);

/* Decide Ideal::within(source[p.s], target[p.t]) (hierarchical rasters required).
 * distance in km with geography (the reference: 10 km, degree coordinates),
 * in coordinate units without (planar mode for projected coordinates). */
int farm_within(farm_store *s, const uint32_t *pairs, uint64_t n, double distance, int geography,
                int target_is_source, int mem, uint8_t *out, uint64_t *found, farm_stats *st);

/* farm_within with a mode: FARM_MODE_EXACT (= farm_within) or FARM_MODE_APPROX,
 * the reference's within "-a" rule (query_within_polygon.cu:332-375, :721-742):
 * a pair the hierarchical descent leaves undecided is within when one of its
 * finest surviving BORDER pixel pairs has min + 0.5 (max - min) <= distance
 * (float), with no refinement. Other modes are FARM_EINVAL. */
int farm_within_mode(farm_store *s, const uint32_t *pairs, uint64_t n, double distance, int geography,
                     int target_is_source, int mode, int mem, uint8_t *out, uint64_t *found, farm_stats *st);

/* Polygon containment, source[p.s] holds target[p.t], per candidate pair
 * (Ideal::contain(Ideal *), Ideal.cpp:1159-1231; the reference's GPU form,
 * query_contain.cu, is commented out, so no reference entry is replaced).
 * out: one byte per pair, 1 / 0, or 2 where either polygon failed to
 * rasterize. pairs and out live in memory `mem`. st may be NULL; border_pairs
 * counts the pixel pairs whose edges were tested and segment_tests the
 * segment pairs. */
int farm_contain(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint8_t *out, uint64_t *found,
                 farm_stats *st);
/* Point containment, polygon p of `side` holds point q (Ideal::contain(Point &),
 * Ideal.cpp:1101-1157), per (p, q) pair: xy holds npoints float32 (x, y)
 * points; pairs are (polygon, point) indices; out as for farm_contain. xy,
 * pairs and out live in memory `mem`. */
int farm_contain_points(farm_store *s, int side, const float *xy, uint64_t npoints, const uint32_t *pairs,
                        uint64_t n, int mem, uint8_t *out, uint64_t *found);

/* FP64 area of source[p.s] ∩ target[p.t] for n pairs (out: n doubles). The
 * reference stops before computing it (Ideal.cpp:1683); this is the project's
 * boundary-integral formulation. */
int farm_intersection_area(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, double *out,
                           farm_stats *st);

/* Copy one rasterized polygon back for inspection (tests): sizes first with
 * NULL buffers, then the arrays. side/index select the polygon. */
typedef struct farm_raster_view {
    double mbr[4];
    int32_t dimx, dimy;
    double step_x, step_y;
    uint32_t nv, status_size, n_seq, n_hnodes, n_vnodes, num_layers;
    int32_t err;
    uint32_t reserved;
} farm_raster_view;
int farm_raster_fetch(farm_store *s, int side, uint64_t index, farm_raster_view *v, uint8_t *status,
                      uint32_t *offset, uint32_t *seq, uint32_t *hoff, double *hnodes, uint32_t *voff,
                      double *vnodes, double *areas, double *layer_info /* 7 doubles per layer */);

/* Allocation-free variant of farm_intersect (no counterpart in the reference):
 * for callers that cannot allocate device memory at query time — code whose
 * device memory belongs to another allocator (e.g. a framework's caching
 * allocator that has reserved the HBM), or threads that must not trigger the
 * device-wide synchronisation of cudaMalloc/cudaFree while other streams run.
 * pairs (2n uint32) and out (n bytes, same encoding as farm_intersect) are
 * HOST buffers; the staged pairs, results and counters live in a fixed
 * file-scope device array of about 9 MiB that every device which loads the
 * library keeps until process exit. At most 1,048,576 pairs per call; larger
 * n is rejected with FARM_EINVAL. The first call on a device looks the array's
 * address up (cudaGetSymbolAddress) with that device current: make that first
 * call before any stream capture. All calls share the array and it keeps the
 * last call's contents, so calls that overlap on the GPU (from different host
 * threads or stores) race; serialise them. The store itself must already be
 * loaded and rasterized (those steps allocate). The looked-up address is kept
 * for the life of the process: do not reset the device (cudaDeviceReset) or
 * tear down its primary context while this entry point is in use. Pair
 * indices are range-checked on the host before any device work. */
int farm_intersect_static(farm_store *s, const uint32_t *pairs, uint64_t n, uint8_t *out, uint64_t *found);

/* Diagnostics: the learned scorer's tcgen05 GEMM on its own, C[M x N] (fp32)
 * = A[M x K] * B[N x K]^T (bf16, row-major, device pointers); M, N multiples
 * of 16, K a multiple of 64, BN the tile width (64, 128, 256). */
int farm_tc_gemm_test(const void *A, const void *B, float *C, int M, int N, int K, int BN);

/* ---- batched area queries (no counterpart in the reference) ----
 * A plan captures one area pass — work items per pair, their scan, the
 * persistent work-stealing area kernel and the per-pair reduction — in a CUDA
 * graph over buffers of fixed capacity. farm_area_plan_run copies a batch of
 * up to max_pairs pairs in and replays the graph (results as
 * farm_intersection_area). max_items bounds the batch's work items: each pair
 * has ceil(edges_s / chunk) + ceil(edges_t / chunk) of them (chunk per size
 * bucket, 16 by default); a batch needing more fails with FARM_EOVERFLOW.
 * A plan is tied to the store's current rasterization. */
typedef struct farm_area_plan farm_area_plan;
int farm_area_plan_create(farm_store *s, uint64_t max_pairs, uint64_t max_items, farm_area_plan **out);
int farm_area_plan_run(farm_area_plan *p, const uint32_t *pairs, uint64_t n, int mem, double *out, farm_stats *st);
void farm_area_plan_destroy(farm_area_plan *p);
/* Edges per area work item by size bucket b = floor(log2(larger edge count of
 * the pair)), 32 entries (0 = default 16). */
int farm_area_set_chunks(farm_store *s, const int32_t *chunk_by_bucket);
/* Candidate-window size (pixels of the other polygon's raster) above which an
 * edge is searched by the whole warp rather than its own lane, by size
 * bucket, 32 entries (0 = default 200). */
int farm_area_set_wide(farm_store *s, const int32_t *wide_by_bucket);
/* Per size bucket present in the sample (up to 2048 pairs each): time the
 * chunk sizes 8..256, then at the best chunk the window sizes 24..800, keep
 * the fastest of each in the store and return both tables (32 entries each;
 * either output may be NULL). */
int farm_area_autotune(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, int32_t *chunk_out,
                       int32_t *wide_out);

/* ---- learned scorer (FARM_MODE_LEARNED): 520 -> 256 -> 256 -> 1 MLP, GELU,
 * bf16 weights/activations on tcgen05 tensor cores, fp32 accumulate. It takes
 * the place of the reference's "-a" confidence heuristic
 * (src/cuda/query_intersect.cu:100-134). Parameters are laid out as
 * W1 [256 x 576] | W2 [256 x 256] | b1 [256] | b2 [256] | w3 [256] | b3. */
uint64_t farm_mlp_param_count(void);
int farm_mlp_init(farm_store *s, uint64_t seed);
int farm_mlp_get(farm_store *s, float *params);
int farm_mlp_set(farm_store *s, const float *params);
/* Probability >= hi decides 1, <= lo decides 0, otherwise exact refinement. */
int farm_mlp_set_band(farm_store *s, float lo, float hi);
/* Cost-aware band (0 = off): a pair is also decided (by p >= 0.5) when
 * min(p, 1 - p) <= lambda x its refinement cost proxy (farm_intersect_filter). */
int farm_mlp_set_band_cost(farm_store *s, float lambda);
/* Features (bf16 [rows x 576], rows >= n, zero padding) of n device pairs. */
int farm_mlp_features(farm_store *s, const uint32_t *d_pairs, uint64_t n, void *d_X, uint64_t rows);
/* One forward/backward on device features and labels; loss and gradients
 * (parameter layout) copied to host buffers; no update. */
int farm_mlp_grad(farm_store *s, const void *d_X, const uint8_t *d_y, uint64_t n, uint64_t rows, float *loss,
                  float *grad);
/* Adam training on device pairs with device labels (exact results). */
int farm_mlp_train(farm_store *s, const uint32_t *d_pairs, const uint8_t *d_labels, uint64_t n, int epochs,
                   int batch, float lr, uint64_t seed, float *last_loss);
/* Probabilities of n device pairs into d_prob (device fp32). */
int farm_mlp_predict(farm_store *s, const uint32_t *d_pairs, uint64_t n, float *d_prob);

/* Per-polygon rasterization status of one side (n = that side's polygon
 * count): 0, or FARM_EASSERT for a polygon on which the reference asserts or
 * never terminates (such polygons are reported, not rasterized). */
int farm_raster_errors(farm_store *s, int side, int32_t *err, uint64_t n);

/* Sizes of the last rasterization, summed over both sides: the units the
 * rasterizer's kernels process (crossings, fill-clip points) and the raster
 * arrays it wrote. No counterpart in the reference. */
typedef struct farm_raster_totals {
    uint64_t polygons, vertices;       /* vertices = edges (closing copy included) */
    uint64_t pixels, status_bytes;     /* finest pixels; status incl. coarser layers */
    uint64_t sequences, hnodes, vnodes;
    uint64_t crossings;                /* pixel-boundary crossings of the edge walk */
    uint64_t clip_x_points, clip_y_points; /* points emitted by the column / cell clips */
    uint64_t chunks;
    /* device time (CUDA events) of the edge-walk kernels, the column-clip
     * kernels, the cell-clip kernels, the cell-area kernel, and the whole call */
    double ms_walk, ms_clip_x, ms_clip_y, ms_cells, ms_total;
} farm_raster_totals;
int farm_raster_get_totals(farm_store *s, farm_raster_totals *out);

/* Wait for outstanding work of the store's stream. */
int farm_sync(farm_store *s);

/* CUDA-event timing on the store's stream (slots 0-5): record, then elapsed ms a -> b. */
int farm_event_record(farm_store *s, int slot);
int farm_event_elapsed(farm_store *s, int a, int b, double *ms);
/* Engine kernels launched through this store so far. */
uint64_t farm_store_launches(farm_store *s);
/* Measured non-fused FP64 and FP32 arithmetic rates of the current device
 * (multiplies or adds per second), the denominators of the FP64- and
 * FP32-bound rooflines. No counterpart in the reference. */
int farm_probe_issue_rates(double *fp64_ops_per_s, double *fp32_ops_per_s);

/* Device bytes the store currently holds in its own allocations (rings,
 * rasters, query scratch), the learned scorer's state excluded. No
 * counterpart in the reference. */
int farm_store_device_bytes(farm_store *s, uint64_t *bytes);

#ifdef __cplusplus
}
#endif
#endif
