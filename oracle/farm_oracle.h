/*
 * farm_oracle.h — CPU restatement of the FARM reference's polygon-join hot
 * path, in plain C. TEST INFRASTRUCTURE ONLY: the parity tests, smoke() and
 * bench.py's CPU-baseline leg use it to verify results; the product never
 * links, loads or calls it.
 *
 * Each function states the reference file:line it follows (paths relative to
 * the reference's src/). Behaviour is reproduced literally, including the
 * reference's quirks, because the pair sets it decides are the parity target.
 */
#ifndef FARM_ORACLE_H
#define FARM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FO_OK 0
#define FO_EASSERT (-10) /* a condition the reference asserts on was violated */
#define FO_ENOMEM (-3)
#define FO_EINVAL (-1)

typedef struct fo_layer {
    double mbr[4];
    int32_t dimx, dimy;
    double step_x, step_y;
    uint32_t offset; /* into status[] */
} fo_layer;

typedef struct fo_raster {
    double mbr[4]; /* lowx lowy highx highy (grid-aligned when hierarchical) */
    int32_t dimx, dimy;
    double step_x, step_y;
    uint32_t nv;          /* in-memory ring length (stored vertices + 1) */
    uint32_t status_size; /* finest layer pixels + coarser layers */
    uint8_t *status;
    uint32_t P;       /* dimx * dimy */
    uint32_t *offset; /* P + 1 */
    uint32_t n_seq;
    uint32_t *seq; /* n_seq x (start, length) */
    uint32_t n_hlines, n_hnodes;
    uint32_t *hoff;
    double *hnodes;
    uint32_t n_vlines, n_vnodes;
    uint32_t *voff;
    double *vnodes;
    double *areas; /* P */
    uint32_t num_layers;
    fo_layer *layers;
} fo_raster;

/* Options that are fixed in the reference but selectable here. */
typedef struct fo_opts {
    int vpr;            /* -v: vertices per pixel (preprocessing.cpp:15) */
    int hierarchy;      /* -h: grid_align + layering (preprocessing.cpp:17-19) */
    int category_count; /* fill classes; the reference fixes 16 (MyRaster.h:33) */
    int merge_carry;    /* see fo_rasterize(): how merge_status seeds its status */
    double grid_extent; /* hierarchy grid extent; 0 = 360 (the reference's degrees) */
} fo_opts;

/* Rasterize one polygon. `ring` holds the in-memory ring the reference builds
 * from a .dt record: the stored vertices, one more copy of the first, and one
 * pad vertex (copy of the first) read by single-pixel sequences; nv = stored + 1.
 * Follows preprocessing.cpp:4-29, MyRaster.cpp:8-33,444-491, Ideal.cpp:240-955,
 * 1008-1099. Returns FO_OK or FO_EASSERT. */
int fo_rasterize(const float *ring, uint32_t nv, const fo_opts *o, fo_raster *out);
void fo_raster_free(fo_raster *r);

/* Work counters of one pair decision, in the reference's evaluation order. */
typedef struct fo_counters {
    uint64_t window_pixels;   /* source pixels retrieved */
    uint64_t pixel_pairs;     /* (non-OUT, non-OUT) pixel pairs visited */
    uint64_t segment_tests;   /* segment-segment or point-segment evaluations */
    uint64_t seq_pairs;       /* edge-sequence pairs evaluated */
} fo_counters;

/* Ideal::intersect (Ideal.cpp:1329-1422). s/t rings as for fo_rasterize. */
int fo_intersect(const fo_raster *s, const float *sring, const fo_raster *t, const float *tring,
                 fo_counters *c);

/* The reference's "-a" approximate intersect (query_intersect.cu:32-134). */
int fo_intersect_heuristic(const fo_raster *s, const fo_raster *t);

/* Ideal::within (Ideal.cpp:2475-2643) with the hierarchy. geography selects
 * the reference's degree-to-km scaling (always on in the reference); off is
 * the planar mode for projected coordinates. */
int fo_within(const fo_raster *s, const float *sring, const fo_raster *t, const float *tring,
              double distance, int geography, fo_counters *c);

/* The reference's within "-a" rule (query_within_polygon.cu:332-375) on the
 * descent of fo_within: 1 / 0, no refinement. */
int fo_within_heuristic(const fo_raster *s, const fo_raster *t, double distance, int geography);

/* Single segment predicates (geometry_computation.h:190-221, :49-89). */
int fo_segment_intersect(const float *a, const float *b, const float *c, const float *d);
double fo_point_to_segment_distance(const float *p, const float *p1, const float *p2, int geography);

/* Ideal::segment_contain (Ideal.cpp:1233-1327): 0 OUT, 1 BORDER, 2 IN. */
int fo_segment_contain(const fo_raster *r, const float *ring, float px, float py);
/* Ideal::contain(Point &) (Ideal.cpp:1101-1157): 1 when the polygon holds the point. */
int fo_contain_point(const fo_raster *r, const float *ring, float px, float py);
/* Ideal::contain(Ideal *) (Ideal.cpp:1159-1231): 1 when s holds t. */
int fo_contain(const fo_raster *s, const float *sring, const fo_raster *t, const float *tring, fo_counters *c);

/* FP64 area of the intersection of two simple polygons (the project's area
 * oracle: the reference never computes areas). Boundary integral: the parts of
 * each boundary inside the other, integrated with the shoelace formula about a
 * common local origin. Rings as stored (closing copy included), m vertices. */
double fo_intersection_area(const float *a, uint32_t ma, const float *b, uint32_t mb);
/* The same area by plain loops over every edge pair (the definition the
 * indexed fo_intersection_area reproduces; for tests). */
double fo_intersection_area_plain(const float *a, uint32_t ma, const float *b, uint32_t mb);

/* Degree tables (util.h:68-96). */
double fo_degree_per_km_longitude(double lat);

#ifdef __cplusplus
}
#endif
#endif
