/*
 * farm_host.h — host-side C ABI of the GB300 polygon-join engine: the .dt
 * polygon file format, the seeded synthetic star-polygon generator and the
 * MBR candidate join. No CUDA types; plain pointers and sizes.
 *
 * Vertex layout ("rings"): polygon k owns xy[2*off[k] .. 2*off[k+1]) as
 * interleaved float32 (x, y) pairs, exactly the vertices of one .dt record
 * (closing copy of the first vertex included, as the reference's WKT loader
 * stores them). off has n+1 entries.
 *
 * Every function returns 0 on success or a negative FARM_E* code; the last
 * error text of the calling thread is available from farm_host_last_error().
 */
#ifndef FARM_HOST_H
#define FARM_HOST_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FARM_OK 0
#define FARM_EINVAL (-1)
#define FARM_EIO (-2)
#define FARM_ENOMEM (-3)
#define FARM_EOVERFLOW (-4)
#define FARM_ECUDA (-5)
#define FARM_ETIMEOUT (-6)
#define FARM_EFORMAT (-7)
#define FARM_EINTERNAL (-8)

const char *farm_host_last_error(void);

/* Seeded star polygons. Polygon i (global index first+i) is drawn from a
 * counter-based generator keyed by (seed, i), so any sub-range can be made
 * independently and in parallel:
 *   centre uniform in [dom_lo, dom_hi]^2; mean radius log-uniform in
 *   [r_lo, r_hi]; vertex count log-uniform in [n_lo, n_hi]; vertex angles
 *   sorted uniform over one turn (counter-clockwise; redrawn until no angular
 *   gap exceeds a third of a turn, which keeps every ring simple and
 *   star-shaped); per-vertex radius = mean radius x lognormal(0, sigma).
 *   Coordinates are computed in FP64 and rounded to float32, as a .dt file
 *   stores them. */
typedef struct farm_gen_params {
    double dom_lo, dom_hi;
    double r_lo, r_hi;
    int32_t n_lo, n_hi;
    double sigma;
} farm_gen_params;

/* Pass 1: per-polygon stored vertex counts (N distinct + 1 closing copy). */
int farm_gen_counts(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count,
                    uint32_t *nverts_out);
/* Centre (cx, cy) and mean radius of each polygon, 3 doubles per polygon,
 * without drawing its vertices (the same counters as farm_gen_fill). */
int farm_gen_centres(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count, double *cxyr);
/* Largest vertex distance from the centre of each polygon (the mean radius
 * times its largest lognormal factor), from the same draws as farm_gen_fill
 * without computing the vertices: every vertex of polygon i lies within
 * rmax[i] of its centre, up to the float32 rounding of its coordinates. */
int farm_gen_radii(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count, double *rmax,
                   int threads);
/* Pass 2: fill rings; off (count+1 entries) must be the exclusive scan of the
 * counts from pass 1 (off[0] may be non-zero: it is an absolute offset into xy). */
int farm_gen_fill(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count,
                  const uint64_t *off, float *xy, int threads);

/* The same two passes for an arbitrary list of generator indices: output
 * polygon k is generator polygon idx[k]. */
int farm_gen_counts_idx(const farm_gen_params *gp, uint64_t seed, const uint64_t *idx, uint64_t count,
                        uint32_t *nverts_out);
int farm_gen_fill_idx(const farm_gen_params *gp, uint64_t seed, const uint64_t *idx, uint64_t count,
                      const uint64_t *off, float *xy, int threads);

/* .dt files (storage.cpp format): records [size_t holes][size_t nv][nv x float2] ...,
 * then PolygonMeta[n] {uint32 size, uint32 nv, uint64 offset, double mbr[4]},
 * then uint64 n. Holes are written as none; on read they are skipped, and
 * polygons whose in-memory ring (stored count + 1) has fewer than 3 vertices
 * are dropped, as the reference loader does. */
int farm_dt_write(const char *path, uint64_t n, const uint64_t *off, const float *xy);
/* Read in two calls: first with xy == NULL to learn n and the total vertex
 * count, then with buffers of that size. */
int farm_dt_read(const char *path, uint64_t *n_out, uint64_t *total_out, uint64_t *off, float *xy);

/* WKT polygons, one per line, parsed by the rules of the reference's
 * load_polygon_wkt / read_polygon (storage.cpp:8-94, :683-715;
 * MyPolygon.cpp:227-262): parsing starts at the line's first '(', a ring has
 * one vertex more than the commas before its first ')', coordinates are runs
 * of [-.0-9e] read by atof and stored as float32, rings keep their order, a
 * MULTIPOLYGON yields its first polygon and empty lines are skipped. A line
 * the reference would assert on or read past gives FARM_EFORMAT.
 *
 * farm_wkt_read returns the boundaries as rings, in the two-call protocol of
 * farm_dt_read. */
int farm_wkt_read(const char *path, uint64_t *n_out, uint64_t *total_out, uint64_t *off, float *xy);
/* WKT file to .dt file, byte for byte what the reference's dump_polygons
 * tool writes (dump_polygons.cpp:4-15, storage.cpp:158-193): records without
 * holes (the reference's parser appends holes to a copy, MyPolygon.h:132),
 * each meta's vertex count the boundary's as parsed. n_out may be NULL. */
int farm_wkt_to_dt(const char *wkt_path, const char *dt_path, uint64_t *n_out);

/* Minimum bounding rectangles of the rings, as the reference computes them:
 * min/max of the float32 vertices in FP64, widened by the float32 constant 1e-9
 * (vertex_sequence.cpp:152-168). mbr is 4 doubles per polygon (lowx lowy highx highy). */
int farm_mbr(uint64_t n, const uint64_t *off, const float *xy, double *mbr, int threads);

/* MBR candidate join: every (s, t) whose closed rectangles overlap after the
 * target rectangle is widened by `expand` (0 for intersect), excluding s == t
 * when skip_same is set (self-join). The pair list is sorted by (s, t).
 * Two-call protocol: pairs == NULL returns the count in *npairs. With
 * geography set the widening follows the reference's degree conversion
 * (Box.cpp:200-214). */
int farm_mbr_join(uint64_t ns, const double *mbr_s, uint64_t nt, const double *mbr_t, double expand,
                  int geography, int skip_same, uint64_t *npairs, uint32_t *pairs, int threads);

/* The reference's longitude degree-per-km table (900 entries, util.h:73),
 * regenerated from its defining formula. */
void farm_degree_table(double *out900);

#ifdef __cplusplus
}
#endif
#endif
