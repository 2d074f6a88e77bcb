/*
 * farm_oracle.c — CPU restatement of the FARM reference's polygon-join hot
 * path. TEST INFRASTRUCTURE ONLY (see farm_oracle.h): it verifies the GPU
 * engine's results and is never part of it.
 *
 * Built with -ffp-contract=off: the reference is compiled for x86-64 without
 * -march (src/Makefile:11), so none of its multiply-adds are fused; every
 * expression below is evaluated in the same order and precision.
 */
#include "farm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- util.h -- */

/* util.h:98-106 */
static int double_to_int(double val) {
    int vi = (int)val;
    if (fabs(1.0 * (vi + 1) - val) < 0.00000001) vi++;
    return vi;
}

/* util.h:53-66 */
static double round_sig(double num, int n) {
    if (num == 0) return 0;
    double d = ceil(log10(num < 0 ? -num : num));
    int power = n - (int)d;
    double magnitude = pow(10.0, power);
    double shifted = round(num * magnitude);
    return shifted / magnitude;
}

/* util.h:68: fitted mean fill of a pixel pair by class (float constants). */
static const float k_mean20[20] = {0.0f,  0.7f,  0.62f, 0.55f, 0.52f, 0.45f, 0.42f, 0.4f,  0.38f, 0.34f,
                                   0.31f, 0.28f, 0.25f, 0.22f, 0.18f, 0.15f, 0.1f,  0.05f, 0.0f,  0.0f};

/* util.h:72-96; table entries regenerated from the formula they were printed from. */
static double g_deg_lon[900];
static int g_deg_ready = 0;
static void deg_init(void) {
    if (g_deg_ready) return;
    const double PI = 3.14159265;
    for (int i = 0; i < 900; i++) {
        double lat = i / 10.0;
        double v = 360.0 / (sin((90 - lat) * PI / 180) * 40076);
        /* printed with 6 decimals */
        g_deg_lon[i] = round(v * 1e6) / 1e6;
        char buf[64];
        /* use the decimal text so the double equals the compiled literal */
        int k = 0;
        long long iv = (long long)llround(v * 1e6);
        long long ip = iv / 1000000, fp = iv % 1000000;
        k = 0;
        (void)k;
        {
            /* build "ip.ffffff" */
            char *q = buf;
            long long t = ip;
            char tmp[32];
            int n = 0;
            do { tmp[n++] = (char)('0' + t % 10); t /= 10; } while (t);
            while (n) *q++ = tmp[--n];
            *q++ = '.';
            long long f = fp;
            for (int d = 5; d >= 0; d--) { q[d] = (char)('0' + f % 10); f /= 10; }
            q[6] = 0;
        }
        g_deg_lon[i] = strtod(buf, NULL);
    }
    g_deg_ready = 1;
}
static const double k_deg_lat = 360.0 / 40076.0;

double fo_degree_per_km_longitude(double latitude) {
    deg_init();
    double absla = fabs(latitude);
    if (absla == 90) absla = 89.9;
    int idx = (int)(absla * 10);
    /* the reference indexes past the table here (it only sees degrees) */
    if (idx < 0 || idx >= 900) idx = 899;
    return g_deg_lon[idx];
}

/* ------------------------------------------------------ Point.h / float -- */

typedef struct { float x, y; } pt;

/* Point.h:402-403 */
static int pt_eq(pt a, pt b) { return fabsf(a.x - b.x) < 1e-9 && fabsf(a.y - b.y) < 1e-9; }
static int pt_ne(pt a, pt b) { return fabsf(a.x - b.x) >= 1e-9 || fabsf(a.y - b.y) >= 1e-9; }

/* Point.h:463-467: (a - o) x (b - o), all in float */
static float cross3(pt o, pt a, pt b) {
    float ax = a.x - o.x, ay = a.y - o.y, bx = b.x - o.x, by = b.y - o.y;
    float l = ax * by;
    float r = ay * bx;
    return l - r;
}

/* geometry_computation.h:190-193 */
static int sgn(double x) { return x >= 0 ? (x ? 1 : 0) : -1; }

/* geometry_computation.h:195-212 */
static int inter1(double a, double b, double c, double d) {
    double tmp;
    if (a > b) { tmp = a; a = b; b = tmp; }
    if (c > d) { tmp = c; c = d; d = tmp; }
    return (a > c ? a : c) <= (b < d ? b : d);
}

/* geometry_computation.h:215-221 */
static int seg_intersect(pt a, pt b, pt c, pt d) {
    if (cross3(c, a, d) == 0 && cross3(c, b, d) == 0)
        return inter1(a.x, b.x, c.x, d.x) && inter1(a.y, b.y, c.y, d.y);
    return sgn(cross3(a, b, c)) != sgn(cross3(a, b, d)) && sgn(cross3(c, d, a)) != sgn(cross3(c, d, b));
}

int fo_segment_intersect(const float *a, const float *b, const float *c, const float *d) {
    pt A = {a[0], a[1]}, B = {b[0], b[1]}, C = {c[0], c[1]}, D = {d[0], d[1]};
    return seg_intersect(A, B, C, D);
}

/* geometry_computation.h:49-89 */
static double pt_seg_dist(pt p, pt p1, pt p2, int geography) {
    double A = (float)(p.x - p1.x);
    double B = (float)(p.y - p1.y);
    double C = (float)(p2.x - p1.x);
    double D = (float)(p2.y - p1.y);
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
    double dx = p.x - xx;
    double dy = p.y - yy;
    if (geography) {
        dx = dx / fo_degree_per_km_longitude(p.y);
        dy = dy / k_deg_lat;
    }
    return sqrt(dx * dx + dy * dy);
}

double fo_point_to_segment_distance(const float *p, const float *p1, const float *p2, int geography) {
    pt P = {p[0], p[1]}, P1 = {p1[0], p1[1]}, P2 = {p2[0], p2[1]};
    return pt_seg_dist(P, P1, P2, geography);
}

/* geometry_computation.h:136-182: `n1` points of vs1 against the n2 - 1
 * segments of vs2 and the reverse (the sequences' last edges are not used). */
static double seq_within_batch(const pt *vs1, const pt *vs2, int s1, int s2, int geography, uint64_t *tests) {
    double mindist = 1.7976931348623157e308;
    for (int i = 0; i < s1; i++) {
        double m = 1.7976931348623157e308;
        for (int j = 0; j < s2 - 1; j++) {
            double d = pt_seg_dist(vs1[i], vs2[j], vs2[j + 1], geography);
            if (d < m) m = d;
        }
        if (tests) *tests += (s2 > 1) ? (uint64_t)(s2 - 1) : 0;
        if (m < mindist) mindist = m;
    }
    for (int i = 0; i < s2; i++) {
        double m = 1.7976931348623157e308;
        for (int j = 0; j < s1 - 1; j++) {
            double d = pt_seg_dist(vs2[i], vs1[j], vs1[j + 1], geography);
            if (d < m) m = d;
        }
        if (tests) *tests += (s1 > 1) ? (uint64_t)(s1 - 1) : 0;
        if (m < mindist) mindist = m;
    }
    return mindist;
}

/* ------------------------------------------------------------- raster --- */

typedef struct {
    uint32_t pix;
    uint8_t type; /* 0 ENTER, 1 LEAVE (Ideal.h:16-20) */
    int32_t edge;
} rec_t;
typedef struct {
    uint32_t line;
    double v;
} node_t;

typedef struct {
    rec_t *r;
    size_t n, cap;
} recv_t;
typedef struct {
    node_t *r;
    size_t n, cap;
} nodev_t;

static int recv_push(recv_t *v, uint32_t pix, uint8_t type, int32_t edge) {
    if (v->n == v->cap) {
        size_t nc = v->cap ? v->cap * 2 : 64;
        rec_t *nr = (rec_t *)realloc(v->r, nc * sizeof(rec_t));
        if (!nr) return FO_ENOMEM;
        v->r = nr;
        v->cap = nc;
    }
    v->r[v->n].pix = pix;
    v->r[v->n].type = type;
    v->r[v->n].edge = edge;
    v->n++;
    return FO_OK;
}
static int nodev_push(nodev_t *v, uint32_t line, double val) {
    if (v->n == v->cap) {
        size_t nc = v->cap ? v->cap * 2 : 64;
        node_t *nr = (node_t *)realloc(v->r, nc * sizeof(node_t));
        if (!nr) return FO_ENOMEM;
        v->r = nr;
        v->cap = nc;
    }
    v->r[v->n].line = line;
    v->r[v->n].v = val;
    v->n++;
    return FO_OK;
}

typedef struct {
    fo_raster *R;
    const pt *p;
    uint32_t nv;
    int cc;
    recv_t recs;
    nodev_t hn, vn;
    int err;
} rctx;

/* MyRaster.cpp:228-239 */
static int show_status_cc(uint8_t s, int cc) {
    if (s == 0) return 0;          /* OUT */
    if (s == cc - 1) return 2;     /* IN */
    return 1;                      /* BORDER */
}

#define CHK(c)                       \
    do {                             \
        if (!(c)) {                  \
            X->err = FO_EASSERT;     \
            return;                  \
        }                            \
    } while (0)

/* MyRaster.cpp:170-174 */
static int pid(rctx *X, int x, int y) {
    fo_raster *R = X->R;
    if (x < 0 || x >= R->dimx || y < 0 || y >= R->dimy) {
        X->err = FO_EASSERT;
        return 0;
    }
    return y * R->dimx + x;
}
static void set_border(rctx *X, int x, int y) {
    int id = pid(X, x, y);
    if (X->err) return;
    X->R->status[id] = 1; /* BORDER */
}
static void push_rec(rctx *X, int x, int y, int type, int edge) {
    int id = pid(X, x, y);
    if (X->err) return;
    if (recv_push(&X->recs, (uint32_t)id, (uint8_t)type, edge)) X->err = FO_ENOMEM;
}

#define ENTER 0
#define LEAVE 1

/* Ideal.cpp:252-538 (the edge walk) */
static void evaluate_edges(rctx *X) {
    fo_raster *R = X->R;
    const double start_x = R->mbr[0];
    const double start_y = R->mbr[1];
    const double step_x = R->step_x, step_y = R->step_y;
    const int dimx = R->dimx, dimy = R->dimy;
    for (int i = 0; i < (int)X->nv - 1; i++) {
        double x1 = X->p[i].x, y1 = X->p[i].y, x2 = X->p[i + 1].x, y2 = X->p[i + 1].y;
        int cur_startx = double_to_int((x1 - start_x) / step_x);
        int cur_endx = double_to_int((x2 - start_x) / step_x);
        int cur_starty = double_to_int((y1 - start_y) / step_y);
        int cur_endy = double_to_int((y2 - start_y) / step_y);
        if (cur_startx == dimx) cur_startx--;
        if (cur_endx == dimx) cur_endx--;
        if (cur_starty == dimy) cur_starty--;
        if (cur_endy == dimy) cur_endy--;
        CHK(cur_startx < dimx && cur_endx < dimx && cur_starty < dimy && cur_endy < dimy);
        set_border(X, cur_startx, cur_starty);
        set_border(X, cur_endx, cur_endy);
        if (X->err) return;
        if (cur_startx == cur_endx && cur_starty == cur_endy) continue;

        if (y1 == y2) {
            if (cur_startx < cur_endx) {
                for (int x = cur_startx; x < cur_endx; x++) {
                    if (nodev_push(&X->vn, (uint32_t)(x + 1), y1)) { X->err = FO_ENOMEM; return; }
                    push_rec(X, x, cur_starty, LEAVE, i);
                    push_rec(X, x + 1, cur_starty, ENTER, i);
                    set_border(X, x, cur_starty);
                    set_border(X, x + 1, cur_starty);
                    if (X->err) return;
                }
            } else {
                for (int x = cur_startx; x > cur_endx; x--) {
                    if (nodev_push(&X->vn, (uint32_t)x, y1)) { X->err = FO_ENOMEM; return; }
                    push_rec(X, x, cur_starty, LEAVE, i);
                    push_rec(X, x - 1, cur_starty, ENTER, i);
                    set_border(X, x, cur_starty);
                    set_border(X, x - 1, cur_starty);
                    if (X->err) return;
                }
            }
        } else if (x1 == x2) {
            if (cur_starty < cur_endy) {
                for (int y = cur_starty; y < cur_endy; y++) {
                    if (nodev_push(&X->hn, (uint32_t)(y + 1), x1)) { X->err = FO_ENOMEM; return; }
                    push_rec(X, cur_startx, y, LEAVE, i);
                    push_rec(X, cur_startx, y + 1, ENTER, i);
                    set_border(X, cur_startx, y);
                    set_border(X, cur_startx, y + 1);
                    if (X->err) return;
                }
            } else {
                for (int y = cur_starty; y > cur_endy; y--) {
                    if (nodev_push(&X->hn, (uint32_t)y, x1)) { X->err = FO_ENOMEM; return; }
                    push_rec(X, cur_startx, y, LEAVE, i);
                    push_rec(X, cur_startx, y - 1, ENTER, i);
                    set_border(X, cur_startx, y);
                    set_border(X, cur_startx, y - 1);
                    if (X->err) return;
                }
            }
        } else {
            double a = (y1 - y2) / (x1 - x2);
            double b = (x1 * y2 - x2 * y1) / (x1 - x2);
            int x = cur_startx;
            int y = cur_starty;
            long guard = 4L * (labs((long)cur_endx - cur_startx) + labs((long)cur_endy - cur_starty) + 4);
            while (x != cur_endx || y != cur_endy) {
                /* the reference loops forever if no step is taken; bound it */
                CHK(--guard > 0);
                int passed = 0;
                double yval = 0;
                double xval = 0;
                int cur_x = 0;
                int cur_y = 0;
                if (x != cur_endx) {
                    if (cur_startx < cur_endx)
                        xval = ((double)x + 1) * step_x + start_x;
                    else
                        xval = (double)x * step_x + start_x;
                    yval = xval * a + b;
                    if (fabs((yval - start_y) / step_y - round((yval - start_y) / step_y)) < 1e-9) {
                        /* Ideal.cpp:396-422: the edge passes a grid corner */
                        if (cur_startx < cur_endx && cur_starty < cur_endy) {
                            if (nodev_push(&X->vn, (uint32_t)(x + 1), yval)) { X->err = FO_ENOMEM; return; }
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            x++;
                            y++;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        } else if (cur_startx < cur_endx && cur_starty > cur_endy) {
                            if (nodev_push(&X->vn, (uint32_t)x, yval)) { X->err = FO_ENOMEM; return; }
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            x++;
                            y--;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        } else if (cur_startx > cur_endx && cur_starty < cur_endy) {
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            x--;
                            y++;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        } else if (cur_startx > cur_endx && cur_starty > cur_endy) {
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            x--;
                            y--;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        }
                        if (X->err) return;
                        continue;
                    }
                    cur_y = (int)((yval - start_y) / step_y);
                    int ymax = cur_endy > cur_starty ? cur_endy : cur_starty;
                    int ymin = cur_endy < cur_starty ? cur_endy : cur_starty;
                    if (cur_y > ymax) cur_y = ymax;
                    if (cur_y < ymin) cur_y = ymin;
                    if (cur_y == y) {
                        passed = 1;
                        if (cur_startx < cur_endx) {
                            if (nodev_push(&X->vn, (uint32_t)(x + 1), yval)) { X->err = FO_ENOMEM; return; }
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            x++;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        } else {
                            if (nodev_push(&X->vn, (uint32_t)x, yval)) { X->err = FO_ENOMEM; return; }
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            x--;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        }
                        if (X->err) return;
                    }
                }
                if (y != cur_endy) {
                    if (cur_starty < cur_endy)
                        yval = (double)(y + 1) * step_y + start_y;
                    else
                        yval = (double)y * step_y + start_y;
                    xval = (yval - b) / a;
                    cur_x = (int)((xval - start_x) / step_x);
                    int xmax = cur_endx > cur_startx ? cur_endx : cur_startx;
                    int xmin = cur_endx < cur_startx ? cur_endx : cur_startx;
                    if (cur_x > xmax) cur_x = xmax;
                    if (cur_x < xmin) cur_x = xmin;
                    if (cur_x == x) {
                        passed = 1;
                        if (cur_starty < cur_endy) {
                            if (nodev_push(&X->hn, (uint32_t)(y + 1), xval)) { X->err = FO_ENOMEM; return; }
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            y++;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        } else {
                            if (nodev_push(&X->hn, (uint32_t)y, xval)) { X->err = FO_ENOMEM; return; }
                            set_border(X, x, y);
                            push_rec(X, x, y, LEAVE, i);
                            y--;
                            push_rec(X, x, y, ENTER, i);
                            set_border(X, x, y);
                        }
                        if (X->err) return;
                    }
                }
                CHK(passed);
            }
        }
    }
}

static int cmp_double(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Ideal.cpp:185-238: nodes of each grid line, sorted; lines without nodes keep
 * offset 0 (the offsets are zero-filled at Grid_line.cpp:3-8). */
static int build_lines(nodev_t *nv, uint32_t nlines_minus2, int vertical, uint32_t **off_out, double **nodes_out,
                       uint32_t *n_out) {
    uint32_t L = nlines_minus2 + 2;
    uint32_t *off = (uint32_t *)calloc(L, sizeof(uint32_t));
    double *nodes = (double *)malloc((nv->n ? nv->n : 1) * sizeof(double));
    uint32_t *cnt = (uint32_t *)calloc(L + 1, sizeof(uint32_t));
    if (!off || !nodes || !cnt) {
        free(off);
        free(nodes);
        free(cnt);
        return FO_ENOMEM;
    }
    for (size_t k = 0; k < nv->n; k++) {
        if (nv->r[k].line >= L) {
            free(off);
            free(nodes);
            free(cnt);
            return FO_EASSERT;
        }
        cnt[nv->r[k].line + 1]++;
    }
    for (uint32_t l = 0; l < L; l++) cnt[l + 1] += cnt[l];
    uint32_t *fillp = (uint32_t *)malloc((L + 1) * sizeof(uint32_t));
    if (!fillp) {
        free(off);
        free(nodes);
        free(cnt);
        return FO_ENOMEM;
    }
    memcpy(fillp, cnt, (L + 1) * sizeof(uint32_t));
    for (size_t k = 0; k < nv->n; k++) nodes[fillp[nv->r[k].line]++] = nv->r[k].v;
    for (uint32_t l = 0; l < L; l++) {
        uint32_t b = cnt[l], e = cnt[l + 1];
        if (e > b) {
            qsort(nodes + b, e - b, sizeof(double), cmp_double);
            off[l] = b;
        }
    }
    uint32_t total = (uint32_t)nv->n;
    if (vertical) {
        off[nlines_minus2 + 1] = total;
        off[nlines_minus2] = total;
    } else {
        off[nlines_minus2] = total;
    }
    free(cnt);
    free(fillp);
    *off_out = off;
    *nodes_out = nodes;
    *n_out = total;
    return FO_OK;
}

/* Ideal.cpp:90-183 over the per-pixel record lists (map order = pixel order,
 * records within a pixel in the order they were produced). */
static int process_crosses(rctx *X) {
    fo_raster *R = X->R;
    size_t n = X->recs.n;
    uint32_t P = R->P;
    /* stable counting sort by pixel */
    uint32_t *cnt = (uint32_t *)calloc((size_t)P + 1, sizeof(uint32_t));
    rec_t *sorted = (rec_t *)malloc((n ? n : 1) * sizeof(rec_t));
    if (!cnt || !sorted) {
        free(cnt);
        free(sorted);
        return FO_ENOMEM;
    }
    for (size_t k = 0; k < n; k++) cnt[X->recs.r[k].pix + 1]++;
    for (uint32_t q = 0; q < P; q++) cnt[q + 1] += cnt[q];
    uint32_t *fp = (uint32_t *)malloc(((size_t)P + 1) * sizeof(uint32_t));
    if (!fp) {
        free(cnt);
        free(sorted);
        return FO_ENOMEM;
    }
    memcpy(fp, cnt, ((size_t)P + 1) * sizeof(uint32_t));
    for (size_t k = 0; k < n; k++) sorted[fp[X->recs.r[k].pix]++] = X->recs.r[k];
    free(fp);
    /* at most one sequence per record pair plus one per pixel */
    size_t cap = n + 2;
    R->seq = (uint32_t *)malloc(cap * 2 * sizeof(uint32_t));
    if (!R->seq) {
        free(cnt);
        free(sorted);
        return FO_ENOMEM;
    }
    uint32_t idx = 0;
    int err = FO_OK;
#define ADD_EDGE(s, e)                               \
    do {                                             \
        int s_ = (s), e_ = (e);                      \
        if (!(e_ - s_ + 1 > 0)) err = FO_EASSERT;    \
        R->seq[2 * idx] = (uint32_t)s_;              \
        R->seq[2 * idx + 1] = (uint32_t)(e_ - s_ + 1); \
        idx++;                                       \
    } while (0)
    rec_t tmp[2];
    for (uint32_t pix = 0; pix < P && !err; pix++) {
        uint32_t b = cnt[pix], e = cnt[pix + 1];
        if (e == b) continue;
        size_t sz = e - b;
        rec_t *L = sorted + b;
        /* odd count: append the opposite of the last (Ideal.cpp:102-105) */
        int odd = (sz % 2 == 1);
        rec_t extra;
        if (odd) {
            extra.type = (uint8_t)!L[sz - 1].type;
            extra.edge = L[sz - 1].edge;
            extra.pix = pix;
        }
        (void)tmp;
        size_t tot = sz + (odd ? 1 : 0);
#define AT(k) ((k) < sz ? L[(k)] : extra)
        int start = 0, end = (int)tot - 1;
        R->offset[pix] = idx;
        if (AT(0).type == LEAVE) {
            if (AT((size_t)end).type != ENTER) err = FO_EASSERT;
            ADD_EDGE(0, AT(0).edge);
            ADD_EDGE(AT((size_t)end).edge, (int)X->nv - 2);
            start++;
            end--;
        }
        for (int i = start; i <= end; i++) {
            if (AT((size_t)i).type != ENTER) err = FO_EASSERT;
            if (i == end || AT((size_t)i + 1).type == ENTER) {
                ADD_EDGE(AT((size_t)i).edge, AT((size_t)i).edge);
            } else {
                ADD_EDGE(AT((size_t)i).edge, AT((size_t)i + 1).edge);
                i++;
            }
        }
#undef AT
    }
#undef ADD_EDGE
    R->n_seq = idx;
    free(cnt);
    free(sorted);
    return err;
}

/* MyRaster.cpp:8-33 */
static void init_raster(fo_raster *R, int num_pixels) {
    const double *m = R->mbr;
    double multi = fabs((m[3] - m[1]) / (m[2] - m[0]));
    R->dimx = (int)pow(num_pixels / multi, 0.5);
    R->dimy = (int)(R->dimx * multi);
    if (R->dimx == 0) R->dimx = 1;
    if (R->dimy == 0) R->dimy = 1;
    R->step_x = (m[2] - m[0]) / R->dimx;
    R->step_y = (m[3] - m[1]) / R->dimy;
    if (R->step_x < 0.00001) {
        R->step_x = 0.00001;
        R->dimx = (int)((m[2] - m[0]) / R->step_x + 1);
    }
    if (R->step_y < 0.00001) {
        R->step_y = 0.00001;
        R->dimy = (int)((m[3] - m[1]) / R->step_y + 1);
    }
}

/* MyRaster.cpp:444-491 with UniversalGrid::configure(25) (UniversalGrid.h:29-35) */
static int grid_align(fo_raster *R, double extent) {
    int max_layers = 25;
    double gstep = round_sig((extent > 0 ? extent : 360.0) / pow(2, max_layers), 2);
    int flag1 = 0, flag2 = 0;
    double x = gstep, y = gstep;
    if (R->step_x <= x) { R->step_x = x; flag1 = 1; }
    if (R->step_y <= y) { R->step_y = y; flag2 = 1; }
    for (int i = max_layers; i > 0; i--) {
        if (!flag1 && R->step_x > x && R->step_x < x * 2) {
            flag1 = 1;
            R->step_x = fabs(R->step_x - x) < fabs(R->step_x - x * 2) ? x : x * 2;
        }
        if (!flag2 && R->step_y > y && R->step_y < y * 2) {
            flag2 = 1;
            R->step_y = fabs(R->step_y - y) < fabs(R->step_y - y * 2) ? y : y * 2;
        }
        if (flag1 && flag2) break;
        x *= 2;
        y *= 2;
    }
    if (!(flag1 && flag2)) return FO_EASSERT;
    R->step_x = R->step_x < R->step_y ? R->step_x : R->step_y;
    R->step_y = R->step_x;
    double *m = R->mbr;
    m[0] = floor(m[0] / R->step_x) * R->step_x;
    m[1] = floor(m[1] / R->step_y) * R->step_y;
    m[2] = ceil(m[2] / R->step_x) * R->step_x;
    m[3] = ceil(m[3] / R->step_y) * R->step_y;
    R->dimx = (int)round((m[2] - m[0]) / R->step_x);
    R->dimy = (int)round((m[3] - m[1]) / R->step_y);
    return FO_OK;
}

/* Ideal.cpp:1061-1099 + Hraster.cpp:3-25 */
static int layering(fo_raster *R, int NLow) {
    int high_layers = (int)ceil(fmax(log(R->dimx) / log(2.0), log(R->dimy) / log(2.0)));
    int low_layers = high_layers;
    double _dimx = R->dimx, _dimy = R->dimy;
    for (int i = high_layers - 1; i >= 0; i--) {
        if (_dimx * _dimy <= NLow) break;
        _dimx = (int)ceil(_dimx / 2.0);
        _dimy = (int)ceil(_dimy / 2.0);
        low_layers--;
    }
    R->num_layers = (uint32_t)(high_layers - low_layers + 1);
    R->layers = (fo_layer *)calloc(R->num_layers, sizeof(fo_layer));
    if (!R->layers) return FO_ENOMEM;
    uint32_t L = R->num_layers;
    fo_layer *ly = R->layers;
    memcpy(ly[L - 1].mbr, R->mbr, sizeof R->mbr);
    ly[L - 1].dimx = R->dimx;
    ly[L - 1].dimy = R->dimy;
    ly[L - 1].step_x = R->step_x;
    ly[L - 1].step_y = R->step_y;
    ly[L - 1].offset = 0;
    uint32_t status_size = (uint32_t)R->dimx * (uint32_t)R->dimy;
    for (int i = (int)L - 2; i >= 0; i--) {
        double sx = ly[i + 1].step_x * 2, sy = ly[i + 1].step_y * 2;
        fo_layer *c = &ly[i];
        c->step_x = sx;
        c->step_y = sy;
        memcpy(c->mbr, R->mbr, sizeof R->mbr);
        c->mbr[0] = floor(c->mbr[0] / sx) * sx;
        c->mbr[1] = floor(c->mbr[1] / sy) * sy;
        c->mbr[2] = ceil(c->mbr[2] / sx) * sx;
        c->mbr[3] = ceil(c->mbr[3] / sy) * sy;
        c->dimx = (int)round((c->mbr[2] - c->mbr[0]) / sx);
        c->dimy = (int)round((c->mbr[3] - c->mbr[1]) / sy);
        c->offset = status_size;
        status_size += (uint32_t)(c->dimx * c->dimy);
    }
    R->status_size = status_size;
    return FO_OK;
}

/* ---- fill ratios: Ideal.cpp:575-918 ------------------------------------ */

typedef struct {
    pt *v;
    size_t n, cap;
} ptv_t;
static int ptv_push(ptv_t *a, pt p) {
    if (a->n == a->cap) {
        size_t nc = a->cap ? a->cap * 2 : 32;
        pt *nv = (pt *)realloc(a->v, nc * sizeof(pt));
        if (!nv) return FO_ENOMEM;
        a->v = nv;
        a->cap = nc;
    }
    a->v[a->n++] = p;
    return FO_OK;
}
/* MyPolygon.h:49-58: append unless an equal point is already present */
static int ptv_add_unique(ptv_t *a, pt p) {
    for (size_t k = 0; k < a->n; k++)
        if (pt_eq(a->v[k], p)) return FO_OK;
    return ptv_push(a, p);
}

/* geometry_computation.h:28-43 */
static int in_h(double Yi, double Yi1, double py) { return !(py < Yi || py > Yi1); }
static int in_v(double Xi, double Xi1, double px) { return !(px < Xi || px > Xi1); }

static pt mkpt(double x, double y) {
    pt r;
    r.x = (float)x;
    r.y = (float)y;
    return r;
}

/* Ideal.cpp:575-678 */
static int clip_x(const pt *ring, uint32_t nv, double Xi, double Xi1, ptv_t *out) {
    out->n = 0;
    for (uint32_t itV = 0; itV + 1 < nv; itV++) {
        pt A = ring[itV], B = ring[itV + 1];
        double yi, yi1;
        if (A.x == B.x) {
            yi = A.y < B.y ? A.y : B.y;
            yi1 = yi;
        } else {
            double slope = ((double)B.y - A.y) / (B.x - A.x); /* getSlope: x difference in float */
            yi = slope * (Xi - B.x) + B.y;
            yi1 = slope * (Xi1 - B.x) + B.y;
        }
        pt pi = mkpt(Xi, yi), pi1 = mkpt(Xi1, yi1);
        if (in_v(Xi, Xi1, A.x) && ptv_add_unique(out, A)) return FO_ENOMEM;
        double mny = A.y < B.y ? A.y : B.y, mxy = A.y < B.y ? B.y : A.y;
        double mnx = A.x < B.x ? A.x : B.x, mxx = A.x < B.x ? B.x : A.x;
        if (A.x < B.x) {
            if (in_h(mny, mxy, pi.y) && in_v(mnx, mxx, pi.x) && ptv_add_unique(out, pi)) return FO_ENOMEM;
            if (in_h(mny, mxy, pi1.y) && in_v(mnx, mxx, pi1.x) && ptv_add_unique(out, pi1)) return FO_ENOMEM;
        } else {
            if (in_h(mny, mxy, pi1.y) && in_v(mnx, mxx, pi1.x) && ptv_add_unique(out, pi1)) return FO_ENOMEM;
            if (in_h(mny, mxy, pi.y) && in_v(mnx, mxx, pi.x) && ptv_add_unique(out, pi)) return FO_ENOMEM;
        }
        if (in_v(Xi, Xi1, B.x) && ptv_add_unique(out, B)) return FO_ENOMEM;
    }
    if (out->n != 0 && ptv_push(out, out->v[0])) return FO_ENOMEM;
    return FO_OK;
}

/* Ideal.cpp:680-818 */
static int clip_y(const ptv_t *in, double Yi, double Yi1, ptv_t *out) {
    out->n = 0;
    for (size_t k = 0; k + 1 < in->n; k++) {
        pt A = in->v[k], B = in->v[k + 1];
        int parallels = 0;
        double xi = 0, xi1 = 0;
        if (A.x == B.x) {
            xi = A.x;
            xi1 = A.x;
        } else {
            double slope = ((double)B.y - A.y) / (B.x - A.x);
            if (A.y == B.y) {
                if (A.y == Yi) {
                    xi = A.x;
                    xi1 = -INFINITY; /* -DBL_MAX converted to float */
                } else if (A.y == Yi1) {
                    xi = -INFINITY;
                    xi1 = A.x;
                } else {
                    parallels = 1;
                }
            } else {
                xi = ((Yi - B.y) / slope) + B.x;
                xi1 = ((Yi1 - B.y) / slope) + B.x;
            }
        }
        if (in_h(Yi, Yi1, A.y) && ptv_push(out, A)) return FO_ENOMEM;
        if (!parallels) {
            pt pi = mkpt(xi, Yi), pi1 = mkpt(xi1, Yi1);
            double mny = A.y < B.y ? A.y : B.y, mxy = A.y < B.y ? B.y : A.y;
            double mnx = A.x < B.x ? A.x : B.x, mxx = A.x < B.x ? B.x : A.x;
            if (A.y < B.y) {
                if (in_v(mnx, mxx, pi.x) && in_h(mny, mxy, pi.y) && ptv_push(out, pi)) return FO_ENOMEM;
                if (in_v(mnx, mxx, pi1.x) && in_h(mny, mxy, pi1.y) && ptv_push(out, pi1)) return FO_ENOMEM;
            } else {
                if (in_v(mnx, mxx, pi1.x) && in_h(mny, mxy, pi1.y) && ptv_push(out, pi1)) return FO_ENOMEM;
                if (in_v(mnx, mxx, pi.x) && in_h(mny, mxy, pi.y) && ptv_push(out, pi)) return FO_ENOMEM;
            }
        }
    }
    if (out->n != 0 && pt_ne(out->v[0], out->v[out->n - 1]) && ptv_push(out, out->v[0])) return FO_ENOMEM;
    return FO_OK;
}

/* geometry_computation.h:275-297 */
static double polygon_area(const ptv_t *p) {
    size_t n = p->n;
    if (n < 3) return 0.0;
    double area = 0.0;
    for (size_t i = 0; i + 1 < n; i++) {
        pt p1 = p->v[i], p2 = p->v[i + 1];
        area += ((double)p1.x * p2.y - (double)p2.x * p1.y);
    }
    return fabs(area) / 2.0;
}

/* geometry_computation.h:299-321 / Ideal.cpp:64-88 */
static int classify(double area, double pixelArea, int count) {
    double ratio = area / pixelArea;
    if (fabs(ratio - 1.0) < 1e-9) return count - 1;
    if (fabs(ratio) < 1e-9) return 0;
    int idx = (int)ceil(ratio * (count - 2));
    if (idx >= count) idx = count - 1;
    return idx;
}

/* Ideal.cpp:820-918 */
static int calculate_fullness(rctx *X) {
    fo_raster *R = X->R;
    int cc = X->cc;
    double Xi = R->mbr[0];
    double Xi1 = Xi + R->step_x;
    double kx = Xi + R->dimx * R->step_x;
    ptv_t col = {0}, cell = {0};
    int err = FO_OK;
    int x = 0;
    double pixel_area = R->step_x * R->step_y;
    while (Xi1 < kx + 1e-9 && !err) {
        err = clip_x(X->p, X->nv, Xi, Xi1, &col);
        if (err) break;
        if (col.n > 0) {
            double ky = R->mbr[1] + R->dimy * R->step_y;
            double Yi = R->mbr[1];
            double Yi1 = Yi + R->step_y;
            int y = 0;
            while (Yi1 < ky + 1e-9) {
                err = clip_y(&col, Yi, Yi1, &cell);
                if (err) break;
                double a = polygon_area(&cell);
                int type = classify(a, pixel_area, cc);
                if (x >= R->dimx || y >= R->dimy) {
                    err = FO_EASSERT;
                    break;
                }
                int id = y * R->dimx + x;
                if (R->status[id] == 1) {
                    int t = type < cc - 2 ? type : cc - 2;
                    R->status[id] = (uint8_t)(t > 1 ? t : 1);
                    R->areas[id] = a;
                } else if (R->status[id] == 2) {
                    R->status[id] = (uint8_t)(cc - 1);
                    R->areas[id] = pixel_area;
                } else {
                    R->status[id] = 0;
                    R->areas[id] = 0.0;
                }
                Yi += R->step_y;
                Yi1 = Yi + R->step_y;
                y++;
            }
        }
        Xi += R->step_x;
        Xi1 = Xi + R->step_x;
        x++;
    }
    free(col.v);
    free(cell.v);
    return err;
}

/* MyRaster.cpp:188-200 for an arbitrary layer geometry */
static int off_x(const double *mbr, double step, int dim, double v) {
    int x = double_to_int((v - mbr[0]) / step);
    if (x < 0) x = 0;
    if (x > dim - 1) x = dim - 1;
    return x;
}
static int off_y(const double *mbr, double step, int dim, double v) {
    int y = double_to_int((v - mbr[1]) / step);
    if (y < 0) y = 0;
    if (y > dim - 1) y = dim - 1;
    return y;
}

/* Ideal.cpp:1008-1059. merge_area's status argument is left uninitialised by
 * merge_status; the compiled reference keeps the previous pixel's value in it
 * (merge_carry = 1) — see the harness comparison in the tests. */
static int merge_layers(fo_raster *R, int cc, int merge_carry) {
    uint32_t L = R->num_layers;
    for (int li = (int)L - 2; li >= 0; li--) {
        fo_layer *c = &R->layers[li];
        int st = 0; /* OUT */
        for (int x = 0; x < c->dimx; x++) {
            for (int y = 0; y < c->dimy; y++) {
                if (!merge_carry) st = 0;
                double lowx = c->mbr[0] + x * c->step_x;
                double lowy = c->mbr[1] + y * c->step_y;
                double highx = c->mbr[0] + (x + 1) * c->step_x;
                double highy = c->mbr[1] + (y + 1) * c->step_y;
                int start_x = off_x(R->mbr, R->step_x, R->dimx, lowx);
                int start_y = off_y(R->mbr, R->step_y, R->dimy, lowy);
                int end_x = off_x(R->mbr, R->step_x, R->dimx, highx) - 1;
                int end_y = off_y(R->mbr, R->step_y, R->dimy, highy) - 1;
                if (!(start_x >= 0 && start_y >= 0 && end_x < R->dimx && end_y < R->dimy)) return FO_EASSERT;
                if (end_y < start_y) end_y = start_y;
                if (end_x < start_x) end_x = start_x;
                double area = 0.0;
                for (int i = start_x; i <= end_x; i++)
                    for (int j = start_y; j <= end_y; j++) {
                        int id = j * R->dimx + i;
                        if (show_status_cc(R->status[id], cc) == 1) st = 1;
                        area += R->areas[id];
                    }
                if (st != 1) st = show_status_cc(R->status[start_y * R->dimx + start_x], cc);
                uint8_t full;
                if (st == 1)
                    full = (uint8_t)classify(area, c->step_x * c->step_y, cc);
                else if (st == 2)
                    full = (uint8_t)(cc - 1);
                else
                    full = 0;
                R->status[c->offset + (uint32_t)(y * c->dimx + x)] = full;
            }
        }
    }
    return FO_OK;
}

void fo_raster_free(fo_raster *r) {
    if (!r) return;
    free(r->status);
    free(r->offset);
    free(r->seq);
    free(r->hoff);
    free(r->hnodes);
    free(r->voff);
    free(r->vnodes);
    free(r->areas);
    free(r->layers);
    memset(r, 0, sizeof *r);
}

int fo_rasterize(const float *ring, uint32_t nv, const fo_opts *o, fo_raster *R) {
    memset(R, 0, sizeof *R);
    if (!ring || nv < 3 || !o || o->vpr <= 0) return FO_EINVAL;
    const pt *p = (const pt *)ring;
    int cc = o->category_count ? o->category_count : 16;
    /* vertex_sequence.cpp:152-168 */
    double lx = 100000.0, ly = 100000.0, hx = -100000.0, hy = -100000.0;
    for (uint32_t i = 0; i < nv; i++) {
        double x = p[i].x, y = p[i].y;
        lx = lx < x ? lx : x;
        hx = hx > x ? hx : x;
        ly = ly < y ? ly : y;
        hy = hy > y ? hy : y;
    }
    float bias = 1e-9f;
    R->mbr[0] = lx - bias;
    R->mbr[1] = ly - bias;
    R->mbr[2] = hx + bias;
    R->mbr[3] = hy + bias;
    R->nv = nv;
    /* preprocessing.cpp:15-21 */
    init_raster(R, (int)(nv / (uint32_t)o->vpr));
    int err = FO_OK;
    if (o->hierarchy) {
        err = grid_align(R, o->grid_extent);
        if (!err) err = layering(R, 1);
    } else {
        R->status_size = (uint32_t)R->dimx * (uint32_t)R->dimy;
    }
    if (err) return err;
    R->P = (uint32_t)R->dimx * (uint32_t)R->dimy;
    /* Ideal.cpp:240-250 */
    R->status = (uint8_t *)calloc(R->status_size ? R->status_size : 1, 1);
    R->areas = (double *)calloc(R->P ? R->P : 1, sizeof(double));
    R->offset = (uint32_t *)calloc((size_t)R->P + 1, sizeof(uint32_t));
    if (!R->status || !R->areas || !R->offset) {
        fo_raster_free(R);
        return FO_ENOMEM;
    }
    rctx X;
    memset(&X, 0, sizeof X);
    X.R = R;
    X.p = p;
    X.nv = nv;
    X.cc = cc;
    evaluate_edges(&X);
    err = X.err;
    if (!err) {
        if (X.recs.n == 0 && nv > 0) {
            /* Ideal.cpp:523-528: the whole ring inside one pixel */
            R->seq = (uint32_t *)malloc(2 * sizeof(uint32_t));
            if (!R->seq) err = FO_ENOMEM;
            else {
                R->n_seq = 1;
                R->offset[0] = 0;
                R->seq[0] = 0;
                R->seq[1] = nv; /* add_edge(0, 0, nv - 1) */
            }
        } else {
            err = process_crosses(&X);
        }
    }
    if (!err) err = build_lines(&X.hn, (uint32_t)R->dimy, 0, &R->hoff, &R->hnodes, &R->n_hnodes);
    if (!err) err = build_lines(&X.vn, (uint32_t)R->dimx, 1, &R->voff, &R->vnodes, &R->n_vnodes);
    R->n_hlines = (uint32_t)R->dimy + 2;
    R->n_vlines = (uint32_t)R->dimx + 2;
    free(X.recs.r);
    free(X.hn.r);
    free(X.vn.r);
    if (err) {
        fo_raster_free(R);
        return err;
    }
    /* Ideal.cpp:35-45 */
    R->offset[R->P] = R->n_seq;
    for (int i = (int)R->P - 1; i >= 0; i--)
        if (show_status_cc(R->status[i], cc) != 1) R->offset[i] = R->offset[i + 1];
    /* Ideal.cpp:540-573 */
    {
        const double start_x = R->mbr[0];
        for (int y = 1; y < R->dimy; y++) {
            int isin = 0;
            uint32_t i = R->hoff[y], j = R->hoff[y + 1];
            for (int x = 0; x < R->dimx; x++) {
                int id = y * R->dimx + x;
                if (show_status_cc(R->status[id], cc) != 1) {
                    R->status[id] = isin ? 2 : 0;
                    continue;
                }
                int pass = 0;
                while (i < j && R->hnodes[i] <= start_x + R->step_x * (x + 1)) {
                    pass++;
                    i++;
                }
                if (pass % 2 == 1) isin = !isin;
            }
        }
    }
    X.err = 0;
    err = calculate_fullness(&X);
    if (!err && o->hierarchy) err = merge_layers(R, cc, o->merge_carry);
    if (err) {
        fo_raster_free(R);
        return err;
    }
    return FO_OK;
}

/* ---------------------------------------------------------- queries ----- */

static int rs_show(const fo_raster *r, uint32_t id, int cc) { return show_status_cc(r->status[id], cc); }

/* MyRaster.cpp:332-346, iterating x outer, y inner */
typedef struct {
    int sx, ex, sy, ey;
} window_t;
static window_t retrieve(const double *mbr, double stx, double sty, int dimx, int dimy, const double *b) {
    window_t w;
    w.sx = off_x(mbr, stx, dimx, b[0] + 1e-6);
    w.sy = off_y(mbr, sty, dimy, b[1] + 1e-6);
    w.ex = off_x(mbr, stx, dimx, b[2] - 1e-6);
    w.ey = off_y(mbr, sty, dimy, b[3] - 1e-6);
    return w;
}

/* Ideal.cpp:47-62 */
static double decode_area(const fo_raster *r, uint32_t id, int isLow, int cc) {
    uint8_t f = r->status[id];
    double pa = r->step_x * r->step_y;
    if (f == 0) return 0.0f;
    if (f == cc - 1) return pa;
    return (1.0 * f - isLow) / (cc - 2) * pa;
}

typedef struct {
    double prob;
    int pa, pb;
} cand_t;
static int cand_desc(const void *a, const void *b) {
    const cand_t *x = (const cand_t *)a, *y = (const cand_t *)b;
    /* tuple comparison a > b sorts descending */
    if (x->prob != y->prob) return x->prob > y->prob ? -1 : 1;
    if (x->pa != y->pa) return x->pa > y->pa ? -1 : 1;
    if (x->pb != y->pb) return x->pb > y->pb ? -1 : 1;
    return 0;
}

static uint32_t nseq(const fo_raster *r, uint32_t id, int cc) {
    if (rs_show(r, id, cc) != 1) return 0;
    return r->offset[id + 1] - r->offset[id];
}

/* geometry_computation.h:224-237, counting the tests performed */
static int batch_intersect(const pt *p1, const pt *p2, int s1, int s2, uint64_t *tests) {
    for (int i = 0; i < s1; i++)
        for (int j = 0; j < s2; j++) {
            if (tests) (*tests)++;
            if (seg_intersect(p1[i], p1[i + 1], p2[j], p2[j + 1])) return 1;
        }
    return 0;
}

int fo_intersect(const fo_raster *s, const float *sring, const fo_raster *t, const float *tring, fo_counters *c) {
    const int cc = 16;
    fo_counters local = {0};
    if (!c) c = &local;
    memset(c, 0, sizeof *c);
    const pt *sp = (const pt *)sring, *tp = (const pt *)tring;
    window_t w = retrieve(s->mbr, s->step_x, s->step_y, s->dimx, s->dimy, t->mbr);
    cand_t *cand = NULL;
    size_t nc = 0, cap = 0;
    double spa = s->step_x * s->step_y, tpa = t->step_x * t->step_y;
    double maxpa = spa > tpa ? spa : tpa;
    for (int i = w.sx; i <= w.ex; i++)
        for (int j = w.sy; j <= w.ey; j++) {
            uint32_t pa = (uint32_t)(j * s->dimx + i);
            c->window_pixels++;
            if (rs_show(s, pa, cc) == 0) continue;
            double bx[4] = {s->mbr[0] + i * s->step_x, s->mbr[1] + j * s->step_y, s->mbr[0] + (i + 1) * s->step_x,
                            s->mbr[1] + (j + 1) * s->step_y};
            window_t tw = retrieve(t->mbr, t->step_x, t->step_y, t->dimx, t->dimy, bx);
            for (int u = tw.sx; u <= tw.ex; u++)
                for (int v = tw.sy; v <= tw.ey; v++) {
                    uint32_t pb = (uint32_t)(v * t->dimx + u);
                    if (rs_show(t, pb, cc) == 0) continue;
                    c->pixel_pairs++;
                    if (rs_show(s, pa, cc) == 2 || rs_show(t, pb, cc) == 2) {
                        free(cand);
                        return 1;
                    }
                    double s_apx = (decode_area(s, pa, 1, cc) + decode_area(s, pa, 0, cc)) / 2;
                    double t_apx = (decode_area(t, pb, 1, cc) + decode_area(t, pb, 0, cc)) / 2;
                    double prob = (s_apx + t_apx) / maxpa;
                    if (nc == cap) {
                        cap = cap ? cap * 2 : 64;
                        cand_t *nn = (cand_t *)realloc(cand, cap * sizeof(cand_t));
                        if (!nn) {
                            free(cand);
                            return FO_ENOMEM;
                        }
                        cand = nn;
                    }
                    cand[nc].prob = prob;
                    cand[nc].pa = (int)pa;
                    cand[nc].pb = (int)pb;
                    nc++;
                }
        }
    if (nc) qsort(cand, nc, sizeof(cand_t), cand_desc);
    for (size_t k = 0; k < nc; k++) {
        uint32_t pa = (uint32_t)cand[k].pa, pb = (uint32_t)cand[k].pb;
        uint32_t na = nseq(s, pa, cc), nb = nseq(t, pb, cc);
        for (uint32_t i = 0; i < na; i++) {
            const uint32_t *r = s->seq + 2 * (s->offset[pa] + i);
            for (uint32_t j = 0; j < nb; j++) {
                const uint32_t *r2 = t->seq + 2 * (t->offset[pb] + j);
                c->seq_pairs++;
                if (batch_intersect(sp + r[0], tp + r2[0], (int)r[1], (int)r2[1], &c->segment_tests)) {
                    free(cand);
                    return 1;
                }
            }
        }
    }
    free(cand);
    return 0;
}

/* The reference's "-a" intersect heuristic (query_intersect.cu:32-134, the
 * GPU path with use_approximation): an IN pixel overlapping a non-OUT pixel
 * decides "true", as does any BORDER x BORDER pixel pair whose fill
 * probability (mean decoded fill of both pixels over the larger pixel area)
 * exceeds 1; no segment is tested. */
int fo_intersect_heuristic(const fo_raster *s, const fo_raster *t) {
    const int cc = 16;
    window_t w = retrieve(s->mbr, s->step_x, s->step_y, s->dimx, s->dimy, t->mbr);
    double spa = s->step_x * s->step_y, tpa = t->step_x * t->step_y;
    double maxpa = spa > tpa ? spa : tpa;
    for (int i = w.sx; i <= w.ex; i++)
        for (int j = w.sy; j <= w.ey; j++) {
            uint32_t pa = (uint32_t)(j * s->dimx + i);
            if (rs_show(s, pa, cc) == 0) continue;
            double bx[4] = {s->mbr[0] + i * s->step_x, s->mbr[1] + j * s->step_y, s->mbr[0] + (i + 1) * s->step_x,
                            s->mbr[1] + (j + 1) * s->step_y};
            window_t tw = retrieve(t->mbr, t->step_x, t->step_y, t->dimx, t->dimy, bx);
            for (int u = tw.sx; u <= tw.ex; u++)
                for (int v = tw.sy; v <= tw.ey; v++) {
                    uint32_t pb = (uint32_t)(v * t->dimx + u);
                    if (rs_show(t, pb, cc) == 0) continue;
                    if (rs_show(s, pa, cc) == 2 || rs_show(t, pb, cc) == 2) return 1;
                    double s_apx = (decode_area(s, pa, 1, cc) + decode_area(s, pa, 0, cc)) / 2;
                    double t_apx = (decode_area(t, pb, 1, cc) + decode_area(t, pb, 0, cc)) / 2;
                    if ((s_apx + t_apx) / maxpa > 1.0) return 1;
                }
        }
    return 0;
}

/* Box.cpp:90-118 */
static double box_distance(const double *a, const double *t, int geography) {
    if (!(t[0] > a[2] || t[2] < a[0] || t[1] > a[3] || t[3] < a[1])) return 0;
    double dx = 0, dy = 0;
    if (t[1] > a[3])
        dy = t[1] - a[3];
    else if (t[3] < a[1])
        dy = a[1] - t[3];
    else
        dy = 0;
    if (t[0] > a[2])
        dx = t[0] - a[2];
    else if (t[2] < a[0])
        dx = a[0] - t[2];
    else
        dx = 0;
    if (geography) {
        dy = dy / k_deg_lat;
        dx = dx / fo_degree_per_km_longitude(a[1]);
    }
    return sqrt(dx * dx + dy * dy);
}

/* Box.cpp:120-149: corners converted to float points first */
static double box_max_distance(const double *a, const double *t, int geography) {
    pt v1[4] = {mkpt(a[0], a[1]), mkpt(a[0], a[3]), mkpt(a[2], a[1]), mkpt(a[2], a[3])};
    pt v2[4] = {mkpt(t[0], t[1]), mkpt(t[0], t[3]), mkpt(t[2], t[1]), mkpt(t[2], t[3])};
    double md = 0.0;
    double dlon = geography ? fo_degree_per_km_longitude(a[1]) : 1.0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double dx = (float)(v1[i].x - v2[j].x);
            double dy = (float)(v1[i].y - v2[j].y);
            if (geography) {
                dy = dy / k_deg_lat;
                dx = dx / dlon;
            }
            double d = sqrt(dx * dx + dy * dy);
            md = md > d ? md : d;
        }
    return md;
}

static void layer_box(const fo_layer *l, int id, double *b) {
    int x = id % l->dimx, y = id / l->dimx;
    b[0] = l->mbr[0] + x * l->step_x;
    b[1] = l->mbr[1] + y * l->step_y;
    b[2] = l->mbr[0] + (x + 1) * l->step_x;
    b[3] = l->mbr[1] + (y + 1) * l->step_y;
}

typedef struct {
    int *v;
    size_t n, cap;
} iv_t;
static int iv_push(iv_t *a, int x) {
    if (a->n == a->cap) {
        size_t nc = a->cap ? a->cap * 2 : 64;
        int *nv = (int *)realloc(a->v, nc * sizeof(int));
        if (!nv) return FO_ENOMEM;
        a->v = nv;
        a->cap = nc;
    }
    a->v[a->n++] = x;
    return FO_OK;
}
static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return x < y ? -1 : (x > y);
}
static void iv_unique(iv_t *a) {
    if (!a->n) return;
    qsort(a->v, a->n, sizeof(int), cmp_int);
    size_t k = 1;
    for (size_t i = 1; i < a->n; i++)
        if (a->v[i] != a->v[k - 1]) a->v[k++] = a->v[i];
    a->n = k;
}

typedef struct {
    double apx, lo, hi;
    int id1, id2;
} wcand_t;
static int wcand_cmp(const void *a, const void *b) {
    const wcand_t *x = (const wcand_t *)a, *y = (const wcand_t *)b;
    if (x->apx != y->apx) return x->apx < y->apx ? -1 : 1;
    if (x->lo != y->lo) return x->lo < y->lo ? -1 : 1;
    if (x->hi != y->hi) return x->hi < y->hi ? -1 : 1;
    if (x->id1 != y->id1) return x->id1 < y->id1 ? -1 : 1;
    if (x->id2 != y->id2) return x->id2 < y->id2 ? -1 : 1;
    return 0;
}

static uint8_t layer_status(const fo_raster *r, uint32_t li, int id) { return r->status[r->layers[li].offset + (uint32_t)id]; }

/* The hierarchical descent of Ideal::within (Ideal.cpp:2478-2584): 1 or 0
 * when it decides the pair, 2 with the finest surviving pixel pairs left in
 * qa / qb (caller frees), or FO_ENOMEM. */
static int within_descend(const fo_raster *s, const fo_raster *t, double distance, int geography, iv_t *qa_out,
                          iv_t *qb_out) {
    const int cc = 16;
    uint32_t s_level = s->num_layers - 1, t_level = t->num_layers - 1;
    /* queue of pixel pairs, as two parallel arrays */
    iv_t qa = {0}, qb = {0};
    int err = 0, result = -1;
    {
        const fo_layer *l0 = &s->layers[0], *m0 = &t->layers[0];
        for (int i = 0; i < l0->dimx * l0->dimy && !err; i++)
            for (int j = 0; j < m0->dimx * m0->dimy && !err; j++) {
                err |= iv_push(&qa, i);
                err |= iv_push(&qb, j);
            }
    }
    uint32_t i = 0, j = 0;
    iv_t sp_set = {0}, tp_set = {0};
    while (!err && result < 0) {
        sp_set.n = 0;
        tp_set.n = 0;
        int s_next = 0, t_next = 0;
        double s_step = s->layers[i].step_x, t_step = t->layers[j].step_x;
        if (i < s_level && (s_step >= t_step || j >= t_level)) {
            i++;
            s_next = 1;
        }
        if (j < t_level && (s_step <= t_step || i >= s_level)) {
            j++;
            t_next = 1;
        }
        size_t size = qa.n;
        if (size == 0) break;
        for (size_t k = 0; k < size && !err; k++) {
            int sid = qa.v[k], tid = qb.v[k];
            if (s_next) {
                double b[4];
                layer_box(&s->layers[i - 1], sid, b);
                b[0] += 1e-6;
                b[1] += 1e-6;
                b[2] -= 1e-6;
                b[3] -= 1e-6;
                const fo_layer *L = &s->layers[i];
                window_t w = retrieve(L->mbr, L->step_x, L->step_y, L->dimx, L->dimy, b);
                for (int x = w.sx; x <= w.ex; x++)
                    for (int y = w.sy; y <= w.ey; y++) {
                        int id = y * L->dimx + x;
                        if (show_status_cc(layer_status(s, i, id), cc) == 1) err |= iv_push(&sp_set, id);
                    }
            } else if (show_status_cc(layer_status(s, i, sid), cc) == 1) {
                err |= iv_push(&sp_set, sid);
            }
            if (t_next) {
                double b[4];
                layer_box(&t->layers[j - 1], tid, b);
                b[0] += 1e-6;
                b[1] += 1e-6;
                b[2] -= 1e-6;
                b[3] -= 1e-6;
                const fo_layer *L = &t->layers[j];
                window_t w = retrieve(L->mbr, L->step_x, L->step_y, L->dimx, L->dimy, b);
                for (int x = w.sx; x <= w.ex; x++)
                    for (int y = w.sy; y <= w.ey; y++) {
                        int id = y * L->dimx + x;
                        if (show_status_cc(layer_status(t, j, id), cc) == 1) err |= iv_push(&tp_set, id);
                    }
            } else if (show_status_cc(layer_status(t, j, tid), cc) == 1) {
                err |= iv_push(&tp_set, tid);
            }
        }
        if (err) break;
        iv_unique(&sp_set);
        iv_unique(&tp_set);
        qa.n = 0;
        qb.n = 0;
        double max_box_dist = 100000.0;
        for (size_t a = 0; a < sp_set.n && result < 0; a++) {
            double b1[4];
            layer_box(&s->layers[i], sp_set.v[a], b1);
            for (size_t b = 0; b < tp_set.n; b++) {
                double b2[4];
                layer_box(&t->layers[j], tp_set.v[b], b2);
                double md = box_max_distance(b1, b2, geography);
                if (md <= distance) {
                    result = 1;
                    break;
                }
                max_box_dist = max_box_dist < md ? max_box_dist : md;
            }
        }
        if (result >= 0) break;
        for (size_t a = 0; a < sp_set.n && !err; a++) {
            double b1[4];
            layer_box(&s->layers[i], sp_set.v[a], b1);
            for (size_t b = 0; b < tp_set.n && !err; b++) {
                double b2[4];
                layer_box(&t->layers[j], tp_set.v[b], b2);
                double mind = box_distance(b1, b2, geography);
                if (mind > distance) continue;
                if (mind < max_box_dist) {
                    err |= iv_push(&qa, sp_set.v[a]);
                    err |= iv_push(&qb, tp_set.v[b]);
                }
            }
        }
        if (!s_next && !t_next) break;
    }
    free(sp_set.v);
    free(tp_set.v);
    if (err || result >= 0) {
        free(qa.v);
        free(qb.v);
        return err ? FO_ENOMEM : result;
    }
    *qa_out = qa;
    *qb_out = qb;
    return 2;
}

/* Ideal.cpp:2475-2643 */
int fo_within(const fo_raster *s, const float *sring, const fo_raster *t, const float *tring, double distance,
              int geography, fo_counters *c) {
    const int cc = 16;
    fo_counters local = {0};
    if (!c) c = &local;
    memset(c, 0, sizeof *c);
    if (!s->num_layers || !t->num_layers) return FO_EINVAL; /* the reference needs -h here */
    const pt *sp = (const pt *)sring, *tp = (const pt *)tring;
    iv_t qa = {0}, qb = {0};
    int result = within_descend(s, t, distance, geography, &qa, &qb);
    if (result != 2) return result;
    size_t nc = qa.n;
    wcand_t *cand = (wcand_t *)malloc((nc ? nc : 1) * sizeof(wcand_t));
    if (!cand) {
        free(qa.v);
        free(qb.v);
        return FO_ENOMEM;
    }
    const fo_layer *sl = &s->layers[s->num_layers - 1], *tl = &t->layers[t->num_layers - 1];
    for (size_t k = 0; k < nc; k++) {
        int id1 = qa.v[k], id2 = qb.v[k];
        int pf = classify(s->areas[id1] + t->areas[id2], s->step_x * s->step_y + t->step_x * t->step_y, 20);
        double b1[4], b2[4];
        layer_box(sl, id1, b1);
        layer_box(tl, id2, b2);
        double lo = box_distance(b1, b2, geography);
        double hi = box_max_distance(b1, b2, geography);
        cand[k].apx = lo + (double)k_mean20[pf] * (hi - lo);
        cand[k].lo = lo;
        cand[k].hi = hi;
        cand[k].id1 = id1;
        cand[k].id2 = id2;
    }
    free(qa.v);
    free(qb.v);
    c->pixel_pairs = nc;
    if (nc) qsort(cand, nc, sizeof(wcand_t), wcand_cmp);
    /* suffix minimum of the lower bounds (Ideal.cpp:2617-2621) */
    double *suffix = (double *)malloc((nc + 1) * sizeof(double));
    if (!suffix) {
        free(cand);
        return FO_ENOMEM;
    }
    suffix[nc] = 100000;
    for (size_t k = nc; k-- > 0;) suffix[k] = suffix[k + 1] < cand[k].lo ? suffix[k + 1] : cand[k].lo;
    double min_dist = 100000.0;
    result = 0;
    for (size_t k = 0; k < nc && result == 0; k++) {
        double reference_dist = suffix[k + 1];
        int id1 = cand[k].id1, id2 = cand[k].id2;
        uint32_t na = nseq(s, (uint32_t)id1, cc), nb = nseq(t, (uint32_t)id2, cc);
        int done = 0;
        for (uint32_t a = 0; a < na && !done; a++) {
            const uint32_t *e1 = s->seq + 2 * (s->offset[id1] + a);
            for (uint32_t b = 0; b < nb; b++) {
                const uint32_t *e2 = t->seq + 2 * (t->offset[id2] + b);
                if (e1[1] < 2 || e2[1] < 2) continue;
                c->seq_pairs++;
                double d = seq_within_batch(tp + e2[0], sp + e1[0], (int)e2[1], (int)e1[1], geography,
                                            &c->segment_tests);
                min_dist = min_dist < d ? min_dist : d;
                if (min_dist < distance) {
                    result = 1;
                    done = 1;
                    break;
                } else if (min_dist < reference_dist) {
                    result = 2; /* decided: false */
                    done = 1;
                    break;
                }
            }
        }
    }
    free(suffix);
    free(cand);
    return result == 1 ? 1 : 0;
}

/* The reference's within "-a" (query_within_polygon.cu:332-375, :721-742) on
 * the descent above: an undecided pair is within when one of its finest
 * surviving pixel pairs has apxDist = minDist + mean (maxDist - minDist) <=
 * distance, all in float. mean = (1.0 - pf / category_count) * 0.5 divides two
 * 8-bit integers (:352), so it is 0.5 for every pf. */
int fo_within_heuristic(const fo_raster *s, const fo_raster *t, double distance, int geography) {
    if (!s->num_layers || !t->num_layers) return FO_EINVAL;
    iv_t qa = {0}, qb = {0};
    int result = within_descend(s, t, distance, geography, &qa, &qb);
    if (result != 2) return result;
    const fo_layer *sl = &s->layers[s->num_layers - 1], *tl = &t->layers[t->num_layers - 1];
    result = 0;
    for (size_t k = 0; k < qa.n && !result; k++) {
        double b1[4], b2[4];
        layer_box(sl, qa.v[k], b1);
        layer_box(tl, qb.v[k], b2);
        const float lo = (float)box_distance(b1, b2, geography);
        const float hi = (float)box_max_distance(b1, b2, geography);
        const float apx = lo + 0.5f * (hi - lo); /* 0.5 (hi - lo) is exact: an FMA rounds the same */
        if ((double)apx <= distance) result = 1;
    }
    free(qa.v);
    free(qb.v);
    return result;
}

/* ------------------------------------------------ point in polygon ------ */

/* Ideal.cpp:988-1006 */
static int count_nodes(const fo_raster *r, int pix, float py) {
    int x = pix % r->dimx + 1;
    uint32_t i = r->voff[x], j = r->voff[x + 1];
    int count = 0;
    while (i < j && r->vnodes[i] < py) {
        count++;
        i++;
    }
    return count;
}

int fo_segment_contain(const fo_raster *r, const float *ring, float px, float py) {
    const int cc = 16;
    const pt *p = (const pt *)ring;
    int xo = off_x(r->mbr, r->step_x, r->dimx, px), yo = off_y(r->mbr, r->step_y, r->dimy, py);
    int target = yo * r->dimx + xo;
    double bx_high = r->mbr[0] + (xo + 1) * r->step_x;
    int st = rs_show(r, (uint32_t)target, cc);
    if (st == 2) return 2;
    if (st == 0) return 0;
    int ret = 0;
    pt P = {px, py};
    uint32_t ns = nseq(r, (uint32_t)target, cc);
    for (uint32_t e = 0; e < ns; e++) {
        const uint32_t *sq = r->seq + 2 * (r->offset[target] + e);
        for (uint32_t k = 0; k < sq[1]; k++) {
            pt v1 = p[sq[0] + k], v2 = p[sq[0] + k + 1];
            if (pt_eq(P, v1) || pt_eq(P, v2)) return 1;
            if ((v1.y >= P.y) != (v2.y >= P.y)) {
                const double dx = v2.x - v1.x;
                const double dy = v2.y - v1.y;
                const double py_diff = P.y - v1.y;
                if (fabs(dy) > 1e-9) {
                    const double int_x = dx * py_diff / dy + v1.x;
                    if (fabs(P.x - int_x) < 1e-9) return 1;
                    if (P.x < int_x && int_x <= bx_high) ret = !ret;
                }
            } else if (v1.y == P.y && v2.y == P.y && (v1.x >= P.x) != (v2.x >= P.x)) {
                return 1;
            }
        }
    }
    int nc = count_nodes(r, target, py);
    if (nc % 2 == 1) ret = !ret;
    return ret ? 2 : 0;
}

/* Ideal::contain(Point &) (Ideal.cpp:1101-1157): 1 when the polygon holds
 * (px, py). The MBR test is box::contain(Point) (Box.cpp:65-70); a BORDER
 * pixel flips the answer for each of its edges whose FP32 crossing abscissa
 * lies in [px, the pixel's right border], then once more when an odd number
 * of the right grid line's nodes lie below py (count_intersection_nodes,
 * Ideal.cpp:988-1006). */
int fo_contain_point(const fo_raster *r, const float *ring, float px, float py) {
    const int cc = 16;
    const pt *p = (const pt *)ring;
    if (!(px >= r->mbr[0] && px <= r->mbr[2] && py >= r->mbr[1] && py <= r->mbr[3])) return 0;
    int xo = off_x(r->mbr, r->step_x, r->dimx, px), yo = off_y(r->mbr, r->step_y, r->dimy, py);
    int target = yo * r->dimx + xo;
    double bx_high = r->mbr[0] + (xo + 1) * r->step_x;
    int st = rs_show(r, (uint32_t)target, cc);
    if (st == 2) return 1;
    if (st == 0) return 0;
    int ret = 0;
    uint32_t ns = nseq(r, (uint32_t)target, cc);
    for (uint32_t e = 0; e < ns; e++) {
        const uint32_t *sq = r->seq + 2 * (r->offset[target] + e);
        for (uint32_t k = 0; k < sq[1]; k++) {
            pt a = p[sq[0] + k], b = p[sq[0] + k + 1];
            if ((a.y >= py) != (b.y >= py)) {
                /* every operand is a float: the reference evaluates this in FP32 */
                float dx = b.x - a.x, dyp = py - a.y, dy = b.y - a.y;
                float prod = dx * dyp;
                float q = prod / dy;
                float ix = q + a.x;
                double int_x = ix;
                if (px <= int_x && int_x <= bx_high) ret = !ret;
            }
        }
    }
    if (count_nodes(r, target, py) % 2 == 1) ret = !ret;
    return ret;
}

/* Ideal::contain(Ideal *) (Ideal.cpp:1159-1231): 1 when polygon s holds
 * polygon t. t's MBR must lie in s's (box::contain(box), Box.cpp:59-64); the
 * s pixels in t's MBR window decide when all are OUT (0) or all IN (1);
 * otherwise any OUT s pixel over an IN t pixel, any t edge of a BORDER t pixel
 * crossing the border of an OUT s pixel over it, or any crossing edge pair of
 * BORDER x BORDER pixels gives 0; failing all of those, t's first vertex
 * decides. The reference returns at the first violation; every check only
 * ever returns 0, so the order of the pixel pairs cannot change the answer. */
int fo_contain(const fo_raster *s, const float *sring, const fo_raster *t, const float *tring, fo_counters *c) {
    const int cc = 16;
    fo_counters local = {0};
    if (!c) c = &local;
    memset(c, 0, sizeof *c);
    const pt *sp = (const pt *)sring, *tp = (const pt *)tring;
    if (!(t->mbr[0] >= s->mbr[0] && t->mbr[2] <= s->mbr[2] && t->mbr[1] >= s->mbr[1] && t->mbr[3] <= s->mbr[3]))
        return 0;
    window_t w = retrieve(s->mbr, s->step_x, s->step_y, s->dimx, s->dimy, t->mbr);
    long nw = (w.ex >= w.sx && w.ey >= w.sy) ? (long)(w.ex - w.sx + 1) * (w.ey - w.sy + 1) : 0;
    long etn = 0, itn = 0;
    for (int i = w.sx; i <= w.ex; i++)
        for (int j = w.sy; j <= w.ey; j++) {
            int st = rs_show(s, (uint32_t)(j * s->dimx + i), cc);
            etn += st == 0;
            itn += st == 2;
        }
    c->window_pixels = (uint64_t)nw;
    if (etn == nw) return 0;
    if (itn == nw) return 1;
    for (int i = w.sx; i <= w.ex; i++)
        for (int j = w.sy; j <= w.ey; j++) {
            uint32_t pa = (uint32_t)(j * s->dimx + i);
            int sst = rs_show(s, pa, cc);
            if (sst == 2) continue;
            double bx[4] = {s->mbr[0] + i * s->step_x, s->mbr[1] + j * s->step_y, s->mbr[0] + (i + 1) * s->step_x,
                            s->mbr[1] + (j + 1) * s->step_y};
            window_t tw = retrieve(t->mbr, t->step_x, t->step_y, t->dimx, t->dimy, bx);
            for (int u = tw.sx; u <= tw.ex; u++)
                for (int v = tw.sy; v <= tw.ey; v++) {
                    uint32_t pb = (uint32_t)(v * t->dimx + u);
                    int tst = rs_show(t, pb, cc);
                    if (sst == 0 && tst == 2) return 0;
                    if (sst == 0 && tst == 1) {
                        c->pixel_pairs++;
                        /* the pixel's border as float points, low-low, low-high, high-high, high-low, low-low */
                        pt border[5] = {{(float)bx[0], (float)bx[1]}, {(float)bx[0], (float)bx[3]},
                                        {(float)bx[2], (float)bx[3]}, {(float)bx[2], (float)bx[1]},
                                        {(float)bx[0], (float)bx[1]}};
                        uint32_t nb = nseq(t, pb, cc);
                        for (uint32_t e = 0; e < nb; e++) {
                            const uint32_t *r2 = t->seq + 2 * (t->offset[pb] + e);
                            c->seq_pairs++;
                            if (batch_intersect(tp + r2[0], border, (int)r2[1], 4, &c->segment_tests)) return 0;
                        }
                    }
                    if (sst == 1 && tst == 1) {
                        c->pixel_pairs++;
                        uint32_t na = nseq(s, pa, cc), nb = nseq(t, pb, cc);
                        for (uint32_t a = 0; a < na; a++) {
                            const uint32_t *r = s->seq + 2 * (s->offset[pa] + a);
                            for (uint32_t b = 0; b < nb; b++) {
                                const uint32_t *r2 = t->seq + 2 * (t->offset[pb] + b);
                                c->seq_pairs++;
                                if (batch_intersect(sp + r[0], tp + r2[0], (int)r[1], (int)r2[1], &c->segment_tests))
                                    return 0;
                            }
                        }
                    }
                }
        }
    return fo_contain_point(s, sring, tp[0].x, tp[0].y);
}

/* --------------------------------------------------- area oracle -------- */

/* Even-odd point in polygon, FP64 (points are float-exact in double). */
static int pip(const pt *r, uint32_t m, double x, double y) {
    int in = 0;
    for (uint32_t i = 0, j = m - 1; i < m; j = i++) {
        double yi = r[i].y, yj = r[j].y;
        if ((yi > y) != (yj > y)) {
            double xi = r[i].x, xj = r[j].x;
            double xint = xi + (y - yi) * (xj - xi) / (yj - yi);
            if (x < xint) in = !in;
        }
    }
    return in;
}

typedef struct {
    double t;
} tv_t;
static int cmp_t(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : (x > y);
}

/* Indexes over ring b that return, for a query, a superset of the edges the
 * plain loops over all of b's edges would accept, in an order that cannot
 * change the result (the crossing parameters are sorted; the point-in-polygon
 * test is a parity). They make the oracle O(edges x local density) instead
 * of O(ma x mb), so polygons of 10^5 vertices can be checked.
 *
 * slab: edges by the y-range [min, max) they span, in nslab horizontal slabs
 *   (an edge that passes the (yi > y) != (yj > y) test of pip() spans y, so
 *   it is in y's slab);
 * grid: edges by their bounding boxes widened by a margin far above the
 *   rounding of the crossing test, in g x g cells (an edge whose widened box
 *   misses a segment's box cannot pass that test). */
typedef struct {
    double x0, y0, x1, y1, cw, ch, sh;  /* extent of b, cell sizes, slab height */
    int g, nslab;
    uint32_t *cstart, *cidx; /* grid CSR */
    uint32_t *sstart, *sidx; /* slab CSR */
    uint32_t *stamp;         /* per edge of b: last query that met it */
    uint32_t tick;
} ring_index;

static void ri_free(ring_index *ix) {
    free(ix->cstart);
    free(ix->cidx);
    free(ix->sstart);
    free(ix->sidx);
    free(ix->stamp);
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static int ri_build(ring_index *ix, const pt *b, uint32_t mb) {
    memset(ix, 0, sizeof *ix);
    double x0 = b[0].x, x1 = b[0].x, y0 = b[0].y, y1 = b[0].y;
    for (uint32_t i = 1; i < mb; i++) {
        if (b[i].x < x0) x0 = b[i].x;
        if (b[i].x > x1) x1 = b[i].x;
        if (b[i].y < y0) y0 = b[i].y;
        if (b[i].y > y1) y1 = b[i].y;
    }
    const double span = (x1 - x0) + (y1 - y0) + fabs(x0) + fabs(y0) + 1.0;
    const double mg = 1e-7 * span;
    ix->x0 = x0 - mg;
    ix->y0 = y0 - mg;
    ix->x1 = x1 + mg;
    ix->y1 = y1 + mg;
    int g = (int)sqrt((double)mb / 4.0) + 1;
    if (g > 1024) g = 1024;
    ix->g = g;
    ix->nslab = g * 4;
    ix->cw = (ix->x1 - ix->x0) / g;
    ix->ch = (ix->y1 - ix->y0) / g;
    ix->sh = (ix->y1 - ix->y0) / ix->nslab;
    if (!(ix->cw > 0)) ix->cw = 1.0;
    if (!(ix->ch > 0)) ix->ch = 1.0;
    if (!(ix->sh > 0)) ix->sh = 1.0;
    size_t nc = (size_t)g * g;
    ix->cstart = (uint32_t *)calloc(nc + 1, sizeof(uint32_t));
    ix->sstart = (uint32_t *)calloc((size_t)ix->nslab + 1, sizeof(uint32_t));
    ix->stamp = (uint32_t *)calloc(mb + 1, sizeof(uint32_t));
    if (!ix->cstart || !ix->sstart || !ix->stamp) return -1;
    for (int pass = 0; pass < 2; pass++) {
        uint32_t *cfill = NULL, *sfill = NULL;
        if (pass == 1) {
            for (size_t c = 0; c < nc; c++) ix->cstart[c + 1] += ix->cstart[c];
            for (int c = 0; c < ix->nslab; c++) ix->sstart[c + 1] += ix->sstart[c];
            ix->cidx = (uint32_t *)malloc(((size_t)ix->cstart[nc] + 1) * sizeof(uint32_t));
            ix->sidx = (uint32_t *)malloc(((size_t)ix->sstart[ix->nslab] + 1) * sizeof(uint32_t));
            cfill = (uint32_t *)calloc(nc, sizeof(uint32_t));
            sfill = (uint32_t *)calloc((size_t)ix->nslab, sizeof(uint32_t));
            if (!ix->cidx || !ix->sidx || !cfill || !sfill) {
                free(cfill);
                free(sfill);
                return -1;
            }
        }
        for (uint32_t i = 0, j = mb - 1; i < mb; j = i++) {  /* edge (j, i), as pip() walks them */
            double ex0 = b[j].x < b[i].x ? b[j].x : b[i].x, ex1 = b[j].x < b[i].x ? b[i].x : b[j].x;
            double ey0 = b[j].y < b[i].y ? b[j].y : b[i].y, ey1 = b[j].y < b[i].y ? b[i].y : b[j].y;
            int cx0 = clampi((int)floor((ex0 - mg - ix->x0) / ix->cw), 0, g - 1);
            int cx1 = clampi((int)floor((ex1 + mg - ix->x0) / ix->cw), 0, g - 1);
            int cy0 = clampi((int)floor((ey0 - mg - ix->y0) / ix->ch), 0, g - 1);
            int cy1 = clampi((int)floor((ey1 + mg - ix->y0) / ix->ch), 0, g - 1);
            for (int cy = cy0; cy <= cy1; cy++)
                for (int cx = cx0; cx <= cx1; cx++) {
                    size_t c = (size_t)cy * g + cx;
                    if (pass == 0)
                        ix->cstart[c + 1]++;
                    else
                        ix->cidx[ix->cstart[c] + cfill[c]++] = i;
                }
            int s0 = clampi((int)floor((ey0 - mg - ix->y0) / ix->sh), 0, ix->nslab - 1);
            int s1 = clampi((int)floor((ey1 + mg - ix->y0) / ix->sh), 0, ix->nslab - 1);
            for (int sl = s0; sl <= s1; sl++) {
                if (pass == 0)
                    ix->sstart[sl + 1]++;
                else
                    ix->sidx[ix->sstart[sl] + sfill[sl]++] = i;
            }
        }
        free(cfill);
        free(sfill);
    }
    return 0;
}

/* pip() through the slab index: the same edges pass the same test, and the
 * parity does not depend on their order. */
static int pip_ix(const pt *r, uint32_t m, const ring_index *ix, double x, double y) {
    if (y < ix->y0 || y > ix->y1) return 0;
    int sl = clampi((int)floor((y - ix->y0) / ix->sh), 0, ix->nslab - 1);
    int in = 0;
    for (uint32_t k = ix->sstart[sl]; k < ix->sstart[sl + 1]; k++) {
        uint32_t i = ix->sidx[k], j = i == 0 ? m - 1 : i - 1;
        double yi = r[i].y, yj = r[j].y;
        if ((yi > y) != (yj > y)) {
            double xi = r[i].x, xj = r[j].x;
            double xint = xi + (y - yi) * (xj - xi) / (yj - yi);
            if (x < xint) in = !in;
        }
    }
    return in;
}

/* Sum over the edges of ring a of the parts inside ring b:
 * 0.5 * integral (x dy - y dx) about origin (ox, oy). Candidate edges of b
 * and the inside tests come from b's index; the crossing parameters and the
 * sums are computed and ordered exactly as a loop over all of b would. */
static double half_integral(const pt *a, uint32_t ma, const pt *b, uint32_t mb, double ox, double oy) {
    double acc = 0.0;
    ring_index ix;
    double *ts = (double *)malloc((mb + 2) * sizeof(double));
    if (!ts || ri_build(&ix, b, mb) != 0) {
        free(ts);
        ri_free(&ix);
        return NAN;
    }
    const double mg = 1e-7 * ((ix.x1 - ix.x0) + (ix.y1 - ix.y0) + fabs(ix.x0) + fabs(ix.y0) + 1.0);
    for (uint32_t i = 0; i + 1 < ma; i++) {
        double px = (double)a[i].x - ox, py = (double)a[i].y - oy;
        double qx = (double)a[i + 1].x - ox, qy = (double)a[i + 1].y - oy;
        double dx = qx - px, dy = qy - py;
        if (dx == 0 && dy == 0) continue;
        uint32_t nt = 0;
        ts[nt++] = 0.0;
        ts[nt++] = 1.0;
        double sx0 = a[i].x < a[i + 1].x ? a[i].x : a[i + 1].x, sx1 = a[i].x < a[i + 1].x ? a[i + 1].x : a[i].x;
        double sy0 = a[i].y < a[i + 1].y ? a[i].y : a[i + 1].y, sy1 = a[i].y < a[i + 1].y ? a[i + 1].y : a[i].y;
        if (!(sx1 + mg < ix.x0 || sx0 - mg > ix.x1 || sy1 + mg < ix.y0 || sy0 - mg > ix.y1)) {
            int cx0 = clampi((int)floor((sx0 - mg - ix.x0) / ix.cw), 0, ix.g - 1);
            int cx1 = clampi((int)floor((sx1 + mg - ix.x0) / ix.cw), 0, ix.g - 1);
            int cy0 = clampi((int)floor((sy0 - mg - ix.y0) / ix.ch), 0, ix.g - 1);
            int cy1 = clampi((int)floor((sy1 + mg - ix.y0) / ix.ch), 0, ix.g - 1);
            uint32_t tick = ++ix.tick;
            for (int cy = cy0; cy <= cy1; cy++)
                for (int cx = cx0; cx <= cx1; cx++) {
                    size_t c = (size_t)cy * ix.g + cx;
                    for (uint32_t k = ix.cstart[c]; k < ix.cstart[c + 1]; k++) {
                        uint32_t e = ix.cidx[k];  /* edge (e - 1, e) of b, i.e. j = e - 1 below */
                        if (e == 0 || ix.stamp[e] == tick) continue;  /* (mb - 1, 0): not among j + 1 < mb */
                        ix.stamp[e] = tick;
                        uint32_t j = e - 1;
                        double cx_ = (double)b[j].x - ox, cy_ = (double)b[j].y - oy;
                        double ex = (double)b[j + 1].x - ox - cx_, ey = (double)b[j + 1].y - oy - cy_;
                        double den = dx * ey - dy * ex;
                        if (den == 0) continue;
                        double rx = cx_ - px, ry = cy_ - py;
                        double tt = (rx * ey - ry * ex) / den;
                        double uu = (rx * dy - ry * dx) / den;
                        if (tt > 0 && tt < 1 && uu >= 0 && uu <= 1) ts[nt++] = tt;
                    }
                }
        }
        qsort(ts, nt, sizeof(double), cmp_t);
        for (uint32_t k = 0; k + 1 < nt; k++) {
            double t0 = ts[k], t1 = ts[k + 1];
            if (t1 <= t0) continue;
            double tm = 0.5 * (t0 + t1);
            double mx = px + tm * dx + ox, my = py + tm * dy + oy;
            if (!pip_ix(b, mb, &ix, mx, my)) continue;
            double x0 = px + t0 * dx, y0 = py + t0 * dy;
            double x1 = px + t1 * dx, y1 = py + t1 * dy;
            acc += x0 * y1 - x1 * y0;
        }
    }
    free(ts);
    ri_free(&ix);
    return 0.5 * acc;
}

/* The same sum by plain loops over every edge of b (the definition the
 * indexed version must reproduce; kept for the test that checks it). */
static double half_integral_plain(const pt *a, uint32_t ma, const pt *b, uint32_t mb, double ox, double oy) {
    double acc = 0.0;
    double *ts = (double *)malloc((mb + 2) * sizeof(double));
    if (!ts) return NAN;
    for (uint32_t i = 0; i + 1 < ma; i++) {
        double px = (double)a[i].x - ox, py = (double)a[i].y - oy;
        double qx = (double)a[i + 1].x - ox, qy = (double)a[i + 1].y - oy;
        double dx = qx - px, dy = qy - py;
        if (dx == 0 && dy == 0) continue;
        uint32_t nt = 0;
        ts[nt++] = 0.0;
        ts[nt++] = 1.0;
        for (uint32_t j = 0; j + 1 < mb; j++) {
            double cx = (double)b[j].x - ox, cy = (double)b[j].y - oy;
            double ex = (double)b[j + 1].x - ox - cx, ey = (double)b[j + 1].y - oy - cy;
            double den = dx * ey - dy * ex;
            if (den == 0) continue;
            double rx = cx - px, ry = cy - py;
            double tt = (rx * ey - ry * ex) / den;
            double uu = (rx * dy - ry * dx) / den;
            if (tt > 0 && tt < 1 && uu >= 0 && uu <= 1) ts[nt++] = tt;
        }
        qsort(ts, nt, sizeof(double), cmp_t);
        for (uint32_t k = 0; k + 1 < nt; k++) {
            double t0 = ts[k], t1 = ts[k + 1];
            if (t1 <= t0) continue;
            double tm = 0.5 * (t0 + t1);
            double mx = px + tm * dx + ox, my = py + tm * dy + oy;
            if (!pip(b, mb, mx, my)) continue;
            double x0 = px + t0 * dx, y0 = py + t0 * dy;
            double x1 = px + t1 * dx, y1 = py + t1 * dy;
            acc += x0 * y1 - x1 * y0;
        }
    }
    free(ts);
    return 0.5 * acc;
}

static double orient(const pt *r, uint32_t m, double ox, double oy) {
    double s = 0;
    for (uint32_t i = 0; i + 1 < m; i++)
        s += ((double)r[i].x - ox) * ((double)r[i + 1].y - oy) - ((double)r[i + 1].x - ox) * ((double)r[i].y - oy);
    return s >= 0 ? 1.0 : -1.0;
}

double fo_intersection_area(const float *a, uint32_t ma, const float *b, uint32_t mb) {
    const pt *A = (const pt *)a, *B = (const pt *)b;
    if (ma < 4 || mb < 4) return 0.0;
    double ox = A[0].x, oy = A[0].y;
    /* each boundary integrated with its own orientation */
    double s = orient(A, ma, ox, oy) * half_integral(A, ma, B, mb, ox, oy) +
               orient(B, mb, ox, oy) * half_integral(B, mb, A, ma, ox, oy);
    return fabs(s);
}

double fo_intersection_area_plain(const float *a, uint32_t ma, const float *b, uint32_t mb) {
    const pt *A = (const pt *)a, *B = (const pt *)b;
    if (ma < 4 || mb < 4) return 0.0;
    double ox = A[0].x, oy = A[0].y;
    double s = orient(A, ma, ox, oy) * half_integral_plain(A, ma, B, mb, ox, oy) +
               orient(B, mb, ox, oy) * half_integral_plain(B, mb, A, ma, ox, oy);
    return fabs(s);
}
