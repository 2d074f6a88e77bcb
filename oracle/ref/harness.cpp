// Harness around the FARM reference's own CPU code (linked from its unmodified
// sources by oracle/ref/Makefile). It makes the reference's per-polygon rasters
// and per-pair decisions observable, which its executables do not: they only
// print "count-found".
//
//   ref_harness raster    <in.dt> <vpr> <hier 0|1> <out.bin>
//   ref_harness intersect <S.dt> <T.dt> <vpr> <out.bin>
//   ref_harness within    <S.dt> <T.dt|-> <vpr> <out.bin>     (hierarchy on)
//   ref_harness contain   <S.dt> <T.dt> <vpr> <out.bin>       (s contains t)
//   ref_harness contain_point <S.dt> <points.bin> <vpr> <out.bin>
//       points.bin: uint64 n, then n float32 (x, y); a pair is (polygon, point)
//       for every polygon whose MBR the R-tree finds holding the point
//
// Two things are pinned so that the reference's output is deterministic:
//  * every heap allocation is zero-filled (the reference leaves some arrays it
//    later reads uninitialised);
//  * each vertex ring gets one extra vertex equal to its first. The reference
//    reads one vertex past the ring for a polygon whose raster is a single
//    pixel (Ideal.cpp:526-529 builds the sequence (0, num_vertices), and
//    geometry_computation.h:230 reads p[i + 1]); the project defines that
//    vertex as the ring's first, a zero-length closing edge.
//
// Test infrastructure only; never linked into the product.
#include <bits/stdc++.h>  // system headers first: the access override below must not reach them
#include <pthread.h>
#include <sys/time.h>
#define private public
#define protected public
#include "Ideal.h"
#include "UniversalGrid.h"
#undef private
#undef protected

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <atomic>
#include <algorithm>

// ---- zero-filled heap -------------------------------------------------------
void *operator new(size_t n) {
    void *p = calloc(1, n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void *operator new[](size_t n) {
    void *p = calloc(1, n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void operator delete(void *p) noexcept { free(p); }
void operator delete[](void *p) noexcept { free(p); }
void operator delete(void *p, size_t) noexcept { free(p); }
void operator delete[](void *p, size_t) noexcept { free(p); }

static int g_threads = 1;

static void pad_rings(vector<Ideal *> &ps) {
    for (Ideal *p : ps) {
        VertexSequence *b = p->get_boundary();
        Point *np = new Point[b->num_vertices + 1];
        memcpy(np, b->p, sizeof(Point) * b->num_vertices);
        np[b->num_vertices] = np[0];
        b->p = np;
    }
}

static vector<Ideal *> load(const char *path) {
    query_context ctx;
    ctx.num_threads = g_threads;
    vector<Ideal *> v = load_binary_file(path, ctx);
    // load_binary_file appends per-thread chunks in completion order and then
    // renumbers; restore file order so ids equal record positions.
    // (Records are decoded in file order within a chunk; with one thread the
    // chunk order is the file order.)
    pad_rings(v);
    return v;
}

template <typename F>
static void parallel_for(size_t n, F f) {
    std::atomic<size_t> next(0);
    vector<std::thread> th;
    for (int t = 0; t < g_threads; t++) {
        th.emplace_back([&]() {
            while (true) {
                size_t i = next.fetch_add(16);
                if (i >= n) break;
                size_t e = std::min(n, i + 16);
                for (size_t k = i; k < e; k++) f(k);
            }
        });
    }
    for (auto &t : th) t.join();
}

static void rasterize_all(vector<Ideal *> &ps, int vpr, bool hier) {
    if (hier) UniversalGrid::getInstance().configure(25);
    parallel_for(ps.size(), [&](size_t i) {
        Ideal *p = ps[i];
        p->init_raster(p->get_boundary()->num_vertices / vpr);
        p->use_hierachy = hier;
        if (hier) {
            p->grid_align();
            p->layering(1);
        } else {
            p->set_status_size();
        }
        p->rasterization(vpr);
    });
}

// ---- binary writer ----------------------------------------------------------
struct W {
    FILE *f;
    explicit W(const char *path) {
        f = fopen(path, "wb");
        if (!f) { perror(path); exit(2); }
    }
    ~W() { fclose(f); }
    template <typename T> void put(const T &v) { fwrite(&v, sizeof(T), 1, f); }
    void raw(const void *p, size_t n) { if (n) fwrite(p, 1, n, f); }
};

static void dump_raster(W &w, Ideal *p) {
    box *m = p->getMBB();
    w.put(m->low[0]); w.put(m->low[1]); w.put(m->high[0]); w.put(m->high[1]);
    int dimx = p->get_dimx(), dimy = p->get_dimy();
    w.put((int32_t)dimx); w.put((int32_t)dimy);
    w.put(p->get_step_x()); w.put(p->get_step_y());
    uint32_t nv = p->get_boundary()->num_vertices;
    w.put(nv);
    uint32_t ss = p->status_size;
    w.put(ss);
    w.raw(p->status, ss);
    uint32_t P = (uint32_t)dimx * (uint32_t)dimy;
    w.put(P);
    w.raw(p->offset, sizeof(uint32_t) * (P + 1));
    uint32_t les = p->len_edge_sequences;
    w.put(les);
    for (uint32_t i = 0; i < les; i++) {
        w.put((uint32_t)p->edge_sequences[i].first);
        w.put((uint32_t)p->edge_sequences[i].second);
    }
    Grid_line *gl[2] = {p->horizontal, p->vertical};
    for (int g = 0; g < 2; g++) {
        uint32_t nl = (uint32_t)gl[g]->get_num_grid_lines();
        w.put(nl);
        w.raw(gl[g]->get_offset(), sizeof(uint32_t) * nl);
        uint32_t nc = (uint32_t)gl[g]->get_num_crosses();
        w.put(nc);
        w.raw(gl[g]->get_intersection_nodes(), sizeof(double) * nc);
    }
    w.raw(p->areas, sizeof(double) * P);
    uint32_t nl = p->num_layers;
    w.put(nl);
    for (uint32_t i = 0; i < nl; i++) {
        RasterInfo &ri = p->layer_info[i];
        w.put(ri.mbr.low[0]); w.put(ri.mbr.low[1]); w.put(ri.mbr.high[0]); w.put(ri.mbr.high[1]);
        w.put((int32_t)ri.dimx); w.put((int32_t)ri.dimy);
        w.put(ri.step_x); w.put(ri.step_y);
        w.put((uint32_t)p->layer_offset[i]);
    }
}

// ---- candidate generation exactly as the reference mains do it --------------
static RTree<Ideal *, double, 2, double> g_tree;
struct SearchCtx {
    Ideal *target;
    bool skip_same;
    vector<pair<uint32_t, uint32_t>> *out;
};
static bool cb(Ideal *ideal, void *arg) {
    SearchCtx *c = (SearchCtx *)arg;
    if (c->skip_same && ideal->id == c->target->id) return true;
    c->out->push_back(make_pair((uint32_t)ideal->id, (uint32_t)c->target->id));
    return true;
}

static void write_pairs(const char *path, vector<pair<uint32_t, uint32_t>> &pairs, vector<uint8_t> &res) {
    vector<size_t> idx(pairs.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return pairs[a] < pairs[b]; });
    W w(path);
    w.put((uint64_t)pairs.size());
    for (size_t k : idx) {
        w.put(pairs[k].first);
        w.put(pairs[k].second);
        w.put(res[k]);
    }
}

int main(int argc, char **argv) {
    const char *th = getenv("FARM_REF_THREADS");
    g_threads = th ? atoi(th) : (int)std::thread::hardware_concurrency();
    if (g_threads < 1) g_threads = 1;
    if (argc < 2) { fprintf(stderr, "usage: see header\n"); return 2; }
    string mode(argv[1]);
    if (mode == "raster" && argc == 6) {
        int saved = g_threads;
        g_threads = 1;  // keep file order
        vector<Ideal *> ps = load(argv[2]);
        g_threads = saved;
        int vpr = atoi(argv[3]);
        bool hier = atoi(argv[4]) != 0;
        rasterize_all(ps, vpr, hier);
        W w(argv[5]);
        w.put((uint32_t)0x46415231u);
        w.put((uint32_t)ps.size());
        for (Ideal *p : ps) dump_raster(w, p);
        return 0;
    }
    if (mode == "contain_point" && argc == 6) {
        int saved = g_threads;
        g_threads = 1;
        vector<Ideal *> S = load(argv[2]);
        g_threads = saved;
        FILE *pf = fopen(argv[3], "rb");
        if (!pf) { perror(argv[3]); return 2; }
        uint64_t np = 0;
        if (fread(&np, 8, 1, pf) != 1) { fprintf(stderr, "bad points file\n"); return 2; }
        vector<Point> pts(np);
        for (uint64_t k = 0; k < np; k++) {
            float xy[2];
            if (fread(xy, 4, 2, pf) != 2) { fprintf(stderr, "bad points file\n"); return 2; }
            pts[k] = Point(xy[0], xy[1]);
        }
        fclose(pf);
        int vpr = atoi(argv[4]);
        for (Ideal *p : S) g_tree.Insert(p->getMBB()->low, p->getMBB()->high, p);
        vector<pair<uint32_t, uint32_t>> pairs;
        for (uint64_t k = 0; k < np; k++) {
            double lo[2] = {pts[k].x, pts[k].y};
            vector<uint32_t> hit;
            g_tree.Search(lo, lo, [](Ideal *ideal, void *arg) {
                ((vector<uint32_t> *)arg)->push_back((uint32_t)ideal->id);
                return true;
            }, &hit);
            for (uint32_t h : hit) pairs.push_back(make_pair(h, (uint32_t)k));
        }
        rasterize_all(S, vpr, false);
        vector<uint8_t> res(pairs.size(), 0);
        parallel_for(pairs.size(), [&](size_t i) {
            query_context ctx;
            res[i] = (uint8_t)S[pairs[i].first]->contain(pts[pairs[i].second], &ctx, false);
        });
        write_pairs(argv[5], pairs, res);
        size_t found = 0;
        for (auto r : res) found += r;
        printf("pairs %zu found %zu\n", pairs.size(), found);
        return 0;
    }
    if ((mode == "intersect" || mode == "within" || mode == "contain") && argc == 6) {
        int saved = g_threads;
        g_threads = 1;
        vector<Ideal *> S = load(argv[2]);
        bool self = (string(argv[3]) == "-");
        vector<Ideal *> T = self ? S : load(argv[3]);
        g_threads = saved;
        int vpr = atoi(argv[4]);
        bool within = (mode == "within");
        for (Ideal *p : S) g_tree.Insert(p->getMBB()->low, p->getMBB()->high, p);
        vector<pair<uint32_t, uint32_t>> pairs;
        query_context qctx;  // defaults: within_distance 10, geography true
        for (Ideal *t : T) {
            SearchCtx c{t, within && self, &pairs};
            if (within) {
                box qb = t->getMBB()->expand(qctx.within_distance, qctx.geography);
                g_tree.Search(qb.low, qb.high, cb, &c);
            } else {
                box *b = t->getMBB();
                g_tree.Search(b->low, b->high, cb, &c);
            }
        }
        vector<Ideal *> all(S);
        if (!self) all.insert(all.end(), T.begin(), T.end());
        rasterize_all(all, vpr, within);
        vector<uint8_t> res(pairs.size(), 0);
        parallel_for(pairs.size(), [&](size_t i) {
            query_context ctx;
            Ideal *s = S[pairs[i].first];
            Ideal *t = T[pairs[i].second];
            res[i] = within ? (uint8_t)s->within(t, &ctx)
                            : mode == "contain" ? (uint8_t)s->contain(t, &ctx, false) : (uint8_t)s->intersect(t, &ctx);
        });
        write_pairs(argv[5], pairs, res);
        size_t found = 0;
        for (auto r : res) found += r;
        printf("pairs %zu found %zu\n", pairs.size(), found);
        return 0;
    }
    fprintf(stderr, "bad arguments\n");
    return 2;
}
