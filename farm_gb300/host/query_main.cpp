// Drop-in query programs for FARM's polygon-join path on one GB300:
//
//   intersect       -s S.dt -t T.dt -r [-g] [-a] [-v vpr] [-w classes] [-b batch] [-n threads]
//   within_polygon  -s S.dt -r -h [-g] [-a] [-d km] [-v vpr] [-w classes] [-b batch] [-n threads]
//   intersection    -s S.dt -t T.dt -r [-g] [-v vpr] [-w classes] [-b batch] [-n threads]
//
// One binary; the program is chosen by the name it is invoked under (the
// build links the three names to it), or by a first argument naming it. The
// flags are the reference's (query_context.cpp:227-272: -r -g -a -h -s -t -n
// -v -b -m -u, and -d / -w, which the reference declares but never
// registers); -r and -g are accepted for compatibility, since this engine
// always rasterizes and always runs the query on the GPU. The pipeline
// follows the reference's mains (intersect.cpp:41-91, within_polygon.cpp:
// 51-107, intersection.cpp:55-94): load the .dt files (streamed into the
// device store by all -n host threads, farm_store_load_dt), candidate pairs
// from MBR overlap on the GPU (farm_mbr_join_gpu: the set and order the
// reference's R-tree search returns; the within join widens each query MBR
// by the distance and skips a polygon against itself), rasterize, query in
// batches of -b pairs (0 = all), and
// print "count-found" as query_context::print_stats does
// (query_context.cpp:172-173). intersection, whose reference stops before
// computing areas, prints the number of overlapping pairs and their total
// FP64 intersection area.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>

#include <string>
#include <vector>

#include "farm_gpu.h"

namespace {

enum Kind { K_INTERSECT, K_WITHIN, K_INTERSECTION, K_UNKNOWN };

struct Args {
    Kind kind = K_UNKNOWN;
    std::string source, target;
    bool rasterize = false, gpu = false, approximation = false, hierarchy = false;
    int threads = 0, vpr = 10, unroll = 16, nlow = 0, within_distance = 10, category_count = 16;
    uint64_t batch = 0;
    float merge_threshold = 0.9f;
};

double now_ms() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec * 1e3 + tv.tv_usec / 1e3;
}

std::string stamp() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    struct tm tmv;
    localtime_r(&tv.tv_sec, &tmv);
    char b[64], out[96];
    strftime(b, sizeof b, "%H:%M:%S", &tmv);
    snprintf(out, sizeof out, "%s.%04ld", b, (long)(tv.tv_usec / 1000));
    return out;
}

void say(const char *msg) { fprintf(stderr, "%s:\t%s\n", stamp().c_str(), msg); }

void say_t(const char *msg, double t0) {
    double ms = now_ms() - t0;
    if (ms > 1000)
        fprintf(stderr, "%s:\t%s takes %f s\n", stamp().c_str(), msg, ms / 1000);
    else
        fprintf(stderr, "%s:\t%s takes %f ms\n", stamp().c_str(), msg, ms);
}

[[noreturn]] void die(const char *what, const char *detail) {
    fprintf(stderr, "%s: %s\n", what, detail ? detail : "");
    exit(1);
}

Kind kind_of(const char *name) {
    const char *b = strrchr(name, '/');
    b = b ? b + 1 : name;
    if (!strcmp(b, "intersect")) return K_INTERSECT;
    if (!strcmp(b, "within_polygon")) return K_WITHIN;
    if (!strcmp(b, "intersection")) return K_INTERSECTION;
    return K_UNKNOWN;
}

void usage() {
    fprintf(stderr,
            "query usage:\n"
            "  --help                     produce help message\n"
            "  -r [ --rasterize ]         partition with rasterization\n"
            "  -g [ --gpu ]               query with gpu\n"
            "  -a [ --approximation ]     use approximation (intersect: the fill-ratio heuristic;\n"
            "                             within_polygon: the pixel-pair midpoint distance)\n"
            "  -h [ --hierachy ]          partition with hierarchical grid\n"
            "  -s [ --source ] arg        path to the source\n"
            "  -t [ --target ] arg        path to the target\n"
            "  -n [ --threads ] arg       number of threads\n"
            "  -v [ --vpr ] arg           number of vertices per raster\n"
            "  -b [ --batch_size ] arg    batch size\n"
            "  -m [ --merge_threshold ] arg merge threshold\n"
            "  --NLow arg                 NLow\n"
            "  -u [ --unorll_size ] arg   unroll size\n"
            "  -d [ --within_distance ] arg within distance (km)\n"
            "  -w [ --category_count ] arg category count (4, 16 or 256)\n");
}

Args parse(int argc, char **argv) {
    Args a;
    int i = 1;
    a.kind = kind_of(argv[0]);
    if (a.kind == K_UNKNOWN && argc > 1) {
        a.kind = kind_of(argv[1]);
        i = 2;
    }
    auto val = [&](int &k) -> const char * {
        if (k + 1 >= argc) {
            printf("Undefined Option!\n");
            exit(0);
        }
        return argv[++k];
    };
    for (; i < argc; i++) {
        std::string f = argv[i];
        if (f == "--help") {
            usage();
            exit(0);
        } else if (f == "-r" || f == "--rasterize") {
            a.rasterize = true;
        } else if (f == "-g" || f == "--gpu") {
            a.gpu = true;
        } else if (f == "-a" || f == "--approximation") {
            a.approximation = true;
        } else if (f == "-h" || f == "--hierachy") {
            a.hierarchy = true;
        } else if (f == "-s" || f == "--source") {
            a.source = val(i);
        } else if (f == "-t" || f == "--target") {
            a.target = val(i);
        } else if (f == "-n" || f == "--threads") {
            a.threads = atoi(val(i));
        } else if (f == "-v" || f == "--vpr") {
            a.vpr = atoi(val(i));
        } else if (f == "-b" || f == "--batch_size") {
            a.batch = strtoull(val(i), nullptr, 10);
        } else if (f == "-m" || f == "--merge_threshold") {
            a.merge_threshold = (float)atof(val(i));
        } else if (f == "--NLow") {
            a.nlow = atoi(val(i));
        } else if (f == "-u" || f == "--unorll_size") {
            a.unroll = atoi(val(i));
        } else if (f == "-d" || f == "--within_distance") {
            a.within_distance = atoi(val(i));
        } else if (f == "-w" || f == "--category_count") {
            a.category_count = atoi(val(i));
        } else {
            printf("Undefined Option!\n");
            exit(0);
        }
    }
    return a;
}

void check(int rc, const char *what) {
    if (rc != FARM_OK) die(what, farm_last_error());
}

}  // namespace

int main(int argc, char **argv) {
    Args a = parse(argc, argv);
    if (a.kind == K_UNKNOWN) {
        fprintf(stderr, "run as intersect, within_polygon or intersection (or name one as the first argument)\n");
        return 1;
    }
    if (a.source.empty()) die("missing", "-s source.dt");
    if (a.kind != K_WITHIN && a.target.empty()) die("missing", "-t target.dt");
    if (a.kind == K_WITHIN) a.hierarchy = true;  // the within filter walks the hierarchy's layers

    double t0 = now_ms();
    farm_store *st = nullptr;
    check(farm_store_create(&st), "farm_store_create");
    check(farm_store_load_dt(st, 0, a.source.c_str(), a.threads, nullptr), "farm_store_load_dt(source)");
    // within_polygon joins the source set with itself (within_polygon.cpp:9-48)
    const int self = a.kind == K_WITHIN ? 1 : 0;
    if (!self) check(farm_store_load_dt(st, 1, a.target.c_str(), a.threads, nullptr), "farm_store_load_dt(target)");
    say_t("loading data finished", t0);

    t0 = now_ms();
    const double expand = self ? (double)a.within_distance : 0.0;
    uint64_t np = 0;
    int rc = farm_mbr_join_gpu(st, expand, self, self, nullptr, 0, FARM_MEM_HOST, &np);  // count
    if (rc != FARM_OK && rc != FARM_EOVERFLOW) check(rc, "farm_mbr_join_gpu");
    std::vector<uint32_t> pairs(2 * np + 2);
    if (np) check(farm_mbr_join_gpu(st, expand, self, self, pairs.data(), np, FARM_MEM_HOST, &np), "farm_mbr_join_gpu");
    pairs.resize(2 * np);
    say_t("rtree filtering finished", t0);

    t0 = now_ms();
    farm_raster_opts ro;
    memset(&ro, 0, sizeof ro);
    ro.vpr = a.vpr;
    ro.category_count = a.category_count;
    ro.hierarchy = a.hierarchy ? 1 : 0;
    rc = farm_rasterize(st, &ro);
    if (rc == FARM_EASSERT)
        say("some polygons fail the reference's raster assertions; their pairs are reported as 2 and not counted");
    else
        check(rc, "farm_rasterize");
    say_t("preprocess finished", t0);

    t0 = now_ms();
    const uint64_t batch = a.batch ? a.batch : (np ? np : 1);
    uint64_t found = 0;
    double area_sum = 0.0;
    std::vector<uint8_t> out;
    std::vector<double> area;
    for (uint64_t i = 0; i < np; i += batch) {
        const uint64_t n = np - i < batch ? np - i : batch;
        uint64_t f = 0;
        if (a.kind == K_INTERSECT) {
            out.resize(n);
            check(farm_intersect(st, pairs.data() + 2 * i, n, a.approximation ? FARM_MODE_APPROX : FARM_MODE_EXACT,
                                 FARM_MEM_HOST, out.data(), &f, nullptr),
                  "farm_intersect");
        } else if (a.kind == K_WITHIN) {
            out.resize(n);
            check(farm_within_mode(st, pairs.data() + 2 * i, n, (double)a.within_distance, 1, 1,
                                   a.approximation ? FARM_MODE_APPROX : FARM_MODE_EXACT, FARM_MEM_HOST, out.data(),
                                   &f, nullptr),
                  "farm_within_mode");
        } else {
            area.resize(n);
            check(farm_intersection_area(st, pairs.data() + 2 * i, n, FARM_MEM_HOST, area.data(), nullptr),
                  "farm_intersection_area");
            for (uint64_t k = 0; k < n; k++)
                if (area[k] > 0) {
                    f++;
                    area_sum += area[k];
                }
        }
        found += f;
    }
    char line[160];
    snprintf(line, sizeof line, "count-found:\t%llu", (unsigned long long)found);
    say(line);
    if (a.kind == K_INTERSECTION) {
        snprintf(line, sizeof line, "area-total:\t%.17g", area_sum);
        say(line);
    }
    say_t("query finished", t0);
    farm_store_destroy(st);
    return 0;
}
