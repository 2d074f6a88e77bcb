// Data tools of the polygon-join engine, host only (libfarm_host):
//
//   dump_polygons <input.wkt> <output.dt>
//       WKT polygons, one per line, to the .dt format: the reference's
//       dump_polygons tool (datagen/dump_polygons.cpp:4-15), same bytes.
//   generate_polygons -o out.dt -n count [--seed S] [--first i] [--dom-lo a]
//       [--dom-hi b] [--r-lo a] [--r-hi b] [--n-lo a] [--n-hi b] [--sigma s]
//       [--threads t] [--wkt out.wkt]
//       Seeded star polygons (include/farm_host.h farm_gen_*): polygon i of a
//       seed is the same whatever range it is generated in, so a job's sets
//       can be made in pieces. --wkt also writes them as WKT lines.
//
// One binary; the tool is chosen by the name it is invoked under (the build
// links both names to it), or by a first argument naming it.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "farm_host.h"

namespace {

int usage() {
    fprintf(stderr,
            "usage: dump_polygons <input.wkt> <output.dt>\n"
            "       generate_polygons -o out.dt -n count [--seed S] [--first i] [--dom-lo a] [--dom-hi b]\n"
            "                         [--r-lo a] [--r-hi b] [--n-lo a] [--n-hi b] [--sigma s] [--threads t]\n"
            "                         [--wkt out.wkt]\n");
    return 2;
}

int dump_main(int argc, char **argv) {
    if (argc < 3) return usage();
    uint64_t n = 0;
    if (farm_wkt_to_dt(argv[1], argv[2], &n) != FARM_OK) {
        fprintf(stderr, "dump_polygons: %s\n", farm_host_last_error());
        return 1;
    }
    fprintf(stderr, "dumped %llu polygons to %s\n", (unsigned long long)n, argv[2]);
    return 0;
}

bool write_wkt(const char *path, uint64_t n, const std::vector<uint64_t> &off, const std::vector<float> &xy) {
    FILE *f = fopen(path, "w");
    if (!f) return false;
    bool ok = true;
    for (uint64_t k = 0; k < n && ok; k++) {
        ok &= fputs("POLYGON((", f) >= 0;
        for (uint64_t j = off[k]; j < off[k + 1]; j++)
            ok &= fprintf(f, "%s%.9g %.9g", j == off[k] ? "" : ", ", xy[2 * j], xy[2 * j + 1]) > 0;
        ok &= fputs("))\n", f) >= 0;
    }
    return (fclose(f) == 0) && ok;
}

int generate_main(int argc, char **argv) {
    farm_gen_params gp;
    gp.dom_lo = 0.0;
    gp.dom_hi = 100.0;
    gp.r_lo = 0.05;
    gp.r_hi = 2.0;
    gp.n_lo = 16;
    gp.n_hi = 1000;
    gp.sigma = 0.3;
    uint64_t seed = 1, first = 0, count = 0;
    int threads = 0;
    const char *out = nullptr, *wkt = nullptr;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (i + 1 >= argc) return usage();
        const char *v = argv[++i];
        if (a == "-o") out = v;
        else if (a == "--wkt") wkt = v;
        else if (a == "-n") count = strtoull(v, nullptr, 10);
        else if (a == "--seed") seed = strtoull(v, nullptr, 10);
        else if (a == "--first") first = strtoull(v, nullptr, 10);
        else if (a == "--dom-lo") gp.dom_lo = atof(v);
        else if (a == "--dom-hi") gp.dom_hi = atof(v);
        else if (a == "--r-lo") gp.r_lo = atof(v);
        else if (a == "--r-hi") gp.r_hi = atof(v);
        else if (a == "--n-lo") gp.n_lo = atoi(v);
        else if (a == "--n-hi") gp.n_hi = atoi(v);
        else if (a == "--sigma") gp.sigma = atof(v);
        else if (a == "--threads") threads = atoi(v);
        else return usage();
    }
    if (!out || count == 0) return usage();
    std::vector<uint32_t> nv(count);
    if (farm_gen_counts(&gp, seed, first, count, nv.data()) != FARM_OK) {
        fprintf(stderr, "generate_polygons: %s\n", farm_host_last_error());
        return 1;
    }
    std::vector<uint64_t> off(count + 1, 0);
    for (uint64_t k = 0; k < count; k++) off[k + 1] = off[k] + nv[k];
    std::vector<float> xy(2 * off[count]);
    if (farm_gen_fill(&gp, seed, first, count, off.data(), xy.data(), threads) != FARM_OK ||
        farm_dt_write(out, count, off.data(), xy.data()) != FARM_OK) {
        fprintf(stderr, "generate_polygons: %s\n", farm_host_last_error());
        return 1;
    }
    if (wkt && !write_wkt(wkt, count, off, xy)) {
        fprintf(stderr, "generate_polygons: cannot write %s\n", wkt);
        return 1;
    }
    fprintf(stderr, "generated %llu polygons, %llu vertices, into %s\n", (unsigned long long)count,
            (unsigned long long)off[count], out);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    const char *base = strrchr(argv[0], '/');
    std::string name = base ? base + 1 : argv[0];
    if (name != "dump_polygons" && name != "generate_polygons" && argc > 1) {
        name = argv[1];
        argc--;
        argv++;
    }
    if (name == "dump_polygons") return dump_main(argc, argv);
    if (name == "generate_polygons") return generate_main(argc, argv);
    return usage();
}
