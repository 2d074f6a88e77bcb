// Host-side services of the GB300 polygon-join engine: .dt I/O, the seeded
// star-polygon generator and the MBR candidate join. C ABI in include/farm_host.h.
//
// Reference behaviour followed here:
//  * .dt layout: storage.cpp:158-193 (writer) and :320-449 (reader),
//    MyPolygon.cpp:736-759, vertex_sequence.cpp:196-219.
//  * MBR: vertex_sequence.cpp:152-168 (float32 bias 1e-9 promoted to double).
//  * candidate join: intersect_cpu.cpp:18-36 / within_polygon_cpu.cpp:20-49
//    with RTree::Overlap (RTree.h:1567-1580): closed-rectangle overlap.
//  * widening: Box.cpp:200-214; longitude table util.h:73-96.
#include "../../include/farm_host.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int nthreads(int requested) {
    if (requested > 0) return requested;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

template <typename F>
void parallel_chunks(uint64_t n, int threads, uint64_t grain, F f) {
    threads = nthreads(threads);
    if (n <= grain || threads == 1) {
        f(0, n);
        return;
    }
    std::atomic<uint64_t> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) {
        th.emplace_back([&]() {
            for (;;) {
                uint64_t b = next.fetch_add(grain);
                if (b >= n) break;
                f(b, std::min(n, b + grain));
            }
        });
    }
    for (auto &x : th) x.join();
}

// ---- counter-based random numbers ------------------------------------------
// splitmix64 finaliser over a (seed, polygon, stream, index) counter.
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t rng_u64(uint64_t seed, uint64_t poly, uint32_t stream, uint64_t idx) {
    uint64_t h = mix64(seed ^ 0x5851F42D4C957F2Dull);
    h = mix64(h ^ poly);
    h = mix64(h ^ ((uint64_t)stream << 40) ^ idx);
    return h;
}
// uniform in (0, 1): never exactly 0 or 1
inline double rng_open01(uint64_t seed, uint64_t poly, uint32_t stream, uint64_t idx) {
    uint64_t h = rng_u64(seed, poly, stream, idx);
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

enum : uint32_t { S_CX = 1, S_CY, S_R, S_N, S_PHI, S_GAP, S_NRM_U, S_NRM_V };

uint32_t gen_count(const farm_gen_params *gp, uint64_t seed, uint64_t i) {
    double u = rng_open01(seed, i, S_N, 0);
    double lo = std::log((double)gp->n_lo), hi = std::log((double)gp->n_hi + 1.0);
    int64_t n = (int64_t)std::floor(std::exp(lo + u * (hi - lo)));
    if (n < gp->n_lo) n = gp->n_lo;
    if (n > gp->n_hi) n = gp->n_hi;
    return (uint32_t)n + 1;  // + closing copy
}

}  // namespace

extern "C" {

const char *farm_host_last_error(void) { return g_err.c_str(); }

int farm_gen_counts(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count,
                    uint32_t *nverts_out) {
    if (!gp || (!nverts_out && count)) return fail(FARM_EINVAL, "null argument");
    if (gp->n_lo < 3 || gp->n_hi < gp->n_lo) return fail(FARM_EINVAL, "vertex-count range must satisfy 3 <= n_lo <= n_hi");
    if (!(gp->r_lo > 0) || gp->r_hi < gp->r_lo) return fail(FARM_EINVAL, "radius range must satisfy 0 < r_lo <= r_hi");
    for (uint64_t i = 0; i < count; i++) nverts_out[i] = gen_count(gp, seed, first + i);
    return FARM_OK;
}

int farm_gen_centres(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count, double *cxyr) {
    if (!gp || (!cxyr && count)) return fail(FARM_EINVAL, "null argument");
    if (!(gp->r_lo > 0) || gp->r_hi < gp->r_lo) return fail(FARM_EINVAL, "radius range must satisfy 0 < r_lo <= r_hi");
    const double span = gp->dom_hi - gp->dom_lo;
    const double lr0 = std::log(gp->r_lo), lr1 = std::log(gp->r_hi);
    for (uint64_t k = 0; k < count; k++) {
        uint64_t i = first + k;
        cxyr[3 * k] = gp->dom_lo + span * rng_open01(seed, i, S_CX, 0);
        cxyr[3 * k + 1] = gp->dom_lo + span * rng_open01(seed, i, S_CY, 0);
        cxyr[3 * k + 2] = std::exp(lr0 + rng_open01(seed, i, S_R, 0) * (lr1 - lr0));
    }
    return FARM_OK;
}

}  // extern "C"

namespace {
// Fills polygon k of the output with generator polygon index(k).
template <typename Index>
int gen_fill(const farm_gen_params *gp, uint64_t seed, Index index, uint64_t count, const uint64_t *off, float *xy,
             int threads) {
    if (!gp || !off || (!xy && count)) return fail(FARM_EINVAL, "null argument");
    const double two_pi = 6.283185307179586476925286766559;
    std::atomic<int> bad(0);
    parallel_chunks(count, threads, 64, [&](uint64_t b, uint64_t e) {
        std::vector<double> cum;
        for (uint64_t k = b; k < e; k++) {
            uint64_t i = index(k);
            uint32_t m = gen_count(gp, seed, i);
            if (off[k + 1] - off[k] != m) {
                bad = 1;
                continue;
            }
            uint32_t n = m - 1;
            double span = gp->dom_hi - gp->dom_lo;
            double cx = gp->dom_lo + span * rng_open01(seed, i, S_CX, 0);
            double cy = gp->dom_lo + span * rng_open01(seed, i, S_CY, 0);
            double lr0 = std::log(gp->r_lo), lr1 = std::log(gp->r_hi);
            double rbar = std::exp(lr0 + rng_open01(seed, i, S_R, 0) * (lr1 - lr0));
            double phi = two_pi * rng_open01(seed, i, S_PHI, 0);
            // sorted uniform angles as normalised partial sums of Exp(1) gaps;
            // redrawn (next attempt of the same counter stream) until no
            // angular gap exceeds 2*pi/3, so the ring is simple and star-shaped
            // about its centre (a gap beyond pi lets a chord cross other edges)
            cum.resize(n + 1);
            double acc = 0.0;
            for (uint64_t attempt = 0;; attempt++) {
                acc = 0.0;
                double gmax = 0.0, g0 = 0.0, gap = 0.0;
                for (uint32_t j = 0; j <= n; j++) {
                    gap = -std::log(rng_open01(seed, i, S_GAP, attempt * (uint64_t)(n + 1) + j));
                    acc += gap;
                    cum[j] = acc;
                    if (j == 0) g0 = gap;
                    else if (j < n) gmax = std::max(gmax, gap);
                }
                gmax = std::max(gmax, g0 + gap);  // the wrap-around gap
                if (gmax / acc <= 1.0 / 3.0 || attempt >= 64) break;
            }
            float *out = xy + 2 * off[k];
            for (uint32_t j = 0; j < n; j++) {
                double th = phi + two_pi * (cum[j] / acc);
                double u = rng_open01(seed, i, S_NRM_U, j), v = rng_open01(seed, i, S_NRM_V, j);
                double z = std::sqrt(-2.0 * std::log(u)) * std::cos(two_pi * v);
                double r = rbar * std::exp(gp->sigma * z);
                out[2 * j] = (float)(cx + r * std::cos(th));
                out[2 * j + 1] = (float)(cy + r * std::sin(th));
            }
            out[2 * n] = out[0];
            out[2 * n + 1] = out[1];
        }
    });
    if (bad) return fail(FARM_EINVAL, "offsets do not match the generator's vertex counts");
    return FARM_OK;
}
}  // namespace

extern "C" {

int farm_gen_fill(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count, const uint64_t *off,
                  float *xy, int threads) {
    return gen_fill(gp, seed, [first](uint64_t k) { return first + k; }, count, off, xy, threads);
}

int farm_gen_radii(const farm_gen_params *gp, uint64_t seed, uint64_t first, uint64_t count, double *rmax,
                   int threads) {
    if (!gp || (!rmax && count)) return fail(FARM_EINVAL, "null argument");
    if (gp->n_lo < 3 || gp->n_hi < gp->n_lo) return fail(FARM_EINVAL, "vertex-count range must satisfy 3 <= n_lo <= n_hi");
    if (!(gp->r_lo > 0) || gp->r_hi < gp->r_lo) return fail(FARM_EINVAL, "radius range must satisfy 0 < r_lo <= r_hi");
    const double two_pi = 6.283185307179586476925286766559;
    const double lr0 = std::log(gp->r_lo), lr1 = std::log(gp->r_hi);
    parallel_chunks(count, threads, 64, [&](uint64_t b, uint64_t e) {
        for (uint64_t k = b; k < e; k++) {
            const uint64_t i = first + k;
            const uint32_t n = gen_count(gp, seed, i) - 1;
            const double rbar = std::exp(lr0 + rng_open01(seed, i, S_R, 0) * (lr1 - lr0));
            // the same draws as gen_fill's per-vertex radius; every step from
            // z to r is monotone, so the largest z gives the largest r. As
            // z <= sqrt(-2 ln u), a vertex whose u lies above exp(-zmax^2 / 2)
            // (with a relative margin far above the rounding of that bound)
            // cannot raise zmax, and its logarithm and cosine are skipped.
            double zmax = -1e300, ucut = 1.0;
            for (uint32_t j = 0; j < n; j++) {
                double u = rng_open01(seed, i, S_NRM_U, j);
                if (u > ucut) continue;
                double v = rng_open01(seed, i, S_NRM_V, j);
                double z = std::sqrt(-2.0 * std::log(u)) * std::cos(two_pi * v);
                if (z > zmax) {
                    zmax = z;
                    ucut = zmax > 0 ? std::exp(-0.5 * zmax * zmax) * (1.0 + 1e-9) : 1.0;
                }
            }
            rmax[k] = rbar * std::exp(gp->sigma * zmax);
        }
    });
    return FARM_OK;
}

int farm_gen_counts_idx(const farm_gen_params *gp, uint64_t seed, const uint64_t *idx, uint64_t count,
                        uint32_t *nverts_out) {
    if (!gp || (count && (!idx || !nverts_out))) return fail(FARM_EINVAL, "null argument");
    if (gp->n_lo < 3 || gp->n_hi < gp->n_lo) return fail(FARM_EINVAL, "vertex-count range must satisfy 3 <= n_lo <= n_hi");
    for (uint64_t k = 0; k < count; k++) nverts_out[k] = gen_count(gp, seed, idx[k]);
    return FARM_OK;
}

int farm_gen_fill_idx(const farm_gen_params *gp, uint64_t seed, const uint64_t *idx, uint64_t count,
                      const uint64_t *off, float *xy, int threads) {
    if (count && !idx) return fail(FARM_EINVAL, "null argument");
    return gen_fill(gp, seed, [idx](uint64_t k) { return idx[k]; }, count, off, xy, threads);
}

static void ring_mbr(const float *p, uint64_t m, double *b) {
    // the ring as the reference holds it in memory repeats p[0] once more;
    // that cannot change the min/max, so the stored vertices suffice.
    double lx = 100000.0, ly = 100000.0, hx = -100000.0, hy = -100000.0;  // Box.h:6-12
    for (uint64_t j = 0; j < m; j++) {
        double x = (double)p[2 * j], y = (double)p[2 * j + 1];
        lx = std::min(lx, x);
        hx = std::max(hx, x);
        ly = std::min(ly, y);
        hy = std::max(hy, y);
    }
    const double bias = (double)1e-9f;
    b[0] = lx - bias;
    b[1] = ly - bias;
    b[2] = hx + bias;
    b[3] = hy + bias;
}

int farm_mbr(uint64_t n, const uint64_t *off, const float *xy, double *mbr, int threads) {
    if (!off || (n && (!xy || !mbr))) return fail(FARM_EINVAL, "null argument");
    parallel_chunks(n, threads, 256, [&](uint64_t b, uint64_t e) {
        for (uint64_t k = b; k < e; k++) ring_mbr(xy + 2 * off[k], off[k + 1] - off[k], mbr + 4 * k);
    });
    return FARM_OK;
}

int farm_dt_write(const char *path, uint64_t n, const uint64_t *off, const float *xy) {
    if (!path || !off || (n && !xy)) return fail(FARM_EINVAL, "null argument");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(FARM_EIO, std::string("cannot open ") + path);
    struct Meta {
        uint32_t size, nv;
        uint64_t offset;
        double mbr[4];
    };
    static_assert(sizeof(Meta) == 48, "PolygonMeta layout");
    std::vector<Meta> meta(n);
    uint64_t cur = 0;
    bool ok = true;
    for (uint64_t k = 0; k < n && ok; k++) {
        uint64_t m = off[k + 1] - off[k];
        uint64_t holes = 0;
        ok &= fwrite(&holes, 8, 1, f) == 1;
        ok &= fwrite(&m, 8, 1, f) == 1;
        ok &= fwrite(xy + 2 * off[k], 8, m, f) == m;
        Meta &mt = meta[k];
        mt.size = (uint32_t)(16 + 8 * m);
        // the reference records the in-memory count (stored + 1)
        mt.nv = (uint32_t)(m + 1);
        mt.offset = cur;
        ring_mbr(xy + 2 * off[k], m, mt.mbr);
        cur += 16 + 8 * m;
    }
    if (ok && n) ok &= fwrite(meta.data(), sizeof(Meta), n, f) == n;
    ok &= fwrite(&n, 8, 1, f) == 1;
    ok &= fclose(f) == 0;
    if (!ok) return fail(FARM_EIO, std::string("write failed: ") + path);
    return FARM_OK;
}

int farm_dt_read(const char *path, uint64_t *n_out, uint64_t *total_out, uint64_t *off, float *xy) {
    if (!path || !n_out || !total_out) return fail(FARM_EINVAL, "null argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(FARM_EIO, std::string("cannot open ") + path);
    std::vector<char> buf;
    if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return fail(FARM_EIO, "seek failed"); }
    long sz = ftell(f);
    if (sz < 8) { fclose(f); return fail(FARM_EFORMAT, "file too small for a .dt"); }
    fseek(f, 0, SEEK_SET);
    buf.resize((size_t)sz);
    if (fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) { fclose(f); return fail(FARM_EIO, "short read"); }
    fclose(f);
    uint64_t nrec;
    memcpy(&nrec, buf.data() + sz - 8, 8);
    if (nrec == 0 || nrec > (uint64_t)(sz - 8) / 48) return fail(FARM_EFORMAT, "bad polygon count in .dt trailer");
    const char *meta = buf.data() + sz - 8 - 48 * nrec;
    uint64_t data_end = (uint64_t)(sz - 8 - 48 * nrec);
    // decode records in file order, following the meta offsets (storage.cpp:396-430)
    uint64_t kept = 0, total = 0;
    for (int pass = 0; pass < 2; pass++) {
        kept = 0;
        total = 0;
        if (pass == 1) off[0] = 0;
        for (uint64_t r = 0; r < nrec; r++) {
            uint64_t o;
            memcpy(&o, meta + 48 * r + 8, 8);
            if (o + 16 > data_end) return fail(FARM_EFORMAT, "record offset beyond data");
            uint64_t holes, m;
            memcpy(&holes, buf.data() + o, 8);
            memcpy(&m, buf.data() + o + 8, 8);
            if (m == 0 || o + 16 + 8 * m > data_end) return fail(FARM_EFORMAT, "bad vertex count in record");
            // skip holes (decoded and dropped by the reference, MyPolygon.cpp:755-757)
            uint64_t q = o + 16 + 8 * m;
            for (uint64_t h = 0; h < holes; h++) {
                if (q + 8 > data_end) return fail(FARM_EFORMAT, "bad hole record");
                uint64_t hm;
                memcpy(&hm, buf.data() + q, 8);
                q += 8 + 8 * hm;
                if (q > data_end) return fail(FARM_EFORMAT, "bad hole record");
            }
            if (m + 1 < 3) continue;  // storage.cpp:341
            if (pass == 1) {
                memcpy(xy + 2 * total, buf.data() + o + 16, 8 * m);
                off[kept + 1] = total + m;
            }
            total += m;
            kept++;
        }
        if (pass == 0) {
            *n_out = kept;
            *total_out = total;
            if (!xy || !off) return FARM_OK;
        }
    }
    return FARM_OK;
}

void farm_degree_table(double *out) {
    // util.h:73 lists 360 / (sin((90 - lat) * PI / 180) * 40076) for lat = i/10,
    // printed to 6 decimals, with PI = 3.14159265 (util.h:45, :84).
    const double PI = 3.14159265;
    char tmp[64];
    for (int i = 0; i < 900; i++) {
        double lat = i / 10.0;
        double v = 360.0 / (std::sin((90 - lat) * PI / 180) * 40076);
        snprintf(tmp, sizeof tmp, "%.6f", v);
        out[i] = strtod(tmp, nullptr);
    }
}

int farm_mbr_join(uint64_t ns, const double *ms, uint64_t nt, const double *mt, double expand, int geography,
                  int skip_same, uint64_t *npairs, uint32_t *pairs, int threads) {
    if (!npairs || (ns && !ms) || (nt && !mt)) return fail(FARM_EINVAL, "null argument");
    if (ns > 0xFFFFFFFFull || nt > 0xFFFFFFFFull) return fail(FARM_EOVERFLOW, "more than 2^32 polygons on one side");
    static double deg[900];
    static std::once_flag once;
    std::call_once(once, []() { farm_degree_table(deg); });
    const double deg_lat = 360.0 / 40076.0;
    auto widen = [&](const double *b, double *o) {
        double sx = expand, sy = expand;
        if (geography && expand != 0.0) {
            double a = std::fabs(b[1]);
            if (a == 90) a = 89.9;
            int idx = (int)(a * 10);
            if (idx < 0 || idx >= 900) idx = 899;  // the reference indexes out of range here
            sx *= deg[idx];
            sy *= deg_lat;
        }
        o[0] = b[0] - sx;
        o[1] = b[1] - sy;
        o[2] = b[2] + sx;
        o[3] = b[3] + sy;
    };
    if (ns == 0 || nt == 0) {
        *npairs = 0;
        return FARM_OK;
    }
    // uniform grid over the source rectangles; cell ~ mean source extent
    double gx0 = 1e300, gy0 = 1e300, gx1 = -1e300, gy1 = -1e300, wsum = 0, hsum = 0;
    for (uint64_t i = 0; i < ns; i++) {
        const double *b = ms + 4 * i;
        gx0 = std::min(gx0, b[0]);
        gy0 = std::min(gy0, b[1]);
        gx1 = std::max(gx1, b[2]);
        gy1 = std::max(gy1, b[3]);
        wsum += b[2] - b[0];
        hsum += b[3] - b[1];
    }
    double cw = std::max(wsum / ns, 1e-12), ch = std::max(hsum / ns, 1e-12);
    double gw = gx1 - gx0, gh = gy1 - gy0;
    int64_t nx = std::max<int64_t>(1, std::min<int64_t>(4096, (int64_t)(gw / cw) + 1));
    int64_t ny = std::max<int64_t>(1, std::min<int64_t>(4096, (int64_t)(gh / ch) + 1));
    cw = gw / nx;
    ch = gh / ny;
    if (!(cw > 0)) cw = 1;
    if (!(ch > 0)) ch = 1;
    auto cellx = [&](double x) {
        int64_t c = (int64_t)std::floor((x - gx0) / cw);
        return std::min<int64_t>(nx - 1, std::max<int64_t>(0, c));
    };
    auto celly = [&](double y) {
        int64_t c = (int64_t)std::floor((y - gy0) / ch);
        return std::min<int64_t>(ny - 1, std::max<int64_t>(0, c));
    };
    std::vector<uint64_t> cnt(nx * ny + 1, 0);
    for (uint64_t i = 0; i < ns; i++) {
        const double *b = ms + 4 * i;
        for (int64_t y = celly(b[1]); y <= celly(b[3]); y++)
            for (int64_t x = cellx(b[0]); x <= cellx(b[2]); x++) cnt[y * nx + x + 1]++;
    }
    for (size_t c = 1; c < cnt.size(); c++) cnt[c] += cnt[c - 1];
    std::vector<uint32_t> items(cnt.back());
    std::vector<uint64_t> fillp(cnt.begin(), cnt.end() - 1);
    for (uint64_t i = 0; i < ns; i++) {
        const double *b = ms + 4 * i;
        for (int64_t y = celly(b[1]); y <= celly(b[3]); y++)
            for (int64_t x = cellx(b[0]); x <= cellx(b[2]); x++) items[fillp[y * nx + x]++] = (uint32_t)i;
    }
    // per-target results, found in parallel and concatenated in target order
    int T = nthreads(threads);
    uint64_t nchunks = std::min<uint64_t>(nt, (uint64_t)T * 16);
    std::vector<std::vector<uint32_t>> out(nchunks);
    std::atomic<uint64_t> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++) {
        th.emplace_back([&]() {
            std::vector<uint32_t> local;
            for (;;) {
                uint64_t c = next.fetch_add(1);
                if (c >= nchunks) break;
                uint64_t b = nt * c / nchunks, e = nt * (c + 1) / nchunks;
                std::vector<uint32_t> &o = out[c];
                for (uint64_t j = b; j < e; j++) {
                    double q[4];
                    widen(mt + 4 * j, q);
                    if (q[0] > gx1 || q[2] < gx0 || q[1] > gy1 || q[3] < gy0) continue;
                    local.clear();
                    for (int64_t y = celly(q[1]); y <= celly(q[3]); y++)
                        for (int64_t x = cellx(q[0]); x <= cellx(q[2]); x++) {
                            uint64_t cc = y * nx + x;
                            for (uint64_t k = cnt[cc]; k < cnt[cc + 1]; k++) local.push_back(items[k]);
                        }
                    std::sort(local.begin(), local.end());
                    local.erase(std::unique(local.begin(), local.end()), local.end());
                    for (uint32_t s : local) {
                        if (skip_same && s == j) continue;
                        const double *a = ms + 4 * (uint64_t)s;
                        if (a[0] > q[2] || q[0] > a[2] || a[1] > q[3] || q[1] > a[3]) continue;
                        o.push_back(s);
                        o.push_back((uint32_t)j);
                    }
                }
            }
        });
    }
    for (auto &x : th) x.join();
    uint64_t total = 0;
    for (auto &o : out) total += o.size() / 2;
    if (!pairs) {
        *npairs = total;
        return FARM_OK;
    }
    if (*npairs < total) return fail(FARM_EINVAL, "pair buffer too small");
    std::vector<uint64_t> keys;
    keys.reserve(total);
    for (auto &o : out)
        for (size_t k = 0; k < o.size(); k += 2) keys.push_back(((uint64_t)o[k] << 32) | o[k + 1]);
    std::sort(keys.begin(), keys.end());
    for (uint64_t k = 0; k < total; k++) {
        pairs[2 * k] = (uint32_t)(keys[k] >> 32);
        pairs[2 * k + 1] = (uint32_t)keys[k];
    }
    *npairs = total;
    return FARM_OK;
}

}  // extern "C"

// ---- WKT polygons (the reference's dump_polygons tool) ----------------------
//
// Each line of the input is one WKT geometry, parsed by the reference's rules
// (storage.cpp:8-94 load_polygon_wkt, :683-715 read_polygon;
// MyPolygon.cpp:227-262 read_vertices; util.h:108-152 read_double,
// skip_space), which fix what the tool accepts:
//  * parsing starts at the line's first '(' (so "POLYGON" or any other prefix
//    is ignored, and a MULTIPOLYGON yields the boundary of its first polygon);
//  * a ring's vertex count is one more than the commas between its '(' and the
//    first ')' after it; each coordinate is the next run of the characters
//    [-.0-9e] (so "1e+05" reads as the two numbers 1 and 05), converted by
//    atof and stored as float32;
//  * rings keep their order: VertexSequence::area() is an absolute value, so
//    clockwise() is never true; the boundary is never reversed and a hole is
//    reversed twice;
//  * holes are parsed (their syntax is checked) but dropped: read_polygon
//    appends them to the copy that get_holes() returns (MyPolygon.h:132);
//  * an empty line is skipped. Where the reference asserts (a missing
//    parenthesis) or reads past the line (no '(' at all, or too few numbers),
//    this parser reports FARM_EFORMAT with the line number instead.
namespace {

struct WktPolygon {
    std::vector<float> boundary;            // interleaved x, y as the WKT lists them
    std::vector<std::vector<float>> holes;  // the same per hole
};

struct WktCursor {
    const std::string &s;
    size_t o;
    bool at(char c) const { return o < s.size() && s[o] == c; }
    void skip_space() {
        while (o < s.size() && (s[o] == ' ' || s[o] == '\t' || s[o] == '\n')) o++;
    }
    static bool number_char(char c) { return c == '-' || c == '.' || (c >= '0' && c <= '9') || c == 'e'; }
    bool number(double &v) {
        while (o < s.size() && !number_char(s[o])) o++;
        if (o >= s.size()) return false;
        char tmp[100];
        int k = 0;
        while (o < s.size() && number_char(s[o])) {
            if (k == 99) return false;  // the reference's token buffer holds 99 characters
            tmp[k++] = s[o++];
        }
        tmp[k] = 0;
        v = atof(tmp);
        return true;
    }
    bool ring(std::vector<float> &out) {
        skip_space();
        if (!at('(')) return false;
        o++;
        size_t close = s.find(')', o);
        if (close == std::string::npos) return false;
        uint64_t nv = 1;
        for (size_t k = o + 1; k < close; k++) nv += s[k] == ',';
        out.resize(2 * nv);
        for (uint64_t i = 0; i < 2 * nv; i++) {
            double v;
            if (!number(v)) return false;
            out[i] = (float)v;
        }
        skip_space();
        if (!at(')')) return false;
        o++;
        return true;
    }
};

// 0: polygon parsed; 1: empty line (skipped); -1: malformed
int wkt_parse(const std::string &line, WktPolygon &p) {
    if (line.empty()) return 1;
    size_t first = line.find('(');
    if (first == std::string::npos) return -1;
    WktCursor c{line, first};
    c.skip_space();
    if (!c.at('(')) return -1;
    c.o++;
    p.boundary.clear();
    p.holes.clear();
    if (!c.ring(p.boundary)) return -1;
    c.skip_space();
    while (c.at(',')) {
        c.o++;
        p.holes.emplace_back();
        if (!c.ring(p.holes.back())) return -1;
        c.skip_space();
    }
    if (!c.at(')')) return -1;
    return 0;
}

int wkt_load(const char *path, std::vector<WktPolygon> &polys) {
    FILE *f = fopen(path, "rb");
    if (!f) return fail(FARM_EIO, std::string("cannot open ") + path);
    std::string line;
    uint64_t lineno = 0;
    int ch;
    bool more = true;
    while (more) {
        line.clear();
        while ((ch = fgetc(f)) != EOF && ch != '\n') line.push_back((char)ch);
        more = ch != EOF;
        if (!more && line.empty()) break;
        lineno++;
        WktPolygon p;
        int r = wkt_parse(line, p);
        if (r < 0) {
            fclose(f);
            return fail(FARM_EFORMAT, std::string(path) + ":" + std::to_string(lineno) + ": malformed WKT polygon");
        }
        if (r == 0) polys.push_back(std::move(p));
    }
    fclose(f);
    return FARM_OK;
}

}  // namespace

extern "C" {

int farm_wkt_read(const char *path, uint64_t *n_out, uint64_t *total_out, uint64_t *off, float *xy) {
    if (!path || !n_out || !total_out) return fail(FARM_EINVAL, "null argument");
    std::vector<WktPolygon> polys;
    int rc = wkt_load(path, polys);
    if (rc) return rc;
    uint64_t total = 0;
    for (auto &p : polys) total += p.boundary.size() / 2;
    *n_out = polys.size();
    *total_out = total;
    if (!off || !xy) return FARM_OK;
    off[0] = 0;
    uint64_t at = 0;
    for (size_t k = 0; k < polys.size(); k++) {
        memcpy(xy + 2 * at, polys[k].boundary.data(), polys[k].boundary.size() * sizeof(float));
        at += polys[k].boundary.size() / 2;
        off[k + 1] = at;
    }
    return FARM_OK;
}

int farm_wkt_to_dt(const char *wkt_path, const char *dt_path, uint64_t *n_out) {
    if (!wkt_path || !dt_path) return fail(FARM_EINVAL, "null argument");
    std::vector<WktPolygon> polys;
    int rc = wkt_load(wkt_path, polys);
    if (rc) return rc;
    // dump_polygons_to_file (storage.cpp:158-193) with MyPolygon::encode / get_meta
    // (MyPolygon.cpp:728-745). read_polygon adds each hole through get_holes(),
    // which returns the hole list by value (MyPolygon.h:132), so the holes are
    // parsed but never reach the polygon: every record has no holes, and the
    // meta's vertex count is the boundary's as parsed.
    FILE *f = fopen(dt_path, "wb");
    if (!f) return fail(FARM_EIO, std::string("cannot open ") + dt_path);
    struct Meta {
        uint32_t size, nv;
        uint64_t offset;
        double mbr[4];
    };
    static_assert(sizeof(Meta) == 48, "PolygonMeta layout");
    std::vector<Meta> meta(polys.size());
    uint64_t cur = 0;
    bool ok = true;
    for (size_t k = 0; k < polys.size() && ok; k++) {
        const WktPolygon &p = polys[k];
        uint64_t holes = 0, m = p.boundary.size() / 2;
        uint64_t size = 16 + 8 * m;
        if (size > 0xFFFFFFFFull) {
            fclose(f);
            return fail(FARM_EOVERFLOW, "polygon " + std::to_string(k) + " exceeds the 32-bit record size");
        }
        ok &= fwrite(&holes, 8, 1, f) == 1;
        ok &= fwrite(&m, 8, 1, f) == 1;
        ok &= fwrite(p.boundary.data(), 8, m, f) == m;
        Meta &mt = meta[k];
        mt.size = (uint32_t)size;
        mt.nv = (uint32_t)m;
        mt.offset = cur;
        ring_mbr(p.boundary.data(), m, mt.mbr);
        cur += size;
    }
    uint64_t n = polys.size();
    if (ok && n) ok &= fwrite(meta.data(), sizeof(Meta), n, f) == n;
    ok &= fwrite(&n, 8, 1, f) == 1;
    ok &= fclose(f) == 0;
    if (!ok) return fail(FARM_EIO, std::string("write failed: ") + dt_path);
    if (n_out) *n_out = n;
    return FARM_OK;
}

}  // extern "C"
