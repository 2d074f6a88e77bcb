// Streaming .dt loader: a polygon file straight into one side of the store.
//
// The reference loads .dt files with pthreads in chunks of records
// (storage.cpp:320-449) into per-polygon objects, and its GPU path then copies
// each polygon to the device (preprocessing.cu). Here the file is mapped, its
// records are decoded by all host threads straight into pinned staging
// buffers in the store's padded ring layout (stored vertices, the closing
// copy the reference's decode appends, one pad copy), and each filled buffer
// goes to HBM with one asynchronous copy while the threads fill the next: the
// decode of chunk c+1 overlaps the transfer of chunk c, and no device-side
// repacking pass is needed.
//
// What is kept follows the reference's loader: holes are decoded and dropped
// (MyPolygon.cpp:746-759), and a polygon whose in-memory ring (stored count
// + 1) has fewer than 3 vertices is skipped (storage.cpp:341).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace farm {

namespace {

constexpr size_t kStageBytes = 256ull << 20;  // per pinned staging buffer

struct Mapping {
    int fd = -1;
    void *p = MAP_FAILED;
    size_t size = 0;
    ~Mapping() {
        if (p != MAP_FAILED) munmap(p, size);
        if (fd >= 0) close(fd);
    }
};

template <typename F>
void for_threads(int threads, uint64_t n, F f) {
    if (threads <= 1 || n < 2) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    const uint64_t per = (n + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        const uint64_t b = std::min(n, per * t), e = std::min(n, per * (t + 1));
        if (b < e) th.emplace_back([=]() { f(b, e); });
    }
    for (auto &x : th) x.join();
}

// Pinned staging buffers kept by the store between loads.
int store_staging(farm_store *s, size_t bytes, float2 **buf) {
    for (int i = 0; i < 2; i++) {
        if (s->h_stage[i] && s->h_stage_cap >= bytes) continue;
        if (s->h_stage[i]) cudaFreeHost(s->h_stage[i]);
        s->h_stage[i] = nullptr;
        FARM_CUDA(cudaHostAlloc(&s->h_stage[i], bytes, cudaHostAllocDefault));
    }
    s->h_stage_cap = std::max(s->h_stage_cap, bytes);
    for (int i = 0; i < 2; i++) {
        buf[i] = static_cast<float2 *>(s->h_stage[i]);
        if (!s->ev_stage[i]) FARM_CUDA(cudaEventCreateWithFlags(&s->ev_stage[i], cudaEventDisableTiming));
    }
    return FARM_OK;
}

}  // namespace

}  // namespace farm

using namespace farm;

extern "C" int farm_store_load_dt(farm_store *s, int side, const char *path, int threads, uint64_t *n_out) {
    if (!s || side < 0 || side > 1 || !path) {
        set_error("invalid arguments to farm_store_load_dt");
        return FARM_EINVAL;
    }
    if (side == 1 && s->n_side[0] == 0) {
        set_error("load the source side (0) before the target side (1)");
        return FARM_EINVAL;
    }
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    Mapping m;
    m.fd = open(path, O_RDONLY);
    if (m.fd < 0) {
        set_error(std::string("farm_store_load_dt: cannot open ") + path);
        return FARM_EIO;
    }
    struct stat sb;
    if (fstat(m.fd, &sb) != 0 || sb.st_size < 8) {
        set_error(std::string("farm_store_load_dt: not a .dt file: ") + path);
        return FARM_EFORMAT;
    }
    m.size = (size_t)sb.st_size;
    m.p = mmap(nullptr, m.size, PROT_READ, MAP_PRIVATE, m.fd, 0);
    if (m.p == MAP_FAILED) {
        set_error(std::string("farm_store_load_dt: cannot map ") + path);
        return FARM_EIO;
    }
    const unsigned char *base = static_cast<const unsigned char *>(m.p);
    uint64_t nrec;
    memcpy(&nrec, base + m.size - 8, 8);
    if (nrec == 0 || nrec > (m.size - 8) / 48) {
        set_error("farm_store_load_dt: bad polygon count in the .dt trailer");
        return FARM_EFORMAT;
    }
    const unsigned char *meta = base + m.size - 8 - 48 * nrec;
    const uint64_t data_end = m.size - 8 - 48 * nrec;

    // pass 1, all threads: each record's offset and stored vertex count, checked
    std::vector<uint64_t> rec_off(nrec), rec_m(nrec);
    std::atomic<uint64_t> first_bad(~0ull);
    for_threads(threads, nrec, [&](uint64_t b, uint64_t e) {
        for (uint64_t r = b; r < e; r++) {
            uint64_t o, holes, mv;
            memcpy(&o, meta + 48 * r + 8, 8);
            bool ok = o + 16 <= data_end;
            if (ok) {
                memcpy(&holes, base + o, 8);
                memcpy(&mv, base + o + 8, 8);
                ok = mv > 0 && mv <= 0x3FFFFFFFull && o + 16 + 8 * mv <= data_end;
                uint64_t q = o + 16 + 8 * mv;
                for (uint64_t h = 0; ok && h < holes; h++) {
                    uint64_t hm;
                    ok = q + 8 <= data_end;
                    if (!ok) break;
                    memcpy(&hm, base + q, 8);
                    ok = hm <= data_end && q + 8 + 8 * hm <= data_end;
                    q += 8 + 8 * hm;
                }
            }
            if (!ok) {
                uint64_t cur = first_bad.load();
                while (r < cur && !first_bad.compare_exchange_weak(cur, r)) {
                }
                continue;
            }
            rec_off[r] = o;
            rec_m[r] = mv;
        }
    });
    if (first_bad.load() != ~0ull) {
        set_error("farm_store_load_dt: record " + std::to_string(first_bad.load()) + " of " + path + " is malformed");
        return FARM_EFORMAT;
    }
    // kept records, their offsets in this side's vertex numbering
    std::vector<uint64_t> keep;
    keep.reserve(nrec);
    for (uint64_t r = 0; r < nrec; r++)
        if (rec_m[r] + 1 >= 3) keep.push_back(r);
    const uint64_t n = keep.size();
    if (n > 0x7FFFFFFFull) {
        set_error("more than 2^31 polygons on one side");
        return FARM_EOVERFLOW;
    }
    std::vector<uint64_t> h(n + 1, 0);
    for (uint64_t k = 0; k < n; k++) h[k + 1] = h[k] + rec_m[keep[k]];
    uint64_t ring_first = 0;
    FARM_TRY(stage_side(s, side, h, &ring_first));

    // pass 2: chunks of consecutive polygons, each at most one staging buffer
    // of padded rings (a larger single polygon gets a buffer of its own size)
    uint64_t biggest = 0;
    for (uint64_t k = 0; k < n; k++) biggest = std::max(biggest, h[k + 1] - h[k] + 2);
    const size_t stage = std::max(kStageBytes, (size_t)biggest * sizeof(float2));
    float2 *buf[2];
    FARM_TRY(store_staging(s, stage, buf));
    const uint64_t per_buf = stage / sizeof(float2);
    float2 *dring = s->d_ring.as<float2>() + ring_first;
    uint64_t k0 = 0;
    int slot = 0;
    bool pending[2] = {false, false};
    while (k0 < n) {
        uint64_t k1 = k0, used = 0;
        while (k1 < n && used + (h[k1 + 1] - h[k1] + 2) <= per_buf) used += h[k1 + 1] - h[k1] + 2, k1++;
        if (pending[slot]) FARM_CUDA(cudaEventSynchronize(s->ev_stage[slot]));
        float2 *dst = buf[slot];
        const uint64_t pad0 = h[k0] + 2 * k0;  // padded position of polygon k0 within this side
        // threads take equal shares of the chunk's vertices, not of its polygons
        const uint64_t v0 = h[k0], vspan = h[k1] - h[k0];
        for_threads(threads, vspan ? (uint64_t)threads : 0, [&](uint64_t tb, uint64_t te) {
            const uint64_t b = std::lower_bound(h.begin() + k0, h.begin() + k1, v0 + vspan * tb / threads) - h.begin();
            const uint64_t e = std::lower_bound(h.begin() + k0, h.begin() + k1, v0 + vspan * te / threads) - h.begin();
            for (uint64_t j = b; j < (te == (uint64_t)threads ? k1 : e); j++) {
                const uint64_t r = keep[j], mv = rec_m[r];
                float2 *o = dst + (h[j] + 2 * j - pad0);
                memcpy(o, base + rec_off[r] + 16, 8 * mv);
                o[mv] = o[0];
                o[mv + 1] = o[0];
            }
        });
        FARM_CUDA(cudaMemcpyAsync(dring + pad0, dst, used * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
        FARM_CUDA(cudaEventRecord(s->ev_stage[slot], s->stream));
        pending[slot] = true;
        slot ^= 1;
        k0 = k1;
    }
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    if (n_out) *n_out = n;
    return FARM_OK;
}
