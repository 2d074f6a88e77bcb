// Store lifetime, ring upload and the C ABI plumbing (errors, device info,
// raster inspection). Replaces the reference's cuda_create_buffer /
// preprocess_for_gpu (src/cuda/preprocessing.cu:5-358): rings go to HBM once,
// in a 64-bit-offset layout, and the store owns every device allocation.
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

#include "common.cuh"

namespace farm {

void mlp_free(void *p);  // mlp.cu

static thread_local std::string g_error;

void set_error(const std::string &msg) { g_error = msg; }

int cuda_fail(cudaError_t e, const char *what) {
    g_error = std::string(what) + ": " + cudaGetErrorString(e);
    return FARM_ECUDA;
}

int DevBuf::ensure(size_t bytes) {
    if (bytes <= cap && p) return FARM_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        set_error("device allocation of " + std::to_string(want) + " bytes failed");
        return FARM_ENOMEM;
    }
    cap = want;
    return FARM_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

// SM count of the current device, looked up once per device ordinal (hosts
// may mix GPU models, and grids are sized from this).
int sm_count() {
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        dev = 0;
    }
    if (dev < kMaxDev) {
        int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 1;
    }
    if (dev < kMaxDev) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

// Pairs whose source index is >= n_src or target index >= n_tgt.
__global__ void k_check_pairs(const uint32_t *__restrict__ pairs, uint64_t n, uint64_t n_src, uint64_t n_tgt,
                              unsigned long long *__restrict__ bad) {
    unsigned long long mine = 0;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 p = reinterpret_cast<const uint2 *>(pairs)[k];
        mine += (p.x >= n_src) | (p.y >= n_tgt);
    }
    if (mine) atomicAdd(bad, mine);
}

int check_pair_limits(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, uint64_t n_first,
                      uint64_t n_second, const char *who, const char *first_name, const char *second_name) {
    if (!n) return FARM_OK;
    uint64_t bad = 0, first = ~0ull;
    if (mem == FARM_MEM_HOST) {
        for (uint64_t k = 0; k < n; k++)
            if (pairs[2 * k] >= n_first || pairs[2 * k + 1] >= n_second) {
                if (!bad) first = k;
                bad++;
            }
    } else {
        FARM_TRY(s->d_check.ensure(64));
        unsigned long long *d = s->d_check.as<unsigned long long>();
        FARM_CUDA(cudaMemsetAsync(d, 0, 8, s->stream));
        unsigned blocks = grid_for(n, 256);
        if (blocks > 8u * (unsigned)sm_count()) blocks = 8u * (unsigned)sm_count();
        k_check_pairs<<<blocks, 256, 0, s->stream>>>(pairs, n, n_first, n_second, d);
        FARM_CUDA(cudaGetLastError());
        unsigned long long h = 0;
        FARM_CUDA(cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, s->stream));
        FARM_CUDA(cudaStreamSynchronize(s->stream));
        bad = h;
    }
    if (bad) {
        std::string m = std::string(who) + ": " + std::to_string(bad) + " pair index(es) out of range (" +
                        std::to_string(n_first) + " " + first_name + ", " + std::to_string(n_second) + " " +
                        second_name + ")";
        if (first != ~0ull) m += ", first at pair " + std::to_string(first);
        set_error(m);
        return FARM_EINVAL;
    }
    return FARM_OK;
}

int check_pairs(farm_store *s, const uint32_t *pairs, uint64_t n, int mem, bool self, const char *who) {
    return check_pair_limits(s, pairs, n, mem, s->n_side[0], self ? s->n_side[0] : s->n_side[1], who, "sources",
                             "targets");
}

// Copy stored rings into the padded layout: per polygon the stored vertices,
// then a copy of the first (the vertex the reference's decode appends,
// vertex_sequence.cpp:206-219) and one more copy as the pad vertex read by the
// whole-ring sequence of single-pixel polygons (Ideal.cpp:523-529).
__global__ void k_pad_rings(const float2 *__restrict__ xy, const uint64_t *__restrict__ off, uint32_t npoly,
                            uint64_t first_poly, float2 *__restrict__ ring) {
    // off: this side's slice of the concatenated (global) vertex offsets;
    // xy: this side's vertices, indexed from its own first vertex
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t base = off[0];
    uint64_t total = off[npoly] - base;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < total; v += stride) {
        uint64_t gv = v + base;
        uint32_t p = find_segment(off, npoly, gv);
        uint64_t gp = first_poly + p;
        float2 q = xy[v];
        ring[gv + 2 * gp] = q;
        if (gv == off[p]) {
            uint64_t end = off[p + 1] + 2 * gp;
            ring[end] = q;
            ring[end + 1] = q;
        }
    }
}

}  // namespace farm

using namespace farm;

farm::StoreView farm_store::view() const {
    farm::StoreView v;
    v.ring = d_ring.as<float2>();
    v.hdr = d_hdr.as<PolyHdr>();
    v.status = d_status.as<uint8_t>();
    v.offset = d_offset.as<uint32_t>();
    v.seq = d_seq.as<uint2>();
    v.hoff = d_hoff.as<uint32_t>();
    v.hnodes = d_hnodes.as<double>();
    v.voff = d_voff.as<uint32_t>();
    v.vnodes = d_vnodes.as<double>();
    v.areas = d_areas.as<double>();
    v.category_count = ropts.category_count ? ropts.category_count : 16;
    return v;
}

extern "C" {

const char *farm_last_error(void) { return g_error.c_str(); }

int farm_device_info(int *ordinal, char *name, size_t name_len) {
    int dev = 0;
    FARM_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    FARM_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (ordinal) *ordinal = dev;
    if (name && name_len) {
        strncpy(name, prop.name, name_len - 1);
        name[name_len - 1] = 0;
    }
    return FARM_OK;
}

int farm_store_create(farm_store **out) {
    if (!out) {
        set_error("null output pointer");
        return FARM_EINVAL;
    }
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device is available");
        return FARM_ECUDA;
    }
    farm_store *s = new (std::nothrow) farm_store();
    if (!s) {
        set_error("host allocation failed");
        return FARM_ENOMEM;
    }
    cudaGetDevice(&s->device);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return cuda_fail(cudaGetLastError(), "cudaStreamCreate");
    }
    for (auto &ev : s->ev) cudaEventCreate(&ev);
    *out = s;
    return FARM_OK;
}

void farm_store_destroy(farm_store *s) {
    if (!s) return;
    cudaStreamSynchronize(s->stream);
    farm::mlp_free(s->mlp);
    s->mlp = nullptr;
    DevBuf *bufs[] = {&s->d_xy_in, &s->d_off, &s->d_ring, &s->d_hdr, &s->d_status, &s->d_offset, &s->d_seq,
                      &s->d_hoff, &s->d_hnodes, &s->d_voff, &s->d_vnodes, &s->d_areas, &s->cub_tmp,
                      &s->d_pairs, &s->d_out, &s->d_counters, &s->d_check, &s->d_points};
    for (DevBuf *b : bufs) b->release();
    for (auto &b : s->s) b.release();
    for (auto &ev : s->ev)
        if (ev) cudaEventDestroy(ev);
    for (int i = 0; i < 2; i++) {
        if (s->h_stage[i]) cudaFreeHost(s->h_stage[i]);
        if (s->ev_stage[i]) cudaEventDestroy(s->ev_stage[i]);
    }
    cudaStreamDestroy(s->stream);
    delete s;
}

int farm_store_device_bytes(farm_store *s, uint64_t *bytes) {
    if (!s || !bytes) {
        set_error("invalid arguments to farm_store_device_bytes");
        return FARM_EINVAL;
    }
    const DevBuf *bufs[] = {&s->d_xy_in, &s->d_off, &s->d_ring, &s->d_hdr, &s->d_status, &s->d_offset, &s->d_seq,
                            &s->d_hoff, &s->d_hnodes, &s->d_voff, &s->d_vnodes, &s->d_areas, &s->cub_tmp,
                            &s->d_pairs, &s->d_out, &s->d_counters, &s->d_check, &s->d_points};
    uint64_t t = 0;
    for (const DevBuf *b : bufs) t += b->cap;
    for (const auto &b : s->s) t += b.cap;
    *bytes = t;
    return FARM_OK;
}

int farm_sync(farm_store *s) {
    if (!s) return FARM_EINVAL;
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    return FARM_OK;
}

}  // extern "C"

namespace farm {

// Book a side's polygons in the store: per-side offsets (h, from 0), the
// concatenated offsets of both sides on the device, and room in the padded
// ring array, where polygon p's ring starts at cat[p] + 2p (the source side
// first, so a target side appends in place when it fits). *ring_first gets
// the float2 index of this side's first ring. The device offsets are copied
// from s->h_cat, which stays valid until the next call.
int stage_side(farm_store *s, int side, std::vector<uint64_t> h, uint64_t *ring_first) {
    const uint64_t n = h.size() - 1;
    s->rasterized = false;
    if (side == 0) {  // a new source side drops any target side
        s->n_side[1] = 0;
        s->h_off[1].clear();
    }
    s->h_off[side] = std::move(h);
    s->n_side[side] = n;
    const uint64_t n0 = s->n_side[0], n1 = s->n_side[1];
    const uint64_t t0 = s->h_off[0][n0], t1 = n1 ? s->h_off[1][n1] : 0;
    std::vector<uint64_t> &cat = s->h_cat;
    cat.assign(n0 + n1 + 1, 0);
    for (uint64_t k = 0; k <= n0; k++) cat[k] = s->h_off[0][k];
    for (uint64_t k = 1; k <= n1; k++) cat[n0 + k] = t0 + s->h_off[1][k];
    const uint64_t total = t0 + t1;
    const size_t need = (total + 2 * (n0 + n1)) * sizeof(float2) + 64;
    if (need > s->d_ring.cap) {
        DevBuf nr;
        FARM_TRY(nr.ensure(need + need / 8));
        if (side == 1 && s->d_ring.p)
            FARM_CUDA(cudaMemcpyAsync(nr.p, s->d_ring.p, (t0 + 2 * n0) * sizeof(float2), cudaMemcpyDeviceToDevice,
                                      s->stream));
        FARM_CUDA(cudaStreamSynchronize(s->stream));
        s->d_ring.release();
        s->d_ring = nr;
        nr.p = nullptr;
    }
    FARM_TRY(s->d_off.ensure((n0 + n1 + 1) * 8));
    FARM_CUDA(cudaMemcpyAsync(s->d_off.p, cat.data(), (n0 + n1 + 1) * 8, cudaMemcpyHostToDevice, s->stream));
    *ring_first = side == 0 ? 0 : t0 + 2 * n0;
    s->n_poly = n0 + n1;
    s->n_edges = total;
    return FARM_OK;
}

}  // namespace farm

extern "C" {

int farm_store_load(farm_store *s, int side, uint64_t n, const uint64_t *off, const float *xy, int mem) {
    if (!s || side < 0 || side > 1 || !off || (n && !xy)) {
        set_error("invalid arguments to farm_store_load");
        return FARM_EINVAL;
    }
    if (n > 0x7FFFFFFFull) {
        set_error("more than 2^31 polygons on one side");
        return FARM_EOVERFLOW;
    }
    if (side == 1 && s->n_side[0] == 0) {
        set_error("load the source side (0) before the target side (1)");
        return FARM_EINVAL;
    }
    std::vector<uint64_t> h(n + 1);
    if (mem == FARM_MEM_DEVICE)
        FARM_CUDA(cudaMemcpy(h.data(), off, (n + 1) * 8, cudaMemcpyDeviceToHost));
    else
        memcpy(h.data(), off, (n + 1) * 8);
    for (uint64_t k = 0; k < n; k++) {
        if (h[k + 1] < h[k] + 2) {
            set_error("polygon " + std::to_string(k) + " has fewer than 2 stored vertices");
            return FARM_EINVAL;
        }
        if (h[k + 1] - h[k] > 0x3FFFFFFFull) {
            set_error("polygon " + std::to_string(k) + " exceeds 2^30 vertices");
            return FARM_EOVERFLOW;
        }
    }
    const uint64_t o0 = h[0];
    for (auto &v : h) v -= o0;
    const uint64_t side_total = h[n];
    uint64_t ring_first = 0;
    FARM_TRY(stage_side(s, side, std::move(h), &ring_first));
    const float2 *src;
    if (mem == FARM_MEM_DEVICE) {
        // the padding kernel reads whole (x, y) pairs: 8-byte loads
        if (reinterpret_cast<uintptr_t>(xy + 2 * o0) & 7u) {
            set_error("farm_store_load: device vertices must start on an 8-byte boundary");
            return FARM_EINVAL;
        }
        src = reinterpret_cast<const float2 *>(xy) + o0;
    } else {
        // Pinned host memory is read by the padding kernel itself over the
        // host link (the device address the runtime reports for it), with no
        // staging copy; pageable memory is copied into a staging buffer first.
        // (only at an 8-byte boundary, as the kernel's loads are of whole pairs)
        cudaPointerAttributes pa;
        const void *mapped = nullptr;
        if (cudaPointerGetAttributes(&pa, xy + 2 * o0) == cudaSuccess) {
            if (pa.type == cudaMemoryTypeHost && pa.devicePointer &&
                (reinterpret_cast<uintptr_t>(pa.devicePointer) & 7u) == 0)
                mapped = pa.devicePointer;
        } else {
            cudaGetLastError();
        }
        if (mapped) {
            src = reinterpret_cast<const float2 *>(mapped);
        } else {
            FARM_TRY(s->d_xy_in.ensure(side_total * sizeof(float2) + 16));
            FARM_CUDA(cudaMemcpyAsync(s->d_xy_in.p, xy + 2 * o0, side_total * sizeof(float2),
                                      cudaMemcpyHostToDevice, s->stream));
            src = s->d_xy_in.as<float2>();
        }
    }
    const uint64_t first_poly = side == 0 ? 0 : s->n_side[0];
    if (n) {
        unsigned blocks = grid_for(side_total, 256);
        unsigned cap = 32u * (unsigned)sm_count();
        if (blocks > cap) blocks = cap;
        k_pad_rings<<<blocks, 256, 0, s->stream>>>(src, s->d_off.as<uint64_t>() + first_poly, (uint32_t)n,
                                                   first_poly, s->d_ring.as<float2>());
        FARM_CUDA(cudaGetLastError());
        s->launches++;
    }
    FARM_CUDA(cudaStreamSynchronize(s->stream));
    return FARM_OK;
}

__global__ void k_collect_err(const PolyHdr *__restrict__ hdr, uint64_t first, uint64_t n, int32_t *__restrict__ out) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        out[k] = hdr[first + k].err;
}

int farm_raster_errors(farm_store *s, int side, int32_t *err, uint64_t n) {
    if (!s || side < 0 || side > 1 || n != s->n_side[side] || (n && !err)) {
        set_error("invalid arguments to farm_raster_errors");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("store is not rasterized");
        return FARM_EINVAL;
    }
    if (!n) return FARM_OK;
    int32_t *d = nullptr;
    FARM_CUDA(cudaMalloc(&d, 4 * n));
    uint64_t first = side == 0 ? 0 : s->n_side[0];
    k_collect_err<<<grid_for(n, 256) > 4096 ? 4096 : grid_for(n, 256), 256, 0, s->stream>>>(
        s->d_hdr.as<PolyHdr>(), first, n, d);
    cudaError_t e = cudaMemcpyAsync(err, d, 4 * n, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "farm_raster_errors");
    return FARM_OK;
}

int farm_raster_fetch(farm_store *s, int side, uint64_t index, farm_raster_view *v, uint8_t *status,
                      uint32_t *offset, uint32_t *seq, uint32_t *hoff, double *hnodes, uint32_t *voff, double *vnodes,
                      double *areas, double *layer_info) {
    if (!s || !v || side < 0 || side > 1 || index >= s->n_side[side]) {
        set_error("invalid arguments to farm_raster_fetch");
        return FARM_EINVAL;
    }
    if (!s->rasterized) {
        set_error("store is not rasterized");
        return FARM_EINVAL;
    }
    uint64_t p = (side == 0 ? 0 : s->n_side[0]) + index;
    PolyHdr h;
    FARM_CUDA(cudaMemcpy(&h, s->d_hdr.as<PolyHdr>() + p, sizeof h, cudaMemcpyDeviceToHost));
    memcpy(v->mbr, h.mbr, sizeof h.mbr);
    v->dimx = h.dimx;
    v->dimy = h.dimy;
    v->step_x = h.step_x;
    v->step_y = h.step_y;
    v->nv = h.nv;
    v->status_size = h.status_size;
    v->n_seq = h.n_seq;
    v->n_hnodes = h.n_hnodes;
    v->n_vnodes = h.n_vnodes;
    v->num_layers = h.num_layers;
    v->err = h.err;
    if (status) FARM_CUDA(cudaMemcpy(status, s->d_status.as<uint8_t>() + h.st, h.status_size, cudaMemcpyDeviceToHost));
    if (offset)
        FARM_CUDA(cudaMemcpy(offset, s->d_offset.as<uint32_t>() + h.off, 4ull * (h.P + 1), cudaMemcpyDeviceToHost));
    if (seq) FARM_CUDA(cudaMemcpy(seq, s->d_seq.as<uint2>() + h.seq, 8ull * h.n_seq, cudaMemcpyDeviceToHost));
    if (hoff)
        FARM_CUDA(cudaMemcpy(hoff, s->d_hoff.as<uint32_t>() + h.hline, 4ull * (h.dimy + 2), cudaMemcpyDeviceToHost));
    if (hnodes && h.n_hnodes)
        FARM_CUDA(cudaMemcpy(hnodes, s->d_hnodes.as<double>() + h.hnode, 8ull * h.n_hnodes, cudaMemcpyDeviceToHost));
    if (voff)
        FARM_CUDA(cudaMemcpy(voff, s->d_voff.as<uint32_t>() + h.vline, 4ull * (h.dimx + 2), cudaMemcpyDeviceToHost));
    if (vnodes && h.n_vnodes)
        FARM_CUDA(cudaMemcpy(vnodes, s->d_vnodes.as<double>() + h.vnode, 8ull * h.n_vnodes, cudaMemcpyDeviceToHost));
    if (areas) FARM_CUDA(cudaMemcpy(areas, s->d_areas.as<double>() + h.pix, 8ull * h.P, cudaMemcpyDeviceToHost));
    if (layer_info) {
        for (uint32_t i = 0; i < h.num_layers; i++) {
            LayerGeom g;
            layer_geom(h, i, g);
            double *o = layer_info + 7 * i;
            o[0] = g.mbr[0];
            o[1] = g.mbr[1];
            o[2] = g.mbr[2];
            o[3] = g.mbr[3];
            o[4] = g.step_x;
            o[5] = g.step_y;
            o[6] = (double)g.dimx * 65536.0 * 65536.0 + (double)g.dimy;  // packed dims
            (void)o;
        }
    }
    return FARM_OK;
}

}  // extern "C"
