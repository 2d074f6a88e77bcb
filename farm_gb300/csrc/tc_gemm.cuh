// tcgen05 (5th-generation tensor core) GEMM for sm_103a, hand-written PTX.
//
//   C[M x N] (fp32 accumulate) = A[M x K] * B[N x K]^T, A and B bf16, K-major
//
// One CTA (4 warps) computes a 128 x BN tile: operands are staged by all
// threads into shared memory in the canonical no-swizzle K-major layout
// (8 x 16-byte core matrices; LBO = distance between K-adjacent cores, SBO =
// distance between M/N-adjacent 8-row groups), one elected thread issues
// tcgen05.mma.cta_group::1.kind::f16 (K = 16 per instruction) into a TMEM
// accumulator, and tcgen05.commit arrives on an mbarrier per stage (two
// stages, so loading chunk k+1 overlaps the MMAs of chunk k). The epilogue
// reads TMEM with tcgen05.ld (warp w owns lanes 32w..32w+31 = tile rows) and
// hands 16 columns at a time to a functor. Every mbarrier wait is bounded;
// on timeout the CTA records an error, still frees its TMEM, and returns.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace farm {
namespace tc {

constexpr int kBM = 128;          // tile rows (MMA M)
constexpr int kBK = 64;           // K per stage
constexpr int kThreads = 128;     // 4 warps
constexpr uint32_t kLBO = 128;    // K-adjacent core matrices
constexpr uint32_t kSBO = 1024;   // 8-row groups (8 cores of 128 B along K)
constexpr long kSpinLimit = 1L << 26;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared memory matrix descriptor (no swizzle, descriptor version 1)
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    return d;
}

// instruction descriptor: D f32, A/B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

// bounded wait on phase `parity`; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    uint32_t a = smem_addr(bar);
    for (long i = 0; i < kSpinLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 16 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row, k) of a [rows x 64] bf16 tile in core-matrix layout
__device__ __forceinline__ uint32_t tile_off(uint32_t row, uint32_t k) {
    return (row >> 3) * kSBO + (k >> 3) * kLBO + (row & 7) * 16 + (k & 7) * 2;
}

// Stage a [rows x 64] slice of a row-major bf16 matrix (ld elements per row)
// into the core-matrix layout, 16 bytes per access; rows >= nrows and columns
// >= ncols read as zero.
__device__ __forceinline__ void stage_tile(unsigned char *dst, const __nv_bfloat16 *src, int ld, int row0, int nrows,
                                           int k0, int ncols, int rows) {
    const int vecs = rows * 8;  // 8 x 16 B per row of 64 bf16
    for (int v = threadIdx.x; v < vecs; v += kThreads) {
        int r = v >> 3, kc = v & 7;
        int gr = row0 + r, gk = k0 + kc * 8;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (gr < nrows && gk < ncols) val = *reinterpret_cast<const uint4 *>(src + (size_t)gr * ld + gk);
        *reinterpret_cast<uint4 *>(dst + tile_off((uint32_t)r, (uint32_t)(kc * 8))) = val;
    }
}

// Tile GEMM body. smem: 2 stages x (A 16 KB + B BN x 128 B) + barriers.
// epi(row, col0, v[16]) is called for every row < M and 16-column group < N.
template <int BN, typename Epi>
__device__ void gemm_tile(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                          int m0, int n0, unsigned char *smem, int *err, Epi epi) {
    static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "MMA N");
    constexpr uint32_t kTmemCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    constexpr uint32_t kA = kBM * kBK * 2, kB = BN * kBK * 2;
    unsigned char *sA[2] = {smem, smem + kA + kB};
    unsigned char *sB[2] = {smem + kA, smem + 2 * kA + kB};
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * (kA + kB));  // [0],[1] stages, [2] final
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 3);
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot, kTmemCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = make_idesc(kBM, BN);
    const int nk = (K + kBK - 1) / kBK;
    uint32_t phase[2] = {0, 0};
    bool ok = true;
    for (int kc = 0; kc < nk; kc++) {
        int s = kc & 1;
        if (kc >= 2) {  // the MMAs that read this stage two chunks ago must be done
            ok = ok && mbar_wait(&bar[s], phase[s]);
            phase[s] ^= 1;
        }
        stage_tile(sA[s], A, lda, m0, M, kc * kBK, K, kBM);
        stage_tile(sB[s], B, ldb, n0, N, kc * kBK, K, BN);
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
        if (threadIdx.x == 0 && ok) {
#pragma unroll
            for (int kk = 0; kk < kBK / 16; kk++) {
                uint64_t ad = make_desc(smem_addr(sA[s]) + kk * 2 * kLBO);
                uint64_t bd = make_desc(smem_addr(sB[s]) + kk * 2 * kLBO);
                mma_bf16(tmem, ad, bd, idesc, (kc > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&bar[s]);
        }
    }
    // the final commit tracks every MMA issued before it: once it arrives no
    // MMA can still write the accumulator, so TMEM may be read and freed
    if (threadIdx.x == 0) mma_commit(&bar[2]);
    bool fin = mbar_wait(&bar[2], 0) && ok;
    fence_after_sync();
    __syncthreads();
    if (!fin) {
        if (threadIdx.x == 0) atomicExch(err, 1);
    } else {
        const int row = warp * 32 + (threadIdx.x & 31);
        for (int c = 0; c < BN; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            if (m0 + row < M && n0 + c < N) epi(m0 + row, n0 + c, v);
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

template <int BN>
constexpr int smem_bytes() {
    return 2 * (kBM * kBK * 2 + BN * kBK * 2) + 64;
}

}  // namespace tc
}  // namespace farm
