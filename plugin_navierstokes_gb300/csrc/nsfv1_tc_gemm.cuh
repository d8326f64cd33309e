// BF16 GEMM on the 5th-generation tensor cores of sm_103a: C = A * B^T with
// A [M x K] and B [N x K] both row-major (K contiguous), FP32 accumulation in
// tensor memory, operands staged into shared memory by TMA tensor copies
// (cp.async.bulk.tensor, 128-byte swizzle) through a STAGES-deep mbarrier ring.
//
// One CTA = 128 threads computes one 128 x BN tile of C over one K chunk
// (split-K: blockIdx.z selects the chunk; its partial goes to C + z*M*N):
//   warp 0, one lane : TMA producer
//   warp 1, one lane : tcgen05.mma issuer (kind::f16, BF16 x BF16 -> F32)
//   all 4 warps      : epilogue, tcgen05.ld of the accumulator (warp w owns
//                      TMEM lanes 32w..32w+31 = rows of the tile) -> global.
// Every wait is bounded by the global timer; a timeout sets *err and the CTA
// still drains what it issued and frees its tensor memory before returning.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace nsfv1 {
namespace tc {

constexpr int BM = 128;          // rows per tile = TMEM lanes
constexpr int BK = 64;           // K per stage: 64 BF16 = 128 bytes = one swizzle span
constexpr int UK = 16;           // K per tcgen05.mma (kind::f16)
constexpr unsigned long long kWaitNs = 1000000000ull;   // 1 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the phase of the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kWaitNs) return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// shared-memory matrix descriptor of a K-major tile written by TMA with the
// 128-byte swizzle: rows of 128 bytes, 8-row atoms 1024 bytes apart (SBO),
// descriptor version 1, swizzle mode 2 (128B); LBO is unused for this layout.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)2 << 61);
}

// instruction descriptor of kind::f16: D F32, A and B BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <int BN, int STAGES>
struct GemmSmem {
    static constexpr int kA = BM * BK * 2;        // 16 KB
    static constexpr int kB = BN * BK * 2;        // BN * 128 bytes
    static constexpr int kStage = kA + kB;
    static constexpr int kBytes = STAGES * kStage + 1024 /* align */ + 256 /* barriers */;
};

// C[z][M][N] = A[M][kz..] * B[N][kz..]^T over K chunk z of kChunk columns.
// M % 128 == 0, N % BN == 0, K % 64 == 0, kChunk % 64 == 0 (host-checked).
template <int BN, int STAGES>
__global__ void __launch_bounds__(128, 1)
    k_gemm_bf16_tn(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, float* __restrict__ C,
                   int M, int N, int K, int kChunk, int* err) {
    static_assert(BN % 32 == 0 && BN >= 32 && BN <= 256, "tile N");
    extern __shared__ uint8_t smem_raw[];
    using S = GemmSmem<BN, STAGES>;
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(base + STAGES * S::kStage);
    uint32_t* tmemSlot = (uint32_t*)(bars + 2 * STAGES + 1);
    const uint32_t fullBar = smem_u32(bars), emptyBar = fullBar + 8 * STAGES, doneBar = fullBar + 16 * STAGES;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int k0 = blockIdx.z * kChunk;
    const int kEnd = min(K, k0 + kChunk);
    const int nk = (kEnd - k0) / BK;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;   // power of two >= 32

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { mbar_init(fullBar + 8 * s, 1); mbar_init(emptyBar + 8 * s, 1); }
        mbar_init(doneBar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)), "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmemSlot;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // producer
        int issued = 0;
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % STAGES;
            if (kt >= STAGES && !mbar_wait(emptyBar + 8 * s, ((kt / STAGES) & 1) ^ 1)) { ok = false; break; }
            const uint32_t sa = smem_u32(base + s * S::kStage), sb = sa + S::kA;
            mbar_expect_tx(fullBar + 8 * s, S::kStage);
            tma_load_2d(sa, &mapA, k0 + kt * BK, m0, fullBar + 8 * s);
            tma_load_2d(sb, &mapB, k0 + kt * BK, n0, fullBar + 8 * s);
            ++issued;
        }
        // drain: every issued copy has landed before the CTA may exit
        for (int kt = (issued > STAGES ? issued - STAGES : 0); kt < issued; ++kt)
            if (!mbar_wait(fullBar + 8 * (kt % STAGES), (kt / STAGES) & 1)) ok = false;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = idesc_bf16(BM, BN);
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % STAGES;
            if (!mbar_wait(fullBar + 8 * s, (kt / STAGES) & 1)) { ok = false; break; }
            fence_after();
            const uint32_t sa = smem_u32(base + s * S::kStage), sb = sa + S::kA;
#pragma unroll
            for (int k = 0; k < BK / UK; ++k)
                mma_bf16(tmem, sw128_desc(sa + k * UK * 2), sw128_desc(sb + k * UK * 2), idesc, (kt | k) != 0);
            mma_commit(emptyBar + 8 * s);
        }
        mma_commit(doneBar);   // arrives once every MMA issued above has completed
    }
    __syncwarp();
    // epilogue
    // warp-uniform: tcgen05.ld below is a .sync.aligned instruction
    const bool done = __all_sync(0xffffffffu, mbar_wait(doneBar, 0));
    fence_after();
    if (!done) ok = false;
    if (done && nk > 0) {
        const int row = m0 + warp * 32 + lane;
        float* crow = C + ((size_t)blockIdx.z * M + row) * N + n0;
#pragma unroll 1
        for (int c = 0; c < BN; c += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c, v);
#pragma unroll
            for (int i = 0; i < 32; i += 4) *(float4*)(crow + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
    } else if (done) {
        const int row = m0 + warp * 32 + lane;
        float* crow = C + ((size_t)blockIdx.z * M + row) * N + n0;
        for (int c = 0; c < BN; c += 4) *(float4*)(crow + c) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (!ok) atomicOr(err, 4);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

}  // namespace tc
}  // namespace nsfv1
