// bf16 x bf16 -> fp32 matrix product on the 5th-generation tensor cores:
// tcgen05.mma with operands in shared memory (no-swizzle K-major canonical
// layout) and the accumulator in tensor memory, read back with tcgen05.ld.
//
//   C[M][N] (fp32, row-major) = A[M][K] * B[N][K]^T     (A, B bf16, K-major)
//
// One CTA of 128 threads per 128 x 128 output tile and K segment (split-K for
// long K: the segments' partial products are added into C, which then has to
// start at zero).  Per 64-wide K slice the
// four warps stage both operand tiles in shared memory, one thread issues
// four MMAs (K = 16 each) and commits them to an mbarrier; the CTA waits for
// the commit before the next slice overwrites the tiles.  Each warp then
// reads its 32 accumulator rows (TMEM lanes 32w..32w+31) and stores them.
// Every mbarrier wait is bounded; a wait that runs out sets *err and the CTA
// skips the rest of its work (it still frees its tensor memory).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ldo_umma {

constexpr int TM = 128, TN = 128, TK = 64;
constexpr int CORE_BYTES = 128;                    // 8 rows x 16 bytes
constexpr int LBO = CORE_BYTES;                    // next core matrix along K
constexpr int SBO = (TK / 8) * CORE_BYTES;         // next 8-row group (1024 B)
constexpr int TILE_BYTES = TM * TK * 2;            // 16 KB per operand tile
constexpr unsigned WAIT_LIMIT = 1u << 26;

// Instruction descriptor, kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N = TN, M = TM.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((LBO >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((SBO >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Byte offset of element (row r, k) of a tile in the canonical layout.
__device__ __forceinline__ int tile_off(int r, int k) {
    return (r >> 3) * SBO + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned n = 0; n < WAIT_LIMIT; ++n) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Stage rows [r0, r0+128) x cols [k0, k0+64) of a K-major bf16 matrix
// (rows x K, row stride K) into a tile; rows >= rows and columns >= klim are
// zero.
__device__ __forceinline__ void stage_tile(unsigned char* tile, const uint16_t* __restrict__ src, int rows, int K,
                                           int klim, int r0, int k0) {
    // 128 rows x 8 chunks of 8 elements (16 bytes)
    for (int e = threadIdx.x; e < TM * (TK / 8); e += blockDim.x) {
        int r = e >> 3, c = e & 7;
        int gr = r0 + r, gk = k0 + c * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gr < rows) {
            const uint16_t* p = src + (size_t)gr * K + gk;
            if (gk + 8 <= klim && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
                v = *reinterpret_cast<const uint4*>(p);
            }
            else {
                uint16_t t[8];
                #pragma unroll
                for (int q = 0; q < 8; ++q) t[q] = (gk + q < klim) ? p[q] : (uint16_t)0;
                v = *reinterpret_cast<uint4*>(t);
            }
        }
        *reinterpret_cast<uint4*>(tile + tile_off(r, c * 8)) = v;
    }
}

__global__ void __launch_bounds__(128) gemm_tn_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                      float* __restrict__ C, int M, int N, int K, int k_per,
                                                      int* err) {
    __shared__ __align__(1024) unsigned char sA[TILE_BYTES];
    __shared__ __align__(1024) unsigned char sB[TILE_BYTES];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tmem_slot;
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    uint32_t bar = smem_u32(&mbar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"((uint32_t)TN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    uint32_t tmem = tmem_slot;

    bool ok = true;
    uint32_t parity = 0;
    int kb = blockIdx.z * k_per;
    int ke = min(K, kb + k_per);
    int nk = ke > kb ? (ke - kb + TK - 1) / TK : 0;
    bool split = gridDim.z > 1;
    for (int kt = 0; kt < nk && ok; ++kt) {
        stage_tile(sA, A, M, K, ke, m0, kb + kt * TK);
        stage_tile(sB, B, N, K, ke, n0, kb + kt * TK);
        // generic-proxy stores -> visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
            #pragma unroll
            for (int kk = 0; kk < TK / 16; ++kk) {
                uint64_t ad = smem_desc(a0 + kk * 2 * LBO);
                uint64_t bd = smem_desc(b0 + kk * 2 * LBO);
                uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                         : "memory");
        }
        __syncwarp();
        bool done = mbar_wait(bar, parity);
        parity ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // one outcome for the whole CTA: a wait that ran out anywhere stops it
        ok = __syncthreads_and(done) != 0;
        if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    }

    if (ok && nk > 0) {
        int row = m0 + warp * 32 + lane;
        #pragma unroll 1
        for (int c0 = 0; c0 < TN; c0 += 32) {
            uint32_t v[32];
            uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (row < M) {
                #pragma unroll
                for (int j = 0; j < 32; ++j) {
                    int col = n0 + c0 + j;
                    if (col < N) {
                        if (split) atomicAdd(&C[(size_t)row * N + col], __uint_as_float(v[j]));
                        else C[(size_t)row * N + col] = __uint_as_float(v[j]);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"((uint32_t)TN)
                     : "memory");
    }
}

// splits > 1: K is cut into that many segments of whole 64-wide slices whose
// products are added into C (C must be zero on entry).
inline cudaError_t gemm_tn(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K, int* err,
                           cudaStream_t s, int splits = 1) {
    int slices = (K + TK - 1) / TK;
    if (splits < 1) splits = 1;
    if (splits > slices) splits = slices > 0 ? slices : 1;
    int k_per = ((slices + splits - 1) / splits) * TK;
    splits = (K + k_per - 1) / k_per;
    if (splits < 1) splits = 1;
    dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM, splits);
    gemm_tn_kernel<<<grid, 128, 0, s>>>(A, B, C, M, N, K, k_per, err);
    return cudaGetLastError();
}

} // namespace ldo_umma
