// warmstart.cu -- tensor-core kernels of the learned FIRE warm start (sm_103a).
//
// The warm start is a small message-passing network over the polygon
// contact graph (one node per vertex, hidden width 128): every layer is a
// dense product of the node features with a weight matrix, and the
// aggregation over a node's neighbours.  No part of it has a counterpart in
// the reference; plain FIRE stays the minimiser that decides the result.
//
//   k_gemm_bf16     C[M,N] = A[M,K] B[N,K]^T (+ bias, ReLU), BF16 operands,
//                   FP32 accumulation in tensor memory: 128 x BN tiles, the
//                   K loop in 64-wide chunks through a two-stage ring that
//                   the Tensor Memory Accelerator fills (128-byte swizzle),
//                   one thread issuing tcgen05.mma (M = 128, K = 16 each) and
//                   committing to the stage's mbarrier, four warps reading
//                   the accumulator back with tcgen05.ld for the epilogue.
//                   Every wait is bounded: a wait that runs out sets an
//                   error flag (pcp_gemm_status) and the block still frees
//                   its tensor memory.
//   k_graph_sum     out[i] = scale * sum of h[j] over the neighbours j of i
//                   (CSR), BF16 in and out, FP32 sums; a warp per node.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "pcp_common.cuh"
#include "pcp_internal.h"

namespace pcp {

namespace {

constexpr int kBM = 128;           // rows of a tile (the MMA's M)
constexpr int kBK = 64;            // K per chunk: one 128-byte swizzle row of BF16
constexpr int kWaitPolls = 1 << 22;

__device__ int g_gemm_error;

__device__ __forceinline__ uint32_t saddr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bar_init(uint64_t* b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}

__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity) {
    for (int i = 0; i < kWaitPolls; ++i)
        if (bar_try(b, parity)) return true;
    atomicExch(&g_gemm_error, 1);
    return false;
}

__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes)
                 : "memory");
}

// 2-D tiled bulk tensor load: box at (x = K offset, y = row offset)
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* b) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(saddr(b))
        : "memory");
}

// Shared-memory operand descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart; the start address of a K slice moves by its byte offset
// inside the 128-byte row.
__device__ __forceinline__ uint64_t operand_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);       // start address
    d |= (uint64_t)1u << 16;                      // leading byte offset (unused when swizzled)
    d |= (uint64_t)(1024u >> 4) << 32;            // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1u << 46;                      // descriptor version
    d |= (uint64_t)2u << 61;                      // 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     saddr(b))
                 : "memory");
}

__device__ __forceinline__ void ld_16cols(uint32_t addr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
        "%12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
struct GemmSmem {
    static constexpr int kA = kBM * kBK * 2;   // 16 KB
    static constexpr int kB = BN * kBK * 2;
    static constexpr int kStage = kA + kB;     // a multiple of 1024 for every BN used
    static constexpr int kBytes = 2 * kStage + 1024;
    static constexpr int kCols = BN < 32 ? 32 : BN;   // tensor-memory columns allocated
};

template <int BN>
__global__ void __launch_bounds__(128, 1)
k_gemm_bf16(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
            float* __restrict__ C, const float* __restrict__ bias, int M, int N, int K,
            int chunksPerSplit, int relu, int atomic) {
    using S = GemmSmem<BN>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t full[2], empty[2], done;
    __shared__ uint32_t tmemSlot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         saddr(&tmemSlot)),
                     "r"(S::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 32) {
        bar_init(&full[0], 1);
        bar_init(&full[1], 1);
        bar_init(&empty[0], 1);
        bar_init(&empty[1], 1);
        bar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmemSlot;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const int chunks = (K + kBK - 1) / kBK;
    const int c0 = blockIdx.z * chunksPerSplit;
    const int nc = min(chunksPerSplit, chunks - c0);   // >= 1 (the host sizes the splits)
    constexpr uint32_t kIdesc = mma_idesc(kBM, BN);
    if (threadIdx.x == 0) {
        auto load = [&](int c, int s) {
            uint8_t* st = smem + s * S::kStage;
            bar_expect(&full[s], S::kStage);
            tma_2d(st, &mapA, (c0 + c) * kBK, m0, &full[s]);
            tma_2d(st + S::kA, &mapB, (c0 + c) * kBK, n0, &full[s]);
        };
        bool ok = true;
        int issued = 0, landed = 0;   // loads issued; loads whose wait succeeded
        load(0, 0);
        ++issued;
        for (int c = 0; c < nc && ok; ++c) {
            const int s = c & 1;
            if (c + 1 < nc) {
                // the other stage is free once the MMAs of chunk c - 1 are done
                if (c >= 1) ok = bar_wait(&empty[s ^ 1], ((c - 1) >> 1) & 1);
                if (!ok) break;
                load(c + 1, s ^ 1);
                ++issued;
            }
            ok = bar_wait(&full[s], (c >> 1) & 1);
            if (!ok) break;
            ++landed;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = saddr(smem + s * S::kStage), b = a + S::kA;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk)
                mma_bf16(tmem, operand_desc(a + kk * 32), operand_desc(b + kk * 32), kIdesc,
                         (c > 0 || kk > 0) ? 1u : 0u);
            mma_commit(&empty[s]);
        }
        if (!ok) {
            // a wait ran out: let the copies still in flight land (bounded)
            // before the block leaves, so none writes into a later block's
            // shared memory.  Those are the loads landed..issued-1, at most
            // one per stage and each the latest use of its stage, so the
            // parity of its own phase names it (an older phase's parity
            // would alias a newer one).
            for (int c = landed; c < issued; ++c) bar_wait(&full[c & 1], (c >> 1) & 1);
        }
        mma_commit(&done);   // arrives once every MMA issued above has completed
    }
    __syncwarp();
    const bool ok = bar_wait(&done, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = m0 + warp * 32 + lane;
    const bool addBias = bias != nullptr && blockIdx.z == 0;
#pragma unroll 1
    for (int cc = 0; cc < BN; cc += 16) {
        uint32_t r[16];
        ld_16cols(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc, r);
        if (ok && row < M) {
            const int col0 = n0 + cc;
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                v[j] = __uint_as_float(r[j]);
                if (addBias && col0 + j < N) v[j] += bias[col0 + j];
                if (relu) v[j] = fmaxf(v[j], 0.f);
            }
            float* dst = C + (size_t)row * N + col0;
            if (!atomic && col0 + 16 <= N && (N & 3) == 0) {
                // the 16 columns of this row: four 16-byte stores
                float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (col0 + j < N) {
                        if (atomic) atomicAdd(dst + j, v[j]);
                        else dst[j] = v[j];
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(S::kCols)
                     : "memory");
}

__global__ void __launch_bounds__(256)
k_graph_sum(const int* __restrict__ rowptr, const int* __restrict__ col,
            const __nv_bfloat162* __restrict__ h, __nv_bfloat162* __restrict__ out, int V,
            int F2, float scale) {
    const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (i >= V) return;
    const int e0 = rowptr[i], e1 = rowptr[i + 1];
    for (int f = lane; f < F2; f += 32) {
        float2 acc = make_float2(0.f, 0.f);
        for (int e = e0; e < e1; ++e) {
            const float2 v = __bfloat1622float2(h[(size_t)col[e] * F2 + f]);
            acc.x += v.x;
            acc.y += v.y;
        }
        out[(size_t)i * F2 + f] = __floats2bfloat162_rn(scale * acc.x, scale * acc.y);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// rows x K BF16, row-major; box of 64 (K) x boxRows, 128-byte swizzle;
// out-of-range boxes read zeros
bool make_map(CUtensorMap* map, const void* base, int rows, int K, int boxRows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)boxRows};
    cuuint32_t es[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
              es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, float* C, const float* bias,
                        int M, int N, int K, int splits, int relu, cudaStream_t st) {
    using S = GemmSmem<BN>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16<BN>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, S::kBytes);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int chunks = (K + kBK - 1) / kBK;
    const int per = (chunks + splits - 1) / splits;
    const int z = (chunks + per - 1) / per;   // every split gets at least one chunk
    dim3 grid((M + kBM - 1) / kBM, (N + BN - 1) / BN, z);
    k_gemm_bf16<BN><<<grid, 128, S::kBytes, st>>>(ma, mb, C, bias, M, N, K, per, relu,
                                                    z > 1 ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace

// The launchers behind the C ABI (pcp_gemm_bf16 and pcp_graph_sum_bf16 in
// model.cpp, which check the arguments first).
int launch_gemm_bf16(const void* a, const void* b, float* c, int m, int n, int k,
                     const float* bias, int relu, int splits, cudaStream_t st) {
    const int bn = n <= 16 ? 16 : n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 256;
    CUtensorMap ma, mb;
    if (!make_map(&ma, a, m, k, kBM) || !make_map(&mb, b, n, k, bn)) return -1;
    cudaError_t e;
    switch (bn) {
        case 16: e = launch_gemm<16>(ma, mb, c, bias, m, n, k, splits, relu, st); break;
        case 32: e = launch_gemm<32>(ma, mb, c, bias, m, n, k, splits, relu, st); break;
        case 64: e = launch_gemm<64>(ma, mb, c, bias, m, n, k, splits, relu, st); break;
        case 128: e = launch_gemm<128>(ma, mb, c, bias, m, n, k, splits, relu, st); break;
        default: e = launch_gemm<256>(ma, mb, c, bias, m, n, k, splits, relu, st); break;
    }
    return (int)e;
}

cudaError_t gemm_error_flag(int* out) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(out, g_gemm_error, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_gemm_error, &zero, sizeof(int));
    return e;
}

cudaError_t launch_graph_sum_bf16(const int* rowptr, const int* col, const void* h, void* out,
                                  int v, int f, float scale, cudaStream_t st) {
    k_graph_sum<<<(v + 7) / 8, 256, 0, st>>>(rowptr, col, static_cast<const __nv_bfloat162*>(h),
                                             static_cast<__nv_bfloat162*>(out), v, f / 2, scale);
    return cudaGetLastError();
}

}  // namespace pcp
