// BF16 tensor-core kernels of the learned corrector (tcgen05 MMA, FP32 accumulation in tensor
// memory).  This file holds the general GEMM used by training; the fused per-particle inference
// kernel lives in corrector.cu.
//
// k_tc_gemm: D[M][N] = A[M][K] . B[N][K]^T, bf16 operands row-major in global memory, float32 D.
// A CTA of 128 threads owns a 128-row block of D (all N columns, N <= 256, in one TMEM allocation)
// and a K range; per 64-wide K chunk every thread copies 16-byte vectors of A and B into the K-major
// core-matrix layout of tc.cuh, one thread issues four K = 16 MMAs and commits them to an mbarrier,
// and the CTA waits (bounded) before the next chunk overwrites the tiles.  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows of D) and stores or, for
// split-K, adds it to D.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"

namespace ffmpm {
namespace {

constexpr int kGemmThreads = 128;
constexpr int kKChunk = 64;
constexpr uint32_t kChunkSBO = (kKChunk / 8) * 128;  // 8-row groups of a 64-wide K chunk: 1 KB apart

template <int BN>
__global__ void __launch_bounds__(kGemmThreads) k_tc_gemm(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                          float* __restrict__ D, int M, int N, int K, int k_per_split,
                                                          int add_out, int32_t* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sa = smem;                   // 128 x 64 bf16
  unsigned char* sb = smem + 128 * kKChunk * 2;  // BN x 64 bf16
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  constexpr uint32_t kCols = BN < 32 ? 32 : BN;
  constexpr uint32_t kIdesc = tc::idesc_bf16_f32(128, BN);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128;
  const int kbeg = blockIdx.y * k_per_split;
  const int kend = min(K, kbeg + k_per_split);
  if (warp == 0) tc::tmem_alloc(&tmem_base, kCols);
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
    s_fail = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  uint32_t phase = 0;
  bool issued = false;
  for (int k0 = kbeg; k0 < kend; k0 += kKChunk) {
    for (int v = tid; v < 128 * 8; v += kGemmThreads) {
      const int r = v >> 3, c = v & 7;
      const uint4 val = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + 8 * c);
      *reinterpret_cast<uint4*>(sa + tc::kmajor_offset(r, 8 * c, kChunkSBO)) = val;
    }
    for (int v = tid; v < BN * 8; v += kGemmThreads) {
      const int r = v >> 3, c = v & 7;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (r < N) val = *reinterpret_cast<const uint4*>(B + (size_t)r * K + k0 + 8 * c);
      *reinterpret_cast<uint4*>(sb + tc::kmajor_offset(r, 8 * c, kChunkSBO)) = val;
    }
    fence_proxy_async_shared();  // generic-proxy smem writes -> visible to the tensor core
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint32_t a0 = tc::smem_addr(sa), b0 = tc::smem_addr(sb);
#pragma unroll
      for (int s = 0; s < kKChunk / 16; ++s)
        tc::mma_bf16(tmem, tc::make_desc(a0 + 256u * s, tc::kLBO, kChunkSBO),
                     tc::make_desc(b0 + 256u * s, tc::kLBO, kChunkSBO), kIdesc, issued || s > 0);
      tc::commit(&bar);
    }
    issued = true;
    if (!mbar_wait(&bar, phase)) s_fail = 1;
    phase ^= 1u;
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (s_fail) break;
  }
  if (s_fail) {
    if (tid == 0 && status) raise_status(status, FFMPM_STATUS_TIMEOUT);
  } else if (issued) {
    const int row = m0 + 32 * warp + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tc::taddr_of(tmem, 32u * warp, c0), v);
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = c0 + j;
          if (col < N) {
            if (add_out)
              atomicAdd(&D[(size_t)row * N + col], v[j]);
            else
              D[(size_t)row * N + col] = v[j];
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, kCols);
}

template <int BN>
int launch_gemm(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, int split, int32_t* status,
                cudaStream_t s) {
  const size_t smem = size_t(128 + BN) * kKChunk * 2;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_tc_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  const int chunks = K / kKChunk;
  split = std::max(1, std::min(split, chunks));
  const int per = (chunks + split - 1) / split * kKChunk;
  const int gy = (K + per - 1) / per;
  dim3 grid(M / 128, gy);
  k_tc_gemm<BN><<<grid, kGemmThreads, smem, s>>>(A, B, D, M, N, K, per, gy > 1 ? 1 : 0, status);
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

}  // namespace
}  // namespace ffmpm

using namespace ffmpm;

extern "C" {

int ffmpm_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* D, int32_t M, int32_t N, int32_t K,
                       int32_t split_k, int32_t* status, void* stream) {
  if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0) return FFMPM_ERR_BADARG;
  if (M % 128 || N % 16 || N > 256 || K % kKChunk) return FFMPM_ERR_BADARG;
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int split = std::max(1, (int)split_k);
  if (N <= 16) return launch_gemm<16>(A, B, D, M, N, K, split, status, s);
  if (N <= 32) return launch_gemm<32>(A, B, D, M, N, K, split, status, s);
  if (N <= 64) return launch_gemm<64>(A, B, D, M, N, K, split, status, s);
  if (N <= 128) return launch_gemm<128>(A, B, D, M, N, K, split, status, s);
  return launch_gemm<256>(A, B, D, M, N, K, split, status, s);
}

}  // extern "C"
