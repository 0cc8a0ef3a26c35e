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
    if (tid == 0) {
      if (status) raise_status(status, FFMPM_STATUS_TIMEOUT);
      // the MMAs of the last commit may still be running: wait for them once more (bounded) before
      // their tensor memory is freed
      mbar_wait(&bar, phase ^ 1u);
    }
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

// ---------------------------------------------------------------------------------------------
// Training: elementwise kernels between the GEMMs.
constexpr int kEw = 256;

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
// d/dz GELU(z) = Phi(z) + z phi(z)
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.3989422804014327f * expf(-0.5f * z * z);
}

// Z (float [B][N]) += bias, kept for the backward pass; H = act(Z) as bf16 [B][N] and, when Ht is
// given, its transpose [N][B].
__global__ void __launch_bounds__(kEw) k_bias_act(float* __restrict__ Z, const float* __restrict__ bias, int B, int N,
                                                  int act, uint16_t* __restrict__ H, uint16_t* __restrict__ Ht) {
  const int64_t i = (int64_t)blockIdx.x * kEw + threadIdx.x;
  if (i >= (int64_t)B * N) return;
  const int row = (int)(i / N), col = (int)(i % N);
  const float z = Z[i] + bias[col];
  Z[i] = z;
  const uint16_t h = tc::bf16_bits(act ? gelu_f(z) : z);
  H[i] = h;
  if (Ht) Ht[(size_t)col * B + row] = h;
}

// X [B][K] -> Xt [K][B] (bf16); rows k >= kmax of Xt are zeroed (the buffer is strided by B).
__global__ void __launch_bounds__(kEw) k_transpose_bf16(const uint16_t* __restrict__ X, int B, int K, int kmax,
                                                        uint16_t* __restrict__ Xt) {
  const int64_t i = (int64_t)blockIdx.x * kEw + threadIdx.x;
  if (i >= (int64_t)B * K) return;
  const int row = (int)(i / K), col = (int)(i % K);
  Xt[(size_t)col * B + row] = col < kmax ? X[(size_t)row * K + col] : uint16_t(0);
}

// Weighted squared error of Y (+ b4) against T; dY = 2 w (pred - T) / B as bf16 [B][64] (zero beyond
// 12) and its transpose [12..][B]; db4 += column sums; *loss += the loss.
__global__ void __launch_bounds__(kEw) k_loss_grad(const float* __restrict__ Y, const float* __restrict__ b4,
                                                   const float* __restrict__ T, const float* __restrict__ w, int B,
                                                   uint16_t* __restrict__ dY, uint16_t* __restrict__ dYt,
                                                   float* __restrict__ db4, double* __restrict__ loss) {
  __shared__ float s_db[FFMPM_MLP_OUT];
  __shared__ double s_loss;
  if (threadIdx.x < FFMPM_MLP_OUT) s_db[threadIdx.x] = 0.f;
  if (threadIdx.x == 0) s_loss = 0.0;
  __syncthreads();
  const int row = blockIdx.x * kEw + threadIdx.x;
  double l = 0.0;
  if (row < B) {
    const float invB = 1.f / float(B);
#pragma unroll
    for (int j = 0; j < FFMPM_MLP_OUT; ++j) {
      const float e = Y[(size_t)row * 16 + j] + b4[j] - T[(size_t)row * FFMPM_MLP_OUT + j];
      l += double(w[j]) * double(e) * double(e);
      const float g = 2.f * w[j] * e * invB;
      const uint16_t gb = tc::bf16_bits(g);
      dY[(size_t)row * 64 + j] = gb;
      dYt[(size_t)j * B + row] = gb;
      atomicAdd(&s_db[j], g);
    }
#pragma unroll
    for (int j = FFMPM_MLP_OUT; j < 64; ++j) dY[(size_t)row * 64 + j] = 0;
    for (int j = FFMPM_MLP_OUT; j < 128; ++j) dYt[(size_t)j * B + row] = 0;  // padding rows of the transpose
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&s_loss, l);
  __syncthreads();
  if (threadIdx.x < FFMPM_MLP_OUT) atomicAdd(&db4[threadIdx.x], s_db[threadIdx.x]);
  if (threadIdx.x == 0) atomicAdd(loss, s_loss / double(B));
}

// dZ = dH * GELU'(Z) as bf16 [B][64] and transpose [64..][B]; db += column sums.
__global__ void __launch_bounds__(kEw) k_act_back(const float* __restrict__ dH, const float* __restrict__ Z, int B,
                                                  uint16_t* __restrict__ dZ, uint16_t* __restrict__ dZt,
                                                  float* __restrict__ db) {
  __shared__ float s_db[64];
  if (threadIdx.x < 64) s_db[threadIdx.x] = 0.f;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kEw + threadIdx.x;
  if (i < (int64_t)B * 64) {
    const int row = (int)(i >> 6), col = (int)(i & 63);
    const float g = dH[i] * gelu_grad(Z[i]);
    const uint16_t gb = tc::bf16_bits(g);
    dZ[i] = gb;
    dZt[(size_t)col * B + row] = gb;
    dZt[(size_t)(col + 64) * B + row] = 0;  // padding rows 64..127 of the transpose
    atomicAdd(&s_db[col], g);
  }
  __syncthreads();
  if (threadIdx.x < 64) atomicAdd(&db[threadIdx.x], s_db[threadIdx.x]);
}

__global__ void __launch_bounds__(kEw) k_adam(float* __restrict__ p, const float* __restrict__ g,
                                              float* __restrict__ m, float* __restrict__ v, int count, float lr,
                                              float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * kEw + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// params -> bf16 W1 [64][128], W2/W3 [64][64], W4 [16][64] (rows >= 12 zero) and W2t/W3t/W4t [64][64].
__global__ void __launch_bounds__(kEw) k_pack(const float* __restrict__ P, uint16_t* W1, uint16_t* W2, uint16_t* W3,
                                              uint16_t* W4, uint16_t* W2t, uint16_t* W3t, uint16_t* W4t) {
  const int i = blockIdx.x * kEw + threadIdx.x;
  if (i < 64 * 128) W1[i] = tc::bf16_bits(P[FFMPM_MLP_OFF_W1 + i]);
  if (i < 64 * 64) {
    const int r = i >> 6, c = i & 63;
    W2[i] = tc::bf16_bits(P[FFMPM_MLP_OFF_W2 + i]);
    W3[i] = tc::bf16_bits(P[FFMPM_MLP_OFF_W3 + i]);
    W2t[c * 64 + r] = W2[i];
    W3t[c * 64 + r] = W3[i];
    // W4t[h][j] = W4[j][h] for the 12 outputs j, zero for j >= 12
    const float w4 = r < FFMPM_MLP_OUT ? P[FFMPM_MLP_OFF_W4 + r * 64 + c] : 0.f;
    W4t[c * 64 + r] = tc::bf16_bits(w4);
    if (r < 16) W4[r * 64 + c] = tc::bf16_bits(w4);
  }
}

int ew_grid(int64_t n) { return (int)((n + kEw - 1) / kEw); }

int gemm(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, int split, int32_t* st, cudaStream_t s) {
  if (N <= 16) return launch_gemm<16>(A, B, D, M, N, K, split, st, s);
  if (N <= 64) return launch_gemm<64>(A, B, D, M, N, K, split, st, s);
  return launch_gemm<128>(A, B, D, M, N, K, split, st, s);
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

int ffmpm_mlp_train_forward(const ffmpm_mlp_trainer* t, const uint16_t* X, int32_t B, void* stream) {
  if (!t || !X || B <= 0 || B % 128 || B > t->max_batch || (reinterpret_cast<uintptr_t>(X) & 15)) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const float* P = t->params;
  int rc = FFMPM_OK;
  k_transpose_bf16<<<ew_grid((int64_t)B * FFMPM_MLP_IN), kEw, 0, s>>>(X, B, FFMPM_MLP_IN, FFMPM_MLP_FEATURES, t->Xt);
  rc |= gemm(X, t->W1, t->Z1, B, 64, FFMPM_MLP_IN, 1, t->status, s);
  k_bias_act<<<ew_grid((int64_t)B * 64), kEw, 0, s>>>(t->Z1, P + FFMPM_MLP_OFF_B1, B, 64, 1, t->H1, t->H1t);
  rc |= gemm(t->H1, t->W2, t->Z2, B, 64, 64, 1, t->status, s);
  k_bias_act<<<ew_grid((int64_t)B * 64), kEw, 0, s>>>(t->Z2, P + FFMPM_MLP_OFF_B2, B, 64, 1, t->H2, t->H2t);
  rc |= gemm(t->H2, t->W3, t->Z3, B, 64, 64, 1, t->status, s);
  k_bias_act<<<ew_grid((int64_t)B * 64), kEw, 0, s>>>(t->Z3, P + FFMPM_MLP_OFF_B3, B, 64, 1, t->H3, t->H3t);
  rc |= gemm(t->H3, t->W4, t->Y, B, 16, 64, 1, t->status, s);
  if (rc != FFMPM_OK) return FFMPM_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

int ffmpm_mlp_train_backward(const ffmpm_mlp_trainer* t, const float* T, const float* w, int32_t B, double* loss,
                             void* stream) {
  if (!t || !T || !w || !loss || B <= 0 || B % 128 || B > t->max_batch) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float* G = t->grads;
  const float* P = t->params;
  const int split = std::max(1, std::min(2 * sm_count(), B / 1024));
  int rc = FFMPM_OK;
  cudaMemsetAsync(G, 0, sizeof(float) * FFMPM_MLP_PARAMS, s);
  k_loss_grad<<<ew_grid(B), kEw, 0, s>>>(t->Y, P + FFMPM_MLP_OFF_B4, T, w, B, t->dY, t->dYt, G + FFMPM_MLP_OFF_B4, loss);
  // layer 4: dW4 = dY^T H3, dH3 = dY W4
  rc |= gemm(t->dYt, t->H3t, G + FFMPM_MLP_OFF_W4, 128, 64, B, split, t->status, s);
  rc |= gemm(t->dY, t->W4t, t->dH, B, 64, 64, 1, t->status, s);
  k_act_back<<<ew_grid((int64_t)B * 64), kEw, 0, s>>>(t->dH, t->Z3, B, t->dZ, t->dZt, G + FFMPM_MLP_OFF_B3);
  // layer 3
  rc |= gemm(t->dZt, t->H2t, G + FFMPM_MLP_OFF_W3, 128, 64, B, split, t->status, s);
  rc |= gemm(t->dZ, t->W3t, t->dH, B, 64, 64, 1, t->status, s);
  k_act_back<<<ew_grid((int64_t)B * 64), kEw, 0, s>>>(t->dH, t->Z2, B, t->dZ, t->dZt, G + FFMPM_MLP_OFF_B2);
  // layer 2
  rc |= gemm(t->dZt, t->H1t, G + FFMPM_MLP_OFF_W2, 128, 64, B, split, t->status, s);
  rc |= gemm(t->dZ, t->W2t, t->dH, B, 64, 64, 1, t->status, s);
  k_act_back<<<ew_grid((int64_t)B * 64), kEw, 0, s>>>(t->dH, t->Z1, B, t->dZ, t->dZt, G + FFMPM_MLP_OFF_B1);
  // layer 1: dW1 = dZ1^T X
  rc |= gemm(t->dZt, t->Xt, G + FFMPM_MLP_OFF_W1, 128, 128, B, split, t->status, s);
  if (rc != FFMPM_OK) return FFMPM_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

int ffmpm_mlp_train_update(const ffmpm_mlp_trainer* t, float lr, float beta1, float beta2, float eps, int32_t step,
                           void* stream) {
  if (!t || step < 1) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<ew_grid(FFMPM_MLP_PARAMS), kEw, 0, s>>>(t->params, t->grads, t->adam_m, t->adam_v, FFMPM_MLP_PARAMS, lr,
                                                  beta1, beta2, eps, c1, c2);
  k_pack<<<ew_grid(64 * 128), kEw, 0, s>>>(t->params, t->W1, t->W2, t->W3, t->W4, t->W2t, t->W3t, t->W4t);
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

}  // extern "C"
