// Learned-corrector G2P: the 3D G2P of a coarse substep (three_d/g2p.py:9-59) fused with a
// per-particle MLP that corrects its result, run on the 5th-generation tensor cores.
//
// One CTA = 128 threads = 128 particles per tile (persistent over tiles); thread t owns particle
// (tile * 128 + t) and TMEM lane t, i.e. row t of every MLP layer.  Per tile:
//   1. each thread gathers its 27 stencil nodes from the updated grid, forms v', C', F' and x' as the
//      plain G2P does (node velocities taken relative to the stencil's centre node u), and writes
//      its 128 bf16 features into row t of the K-major input tile in shared memory:
//        [0, 9)   F' - I            [9, 18)  C' dt            [18, 21) (v' - u) dt / dx
//        [21,102) (v_i - u) dt / dx for the 27 nodes i
//        [102,104) mu k, lam k      [104,113) PF k (the stress of this step's P2G)      [113,128) 0
//      with k = dt^2 / (rho dx^2) (stiffness and stress in units of the step's own CFL number
//      squared), each multiplied by the network's per-feature input scale;
//   2. four MMA layers 128->64->64->64->16 (GELU between), bf16 operands, FP32 accumulators in
//      TMEM; after each layer every thread reads its own row back (tcgen05.ld), adds the bias,
//      applies GELU and writes the bf16 row of the next layer's operand;
//   3. outputs y[0,12) times the output scale: F' += y[0,9), v' += y[9,12) dx / dt, x' += dt * that.
// Weights (bf16, K-major) and biases stay in shared memory for the whole launch.  Modes: apply the
// network, export the features (no network), or both off (the plain coarse G2P through the same
// arithmetic).  Every mbarrier wait is bounded.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "mpm_kernels.cuh"
#include "tc.cuh"

namespace ffmpm {
namespace {

constexpr int kIn = FFMPM_MLP_IN;    // 128 inputs (FFMPM_MLP_FEATURES used)
constexpr int kHid = FFMPM_MLP_HIDDEN;
constexpr int kOutPad = 16;
constexpr int kOut = FFMPM_MLP_OUT;  // 12
constexpr uint32_t kSboIn = (kIn / 8) * 128;
constexpr uint32_t kSboHid = (kHid / 8) * 128;
constexpr int kThreadsC = 128;
constexpr uint32_t kTmemCols = 128;  // [0, 64): hidden layers, [64, 80): output layer

struct SmemLayout {
  static constexpr size_t w1 = 0;
  static constexpr size_t w2 = w1 + size_t(kHid) * kIn * 2;
  static constexpr size_t w3 = w2 + size_t(kHid) * kHid * 2;
  static constexpr size_t w4 = w3 + size_t(kHid) * kHid * 2;
  static constexpr size_t x = w4 + size_t(kOutPad) * kHid * 2;
  static constexpr size_t h = x + size_t(128) * kIn * 2;
  static constexpr size_t f = h + size_t(128) * kHid * 2;  // floats: b1 b2 b3 b4 in_scale out_scale
  static constexpr int nf = 3 * kHid + kOutPad + kIn + kOutPad;
  static constexpr size_t total = f + sizeof(float) * nf;
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }

// Copy a bf16 row-major [rows][k] matrix into the K-major core-matrix layout.
__device__ __forceinline__ void stage_kmajor(unsigned char* dst, const uint16_t* src, int rows, int k, uint32_t sbo) {
  const int vecs = k / 8;
  for (int v = threadIdx.x; v < rows * vecs; v += blockDim.x) {
    const int r = v / vecs, c = v % vecs;
    *reinterpret_cast<uint4*>(dst + tc::kmajor_offset(r, 8 * c, sbo)) =
        *reinterpret_cast<const uint4*>(src + (size_t)r * k + 8 * c);
  }
}

// Two consecutive features (k even) of row r as one 32-bit shared store.
__device__ __forceinline__ void put2(unsigned char* tile, int r, int k, uint32_t sbo, float a, float b) {
  const uint32_t w = uint32_t(tc::bf16_bits(a)) | (uint32_t(tc::bf16_bits(b)) << 16);
  *reinterpret_cast<uint32_t*>(tile + tc::kmajor_offset(r, k, sbo)) = w;
}

__device__ __forceinline__ void put1(unsigned char* tile, int r, int k, uint32_t sbo, float a) {
  *reinterpret_cast<uint16_t*>(tile + tc::kmajor_offset(r, k, sbo)) = tc::bf16_bits(a);
}

// Order-preserving float -> int key (for atomicMin / atomicMax on signed floats).
__device__ __forceinline__ int float_key(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}

template <bool kApply, bool kExport>
__global__ void __launch_bounds__(kThreadsC) k_corrector(KParams<float> kp, const float* __restrict__ gv,
                                                         PView<float> P, uint32_t n, ffmpm_mlp net,
                                                         uint16_t* __restrict__ feat_out, int* __restrict__ det_keys,
                                                         int32_t* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sW1 = smem + SmemLayout::w1;
  unsigned char* sW2 = smem + SmemLayout::w2;
  unsigned char* sW3 = smem + SmemLayout::w3;
  unsigned char* sW4 = smem + SmemLayout::w4;
  unsigned char* sX = smem + SmemLayout::x;
  unsigned char* sH = smem + SmemLayout::h;
  float* sf = reinterpret_cast<float*>(smem + SmemLayout::f);
  float* sb1 = sf;
  float* sb2 = sb1 + kHid;
  float* sb3 = sb2 + kHid;
  float* sb4 = sb3 + kHid;
  float* s_in = sb4 + kOutPad;
  float* s_out = s_in + kIn;
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int i = tid; i < kIn; i += kThreadsC) s_in[i] = net.in_scale ? net.in_scale[i] : 1.f;
  if (kApply) {
    stage_kmajor(sW1, net.W1, kHid, kIn, kSboIn);
    stage_kmajor(sW2, net.W2, kHid, kHid, kSboHid);
    stage_kmajor(sW3, net.W3, kHid, kHid, kSboHid);
    stage_kmajor(sW4, net.W4, kOutPad, kHid, kSboHid);
    for (int i = tid; i < kHid; i += kThreadsC) {
      sb1[i] = net.b1[i];
      sb2[i] = net.b2[i];
      sb3[i] = net.b3[i];
    }
    for (int i = tid; i < kOutPad; i += kThreadsC) {
      sb4[i] = net.b4[i];
      s_out[i] = net.out_scale[i];
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, kTmemCols);
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
    s_fail = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = kApply ? tmem_base : 0u;
  const uint32_t lane_base = 32u * warp;
  uint32_t phase = 0;
  const float dt = kp.dt, inv_dx = kp.inv_dx;
  const float vs = dt * inv_dx;  // velocity -> cells per step
  float dmin = 3.4e38f, dmax = -3.4e38f;

  for (uint32_t tile = blockIdx.x; tile * 128u < n; tile += gridDim.x) {
    const uint32_t p = tile * 128u + tid;
    bool valid = p < n;
    float xo[3], Fo[9], Co[9], vo[3];
    if (valid) {
      float x[3], F[9], fx[3], w[3][3];  // pre-step state and stencil
      int b[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) x[d] = P.x[P.at(p, d, 3)];
#pragma unroll
      for (int i = 0; i < 9; ++i) F[i] = P.F[P.at(p, i, 9)];
      bool ok = true;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        ok = ok && base_of(x[d], inv_dx, kp.res, b[d], fx[d]);
        float ww[3];
        bspline(fx[d], ww);
        w[0][d] = ww[0];
        w[1][d] = ww[1];
        w[2][d] = ww[2];
      }
      if (!ok) {
        raise_status(status, FFMPM_STATUS_OOB);
        valid = false;
      } else {
        const int R = kp.res + 1;
        const size_t cn = ((size_t)(b[0] + 1) * R + (b[1] + 1)) * R + (b[2] + 1);
        const float u[3] = {gv[3 * cn + 0], gv[3 * cn + 1], gv[3 * cn + 2]};
        float v[3] = {0.f, 0.f, 0.f}, C[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        int node = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k, ++node) {
              const float wt = w[i][0] * w[j][1] * w[k][2];
              const size_t gi = ((size_t)(b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
              const float d0 = gv[3 * gi + 0] - u[0], d1 = gv[3 * gi + 1] - u[1], d2 = gv[3 * gi + 2] - u[2];
              const float r0 = float(i) - fx[0], r1 = float(j) - fx[1], r2 = float(k) - fx[2];
              v[0] += wt * d0;
              v[1] += wt * d1;
              v[2] += wt * d2;
              C[0] += wt * d0 * r0; C[1] += wt * d0 * r1; C[2] += wt * d0 * r2;
              C[3] += wt * d1 * r0; C[4] += wt * d1 * r1; C[5] += wt * d1 * r2;
              C[6] += wt * d2 * r0; C[7] += wt * d2 * r1; C[8] += wt * d2 * r2;
              const int f0 = 21 + 3 * node;  // features of node `node`
              put1(sX, tid, f0, kSboIn, d0 * vs * s_in[f0]);
              put1(sX, tid, f0 + 1, kSboIn, d1 * vs * s_in[f0 + 1]);
              put1(sX, tid, f0 + 2, kSboIn, d2 * vs * s_in[f0 + 2]);
            }
        const float c4 = 4.f * inv_dx;
#pragma unroll
        for (int i = 0; i < 9; ++i) Co[i] = C[i] * c4;
#pragma unroll
        for (int d = 0; d < 3; ++d) vo[d] = u[d] + v[d];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            Fo[r * 3 + c] = F[r * 3 + c] + dt * (Co[r * 3 + 0] * F[0 * 3 + c] + Co[r * 3 + 1] * F[1 * 3 + c] +
                                                 Co[r * 3 + 2] * F[2 * 3 + c]);
#pragma unroll
        for (int d = 0; d < 3; ++d) xo[d] = x[d] + dt * vo[d];
        // features 0..20, then zero padding 102..127
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          put1(sX, tid, i, kSboIn, (Fo[i] - (i % 4 == 0 ? 1.f : 0.f)) * s_in[i]);
          put1(sX, tid, 9 + i, kSboIn, Co[i] * dt * s_in[9 + i]);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) put1(sX, tid, 18 + d, kSboIn, v[d] * vs * s_in[18 + d]);
        // material and stress features 102..112 (from the pre-step F, as the P2G of this step)
        {
          float m_, mu_, lam_;
          lame_of(kp, P, p, m_, mu_, lam_);
          const float kk = dt * dt * inv_dx * inv_dx * kp.volume / m_;
          float FmR[9];
          if (!f_minus_r_small_strain3(F, FmR)) {
            float Rr[9];
            polar3<float>(F, Rr, nullptr);
#pragma unroll
            for (int i = 0; i < 9; ++i) FmR[i] = F[i] - Rr[i];
          }
          const float J = det3(F);
          const float sc = lam_ * (J - 1.f) * J;
          put1(sX, tid, 102, kSboIn, mu_ * kk * s_in[102]);
          put1(sX, tid, 103, kSboIn, lam_ * kk * s_in[103]);
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              float pf = (a == c || kp.model != FFMPM_MODEL_FIXED_COROTATED) ? sc : 0.f;
#pragma unroll
              for (int e = 0; e < 3; ++e) pf += 2.f * mu_ * FmR[a * 3 + e] * F[c * 3 + e];
              put1(sX, tid, 104 + a * 3 + c, kSboIn, pf * kk * s_in[104 + a * 3 + c]);
            }
          for (int k = 113; k < 120; ++k) put1(sX, tid, k, kSboIn, 0.f);
          *reinterpret_cast<uint4*>(sX + tc::kmajor_offset(tid, 120, kSboIn)) = make_uint4(0u, 0u, 0u, 0u);
        }
      }
    }
    if (!valid) {
#pragma unroll
      for (int k = 0; k < kIn; k += 8)
        *reinterpret_cast<uint4*>(sX + tc::kmajor_offset(tid, k, kSboIn)) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (kExport && valid) {
      uint4* dst = reinterpret_cast<uint4*>(feat_out + (size_t)p * kIn);
#pragma unroll
      for (int c = 0; c < kIn / 8; ++c) dst[c] = *reinterpret_cast<const uint4*>(sX + tc::kmajor_offset(tid, 8 * c, kSboIn));
    }
    if (kApply) {
      float y[16];
#pragma unroll 1
      for (int layer = 0; layer < 4; ++layer) {
        fence_proxy_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
          const unsigned char* A = layer == 0 ? sX : sH;
          const unsigned char* B = layer == 0 ? sW1 : layer == 1 ? sW2 : layer == 2 ? sW3 : sW4;
          const int ksteps = (layer == 0 ? kIn : kHid) / 16;
          const uint32_t sbo = layer == 0 ? kSboIn : kSboHid;
          const uint32_t idesc = layer == 3 ? tc::idesc_bf16_f32(128, kOutPad) : tc::idesc_bf16_f32(128, kHid);
          const uint32_t d = tmem + (layer == 3 ? 64u : 0u);
          const uint32_t a0 = tc::smem_addr(A), b0 = tc::smem_addr(B);
          for (int s = 0; s < ksteps; ++s)
            tc::mma_bf16(d, tc::make_desc(a0 + 256u * s, tc::kLBO, sbo), tc::make_desc(b0 + 256u * s, tc::kLBO, sbo),
                         idesc, s > 0);
          tc::commit(&bar);
        }
        if (!mbar_wait(&bar, phase)) s_fail = 1;
        phase ^= 1u;
        tc::fence_after_sync();
        __syncthreads();
        if (s_fail) break;
        if (layer < 3) {
          const float* bias = layer == 0 ? sb1 : layer == 1 ? sb2 : sb3;
#pragma unroll 1
          for (int c0 = 0; c0 < kHid; c0 += 16) {
            float a[16];
            tc::tmem_ld16(tc::taddr_of(tmem, lane_base, c0), a);
#pragma unroll
            for (int j = 0; j < 16; j += 2)
              put2(sH, tid, c0 + j, kSboHid, gelu(a[j] + bias[c0 + j]), gelu(a[j + 1] + bias[c0 + j + 1]));
          }
        } else {
          tc::tmem_ld16(tc::taddr_of(tmem, lane_base, 64u), y);
        }
      }
      if (s_fail) break;
      if (valid) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Fo[i] += (y[i] + sb4[i]) * s_out[i];
        const float inv_vs = 1.f / vs;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float dv = (y[9 + d] + sb4[9 + d]) * s_out[9 + d] * inv_vs;
          vo[d] += dv;
          xo[d] += dt * dv;
        }
      }
    }
    if (valid) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        P.x[P.at(p, d, 3)] = xo[d];
        P.v[P.at(p, d, 3)] = vo[d];
      }
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        P.F[P.at(p, i, 9)] = Fo[i];
        P.C[P.at(p, i, 9)] = Co[i];
      }
      const float J = det3(Fo);
      dmin = fminf(dmin, J);
      dmax = fmaxf(dmax, J);
    }
    // the next tile rewrites sX / sH: every thread is past this tile's MMAs and reads
    __syncthreads();
  }
  if (s_fail && tid == 0) {
    raise_status(status, FFMPM_STATUS_TIMEOUT);
    // the MMAs of the last commit may still be running: wait for them once more (bounded) before
    // their tensor memory is freed
    mbar_wait(&bar, phase ^ 1u);
  }
  if (det_keys) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
      dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    }
    if ((tid & 31) == 0 && dmin <= dmax) {
      atomicMin(&det_keys[0], float_key(dmin));
      atomicMax(&det_keys[1], float_key(dmax));
    }
  }
  if (kApply) {
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, kTmemCols);
  }
}

template <bool A, bool E>
int launch_corrector(const ffmpm_params& p, const ffmpm_grid& g, ffmpm_particles& Pp, const ffmpm_mlp* net,
                     uint16_t* feat, int* det_keys, int32_t* status, cudaStream_t s) {
  auto kern = k_corrector<A, E>;
  const size_t smem = SmemLayout::total;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    attr = true;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreadsC, smem) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  {
    // CTAs per SM that the shared memory holds (each CTA also takes 1 KB reserved by the system)
    int dev = 0, smem_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int by_smem = smem_sm / (int)(smem + 2048);
    per_sm = std::max(per_sm, std::min(by_smem, 4));
  }
  const int64_t tiles = (Pp.n + 127) / 128;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, int64_t(sm_count()) * std::max(1, per_sm)));
  ffmpm_mlp nn{};
  if (net) nn = *net;
  kern<<<grid, kThreadsC, smem, s>>>(kparams<float>(p), static_cast<const float*>(g.velocity), pview<float>(Pp),
                                     (uint32_t)Pp.n, nn, feat, det_keys, status);
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

}  // namespace
}  // namespace ffmpm

using namespace ffmpm;

extern "C" {

int ffmpm_corrector_g2p(const ffmpm_params* p, const ffmpm_grid* grid, ffmpm_particles* P, const ffmpm_mlp* net,
                        uint16_t* features_out, int32_t* det_range, int32_t* status, void* stream) {
  if (!p || !grid || !grid->velocity || !P || P->n < 0 || P->n > int64_t(0x7FFFFFFF)) return FFMPM_ERR_BADARG;
  if (p->dim != 3 || p->real_bytes != 4) return FFMPM_ERR_UNSUPPORTED;
  if (P->stride != 0 && P->stride < P->n) return FFMPM_ERR_BADARG;
  if (P->n == 0) return FFMPM_OK;
  if (!P->x || !P->v || !P->F || !P->C) return FFMPM_ERR_BADARG;
  if (net && (!net->W1 || !net->W2 || !net->W3 || !net->W4 || !net->b1 || !net->b2 || !net->b3 || !net->b4 ||
              !net->out_scale))
    return FFMPM_ERR_BADARG;
  if (features_out && (reinterpret_cast<uintptr_t>(features_out) & 15)) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ffmpm_particles Q = *P;
  if (net && features_out) return launch_corrector<true, true>(*p, *grid, Q, net, features_out, det_range, status, s);
  if (net) return launch_corrector<true, false>(*p, *grid, Q, net, nullptr, det_range, status, s);
  if (features_out) return launch_corrector<false, true>(*p, *grid, Q, nullptr, features_out, det_range, status, s);
  return launch_corrector<false, false>(*p, *grid, Q, nullptr, nullptr, det_range, status, s);
}

}  // extern "C"
