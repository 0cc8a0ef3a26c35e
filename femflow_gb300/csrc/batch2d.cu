// Batched 2D MLS-MPM: many independent scenes (each with its own particles, grid resolution,
// material, dt and walls) advanced by ONE persistent cooperative launch per substep.
//
// Phases of a substep, separated by a grid-wide barrier (bounded spin; co-residency of all CTAs is
// guaranteed by the cooperative launch):
//   1. P2G over every particle of every scene: stress (utils.py:52-92) + 9-node scatter with one
//      vector red per node into the scene's grid A (two_d/p2g.py:11-76)
//   2. grid update over every node of every scene: two_d/grid_op.py:5-24 into B, A re-zeroed
//   3. G2P over every particle: gather v and C from B, advect, F update, Jp (two_d/g2p.py:5-47)
// Scenes are located from a global particle (or node) index by binary search in an offset table
// held in shared memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "mpm_kernels.cuh"

namespace ffmpm {
namespace {

constexpr int kMaxScenes = FFMPM_BATCH2D_MAX_SCENES;
constexpr uint32_t kBarrierSpins = 1u << 24;  // default bound of one grid-barrier wait

struct BatchHeader {
  int32_t status;
  uint32_t barrier_count;
  uint32_t barrier_gen;
  int32_t nscenes;
  int64_t total_particles;
  int64_t total_nodes;
  uint32_t wait_limit;  // grid-barrier wait bound (0: kBarrierSpins), ffmpm_batch2d_set_waits
  uint32_t inject;      // FFMPM_INJECT_* bits (tests only)
  uint32_t pad[54];
};
static_assert(sizeof(BatchHeader) == 256, "one 256-byte line");

struct BatchLayout {
  size_t off_scenes, off_poffs, off_noffs, off_gridA, off_gridB, total;
  int64_t total_nodes;
};

template <typename T>
size_t node_bytes() {
  return 4 * sizeof(T);
}

bool batch_layout(const ffmpm_scene2d* sc, int nscenes, int real_bytes, BatchLayout* L) {
  if (!sc || nscenes < 1 || nscenes > kMaxScenes || (real_bytes != 4 && real_bytes != 8)) return false;
  int64_t nodes = 0;
  for (int i = 0; i < nscenes; ++i) {
    if (sc[i].res < 3 || sc[i].res > 4096 || sc[i].count < 0 || sc[i].offset < 0) return false;
    nodes += int64_t(sc[i].res + 1) * (sc[i].res + 1);
  }
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  size_t off = sizeof(BatchHeader);
  L->off_scenes = off;
  off = up(off + sizeof(ffmpm_scene2d) * nscenes);
  L->off_poffs = off;
  off = up(off + sizeof(int64_t) * (nscenes + 1));
  L->off_noffs = off;
  off = up(off + sizeof(int64_t) * (nscenes + 1));
  L->off_gridA = off;
  off = up(off + size_t(4) * real_bytes * nodes);
  L->off_gridB = off;
  off = up(off + size_t(4) * real_bytes * nodes);
  L->total = off;
  L->total_nodes = nodes;
  return true;
}

// Grid-wide barrier with a bounded wait.  Returns false (and raises FFMPM_STATUS_TIMEOUT) if the
// other CTAs did not arrive in time; the caller then leaves the kernel.
__device__ __forceinline__ bool grid_barrier(BatchHeader* h, int* s_fail, uint32_t limit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* genp = &h->barrier_gen;
    const uint32_t gen = *genp;
    __threadfence();
    const uint32_t arrived = atomicAdd(&h->barrier_count, 1u) + 1u;
    if (arrived == gridDim.x) {
      h->barrier_count = 0;
      __threadfence();
      atomicAdd(&h->barrier_gen, 1u);
    } else {
      uint32_t spins = 0;
      while (*genp == gen) {
        if (++spins > limit) {
          raise_status(&h->status, FFMPM_STATUS_TIMEOUT);
          *s_fail = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *s_fail == 0;
}

__device__ __forceinline__ int find_scene(const int64_t* offs, int n, int64_t gi) {
  int lo = 0, hi = n;  // offs[lo] <= gi < offs[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (offs[mid] <= gi)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

template <typename T>
__device__ __forceinline__ KParams<T> scene_kparams(const ffmpm_scene2d& s) {
  KParams<T> k;
  k.dx = T(s.dx);
  k.inv_dx = T(s.inv_dx);
  k.dt = T(s.dt);
  k.gravity = T(s.gravity);
  k.volume = T(s.volume);
  k.hardening = T(s.hardening);
  k.mass = T(s.mass);
  k.mu0 = T(s.mu_0);
  k.lam0 = T(s.lambda_0);
  k.v_allowed = T(s.dx * 0.9 / s.dt);
  k.res = s.res;
  k.model = s.model;
  k.wall_mode = s.wall_mode;
  k.variant = 0;
  return k;
}

constexpr int kBatchMaxThreads = 512;

template <typename T>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batch2d_substep(unsigned char* ws, PView<T> P, int nscenes) {
  BatchHeader* h = reinterpret_cast<BatchHeader*>(ws);
  __shared__ ffmpm_scene2d s_sc[kMaxScenes];
  __shared__ int64_t s_poff[kMaxScenes + 1];
  __shared__ int64_t s_noff[kMaxScenes + 1];
  __shared__ int s_fail;
  const ffmpm_scene2d* g_sc = reinterpret_cast<const ffmpm_scene2d*>(ws + sizeof(BatchHeader));
  // table offsets follow the host layout (see batch_layout): scenes, particle offsets, node offsets
  const size_t up_sc = (sizeof(BatchHeader) + sizeof(ffmpm_scene2d) * nscenes + 255) / 256 * 256;
  const int64_t* g_poff = reinterpret_cast<const int64_t*>(ws + up_sc);
  const size_t up_po = (up_sc + sizeof(int64_t) * (nscenes + 1) + 255) / 256 * 256;
  const int64_t* g_noff = reinterpret_cast<const int64_t*>(ws + up_po);
  const size_t up_no = (up_po + sizeof(int64_t) * (nscenes + 1) + 255) / 256 * 256;
  const int64_t ntot = g_poff[nscenes], nnodes = g_noff[nscenes];
  Node4<T>* A = reinterpret_cast<Node4<T>*>(ws + up_no);
  Node4<T>* B = A + nnodes + ((256 - (nnodes * sizeof(Node4<T>)) % 256) % 256) / sizeof(Node4<T>);
  for (int i = threadIdx.x; i < nscenes; i += blockDim.x) s_sc[i] = g_sc[i];
  for (int i = threadIdx.x; i <= nscenes; i += blockDim.x) {
    s_poff[i] = g_poff[i];
    s_noff[i] = g_noff[i];
  }
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  const uint32_t limit = h->wait_limit ? h->wait_limit : kBarrierSpins;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // ---- phase 1: P2G
  for (int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gp < ntot; gp += stride) {
    const int si = find_scene(s_poff, nscenes, gp);
    const ffmpm_scene2d& sc = s_sc[si];
    const KParams<T> kp = scene_kparams<T>(sc);
    const uint32_t p = (uint32_t)gp;
    T fx[2], w[3][2];
    int b[2];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      ok = ok && base_of(P.x[P.at(p, d, 2)], kp.inv_dx, kp.res, b[d], fx[d]);
      T ww[3];
      bspline(fx[d], ww);
      w[0][d] = ww[0];
      w[1][d] = ww[1];
      w[2][d] = ww[2];
    }
    if (!ok) {
      raise_status(&h->status, FFMPM_STATUS_OOB);
      continue;
    }
    T F[4], C[4], A2[4], v[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      F[i] = P.F[P.at(p, i, 4)];
      C[i] = P.C[P.at(p, i, 4)];
    }
    v[0] = P.v[P.at(p, 0, 2)];
    v[1] = P.v[P.at(p, 1, 2)];
    const T e = kp.model == FFMPM_MODEL_SNOW ? ffexp(kp.hardening * (T(1) - P.Jp[p])) : kp.hardening;
    affine_of<2, T>(kp, F, C, kp.mass, kp.mu0 * e, kp.lam0 * e, A2, nullptr);
    const int R = kp.res + 1;
    Node4<T>* grid = A + s_noff[si];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T d0 = (T(i) - fx[0]) * kp.dx;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T d1 = (T(j) - fx[1]) * kp.dx;
        const T wt = w[i][0] * w[j][1];
        InternalSink<T>{grid}.add((int64_t)(b[0] + i) * R + (b[1] + j),
                                   wt * (v[0] * kp.mass + (A2[0] * d0 + A2[1] * d1)),
                                   wt * (v[1] * kp.mass + (A2[2] * d0 + A2[3] * d1)), T(0), wt * kp.mass);
      }
    }
  }
  // (fault injection for tests: CTA 0 never arrives, so the first barrier can only end by running out)
  if ((h->inject & FFMPM_INJECT_BARRIER_ABSENT) && blockIdx.x == 0) return;
  if (!grid_barrier(h, &s_fail, limit)) return;
  // ---- phase 2: grid update, every node of every scene
  for (int64_t gn = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gn < nnodes; gn += stride) {
    const int si = find_scene(s_noff, nscenes, gn);
    const ffmpm_scene2d& sc = s_sc[si];
    const KParams<T> kp = scene_kparams<T>(sc);
    const int li = (int)(gn - s_noff[si]);  // node of the scene: at most 257^2, 32-bit division
    const int R = kp.res + 1;
    int I[2] = {li / R, li % R};
    const Node4<T> a = A[gn];
    T vel[3] = {a.x, a.y, a.z};
    grid_node<2, T>(kp, I, vel, a.w);
    B[gn] = Node4<T>{vel[0], vel[1], T(0), a.w};
    A[gn] = Node4<T>{T(0), T(0), T(0), T(0)};
  }
  if (!grid_barrier(h, &s_fail, limit)) return;
  // ---- phase 3: G2P
  for (int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gp < ntot; gp += stride) {
    const int si = find_scene(s_poff, nscenes, gp);
    const ffmpm_scene2d& sc = s_sc[si];
    const KParams<T> kp = scene_kparams<T>(sc);
    const uint32_t p = (uint32_t)gp;
    T xp[2], fx[2], w[3][2];
    int b[2];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      xp[d] = P.x[P.at(p, d, 2)];
      ok = ok && base_of(xp[d], kp.inv_dx, kp.res, b[d], fx[d]);
      T ww[3];
      bspline(fx[d], ww);
      w[0][d] = ww[0];
      w[1][d] = ww[1];
      w[2][d] = ww[2];
    }
    if (!ok) continue;
    const int R = kp.res + 1;
    const Node4<T>* grid = B + s_noff[si];
    // node velocities relative to the stencil's centre node (the bulk velocity cancels exactly in C)
    T v[2] = {T(0), T(0)}, Cn[4] = {T(0), T(0), T(0), T(0)};
    const Node4<T> uc = grid[(int64_t)(b[0] + 1) * R + (b[1] + 1)];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T d0 = T(i) - fx[0];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T d1 = T(j) - fx[1];
        const T wt = w[i][0] * w[j][1];
        const Node4<T> gv = grid[(int64_t)(b[0] + i) * R + (b[1] + j)];
        const T wv0 = wt * (gv.x - uc.x), wv1 = wt * (gv.y - uc.y);
        v[0] += wv0;
        v[1] += wv1;
        Cn[0] += wv0 * d0;
        Cn[1] += wv0 * d1;
        Cn[2] += wv1 * d0;
        Cn[3] += wv1 * d1;
      }
    }
    v[0] += uc.x;
    v[1] += uc.y;
    const T c4 = T(4) * kp.inv_dx;
#pragma unroll
    for (int i = 0; i < 4; ++i) Cn[i] *= c4;
    T F[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) F[i] = P.F[P.at(p, i, 4)];
    T Fn[4];
    // F + dt (C F): (I + dt C) F with the increment rounded once against F
    Fn[0] = F[0] + kp.dt * (Cn[0] * F[0] + Cn[1] * F[2]);
    Fn[1] = F[1] + kp.dt * (Cn[0] * F[1] + Cn[1] * F[3]);
    Fn[2] = F[2] + kp.dt * (Cn[2] * F[0] + Cn[3] * F[2]);
    Fn[3] = F[3] + kp.dt * (Cn[2] * F[1] + Cn[3] * F[3]);
    const T oldJ = Fn[0] * Fn[3] - Fn[1] * Fn[2];
    if (kp.model == FFMPM_MODEL_SNOW) {
      T U[4], s2[2], V[4];
      svd2<T>(Fn, U, s2, V);
      s2[0] = ffclamp(s2[0], T(1.0 - 2.5e-2), T(1.0 + 7.5e-3));
      s2[1] = ffclamp(s2[1], T(1.0 - 2.5e-2), T(1.0 + 7.5e-3));
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) Fn[i * 2 + j] = U[i * 2] * s2[0] * V[j * 2] + U[i * 2 + 1] * s2[1] * V[j * 2 + 1];
    }
    const T det = (Fn[0] * Fn[3] - Fn[1] * Fn[2]) + T(1e-10);
    P.Jp[p] = ffclamp(P.Jp[p] * oldJ / det, T(0.6), T(20.0));
    const T xn[2] = {xp[0] + kp.dt * v[0], xp[1] + kp.dt * v[1]};
    if (nonfinite_probe(xn, 2) + nonfinite_probe(Fn, 4) != T(0)) raise_status(&h->status, FFMPM_STATUS_NONFINITE);
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      P.x[P.at(p, d, 2)] = xn[d];
      P.v[P.at(p, d, 2)] = v[d];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      P.C[P.at(p, i, 4)] = Cn[i];
      P.F[P.at(p, i, 4)] = Fn[i];
    }
  }
}

int batch_threads(int requested) { return requested == 128 || requested == 512 ? requested : kThreads; }

}  // namespace
}  // namespace ffmpm

using namespace ffmpm;

extern "C" {

int ffmpm_batch2d_workspace_size(const ffmpm_scene2d* scenes, int32_t nscenes, int32_t real_bytes, size_t* bytes) {
  BatchLayout L;
  if (!bytes || !batch_layout(scenes, nscenes, real_bytes, &L)) return FFMPM_ERR_BADARG;
  *bytes = L.total;
  return FFMPM_OK;
}

int ffmpm_batch2d_init(const ffmpm_scene2d* scenes, int32_t nscenes, int32_t real_bytes, void* ws, size_t ws_bytes,
                       void* stream) {
  BatchLayout L;
  if (!batch_layout(scenes, nscenes, real_bytes, &L)) return FFMPM_ERR_BADARG;
  if (!ws || ws_bytes < L.total || (reinterpret_cast<uintptr_t>(ws) & 255)) return FFMPM_ERR_WORKSPACE;
  // host image of the table part of the workspace, copied once (synchronously: the caller's
  // scene array may go away after the call)
  std::vector<unsigned char> img(L.off_gridA, 0);
  BatchHeader* h = reinterpret_cast<BatchHeader*>(img.data());
  h->nscenes = nscenes;
  int64_t* poff = reinterpret_cast<int64_t*>(img.data() + L.off_poffs);
  int64_t* noff = reinterpret_cast<int64_t*>(img.data() + L.off_noffs);
  std::memcpy(img.data() + L.off_scenes, scenes, sizeof(ffmpm_scene2d) * nscenes);
  int64_t p = 0, nn = 0;
  for (int i = 0; i < nscenes; ++i) {
    if (scenes[i].offset != p) return FFMPM_ERR_BADARG;  // scenes are consecutive particle ranges
    poff[i] = p;
    noff[i] = nn;
    p += scenes[i].count;
    nn += int64_t(scenes[i].res + 1) * (scenes[i].res + 1);
  }
  poff[nscenes] = p;
  noff[nscenes] = nn;
  h->total_particles = p;
  h->total_nodes = nn;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(ws, img.data(), img.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) return FFMPM_ERR_CUDA;
  if (cudaMemsetAsync(static_cast<unsigned char*>(ws) + L.off_gridA, 0, L.total - L.off_gridA, s) != cudaSuccess)
    return FFMPM_ERR_CUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

int ffmpm_batch2d_substeps(int32_t nscenes, int32_t real_bytes, ffmpm_particles* P, int32_t nsteps, int32_t threads,
                           int32_t ctas_per_sm, void* ws, size_t ws_bytes, void* stream) {
  if (!P || !ws || nsteps < 0 || nscenes < 1 || nscenes > kMaxScenes) return FFMPM_ERR_BADARG;
  if (real_bytes != 4 && real_bytes != 8) return FFMPM_ERR_BADARG;
  if (!P->x || !P->v || !P->F || !P->C || !P->Jp) return FFMPM_ERR_BADARG;
  if (P->stride != 0 && P->stride < P->n) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nt = batch_threads(threads);
  auto launch = [&](auto kern, auto view) -> int {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, 0) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      return FFMPM_ERR_CUDA;
    }
    if (ctas_per_sm > 0) per_sm = std::min(per_sm, (int)ctas_per_sm);
    const int grid = per_sm * sm_count();  // every CTA resident: the cooperative launch checks it
    unsigned char* wsp = static_cast<unsigned char*>(ws);
    // a launch whose barrier ran out leaves its arrivals counted: start every call from zero
    if (cudaMemsetAsync(wsp + offsetof(BatchHeader, barrier_count), 0, sizeof(uint32_t), s) != cudaSuccess)
      return FFMPM_ERR_CUDA;
    int ns = nscenes;
    void* args[] = {&wsp, &view, &ns};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(nt);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    for (int k = 0; k < nsteps; ++k)
      if (cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(kern), args) != cudaSuccess) {
        cudaGetLastError();  // a rejected launch configuration must not linger as the last error
        return FFMPM_ERR_CUDA;
      }
    return FFMPM_OK;
  };
  if (real_bytes == 4) {
    PView<float> v{};
    v.x = static_cast<float*>(P->x);
    v.v = static_cast<float*>(P->v);
    v.F = static_cast<float*>(P->F);
    v.C = static_cast<float*>(P->C);
    v.Jp = static_cast<float*>(P->Jp);
    v.soa = P->stride;
    return launch(k_batch2d_substep<float>, v);
  }
  PView<double> v{};
  v.x = static_cast<double*>(P->x);
  v.v = static_cast<double*>(P->v);
  v.F = static_cast<double*>(P->F);
  v.C = static_cast<double*>(P->C);
  v.Jp = static_cast<double*>(P->Jp);
  v.soa = P->stride;
  return launch(k_batch2d_substep<double>, v);
}

int ffmpm_batch2d_set_waits(void* ws, uint32_t wait_limit, uint32_t inject, void* stream) {
  if (!ws) return FFMPM_ERR_BADARG;
  const uint32_t v[2] = {wait_limit, inject};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(static_cast<unsigned char*>(ws) + offsetof(BatchHeader, wait_limit), v, sizeof(v),
                      cudaMemcpyHostToDevice, s) != cudaSuccess)
    return FFMPM_ERR_CUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

int ffmpm_batch2d_status(void* ws, int32_t* status, void* stream) {
  if (!ws || !status) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BatchHeader h;
  if (cudaMemcpyAsync(&h, ws, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FFMPM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return FFMPM_ERR_CUDA;
  *status = h.status;
  return FFMPM_OK;
}

}  // extern "C"
