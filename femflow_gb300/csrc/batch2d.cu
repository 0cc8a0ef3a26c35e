// Batched 2D MLS-MPM: many independent scenes (each with its own particles, grid resolution,
// material, dt and walls) advanced by ONE persistent cooperative launch per call.
//
// Phases, separated by a grid-wide barrier (bounded spin; co-residency of all CTAs is guaranteed by
// the cooperative launch):
//   P2G over every particle of every scene: stress (utils.py:52-92) + 9-node scatter into the
//     scene's grid A (two_d/p2g.py:11-76); the lanes of a warp that share a base cell sum their
//     contributions before the atomics, and every scene's box of touched nodes is widened
//   then per substep:
//   grid update over the nodes of every scene's box: two_d/grid_op.py:5-24 into B, A re-zeroed
//   G2P over every particle (gather v and C from B, advect, F update, Jp: two_d/g2p.py:5-47),
//     followed in the same pass by the next substep's P2G of the particle's new state
// Scenes are located from a global particle (or node) index by binary search in an offset table
// held in shared memory.  Nodes outside a scene's box carry no mass: the reference's grid update
// leaves them at zero and no particle reads them.
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

// A scene's kernel parameters in the compute type, converted once by ffmpm_batch2d_init (the
// float64 table entries would otherwise be converted, and v_allowed divided in float64, in every
// CTA of every launch).
template <typename T>
struct SceneK {
  T dx, inv_dx, dt, gravity, volume, hardening, mass, mu0, lam0, v_allowed;
  int res, model, wall_mode, wall_lo, wall_hi;
};

template <typename T>
__host__ __device__ inline SceneK<T> scene_k(const ffmpm_scene2d& s) {
  SceneK<T> k;
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
  wall_band_2d(s.res, &k.wall_lo, &k.wall_hi);
  return k;
}

constexpr int kEmptyLo = 0x7fffffff, kEmptyHi = -0x7fffffff - 1;

__host__ __device__ inline size_t up256(size_t v) { return (v + 255) / 256 * 256; }

// Byte offsets of the table part of the workspace (host and device agree on them): the header, the
// scene table, particle offsets, node offsets, then two slots of per-scene node boxes
// {lo0, lo1, hi0, hi1} (int32; empty: lo = kEmptyLo, hi = kEmptyHi), the scenes' SceneK in the
// compute type, then grid A.
struct TableOffsets {
  size_t scenes, poffs, noffs, boxes, sk, grid;
};
__host__ __device__ inline TableOffsets table_offsets(int nscenes) {
  TableOffsets t;
  size_t off = sizeof(BatchHeader);
  t.scenes = off;
  off = up256(off + sizeof(ffmpm_scene2d) * nscenes);
  t.poffs = off;
  off = up256(off + sizeof(int64_t) * (nscenes + 1));
  t.noffs = off;
  off = up256(off + sizeof(int64_t) * (nscenes + 1));
  t.boxes = off;
  off = up256(off + sizeof(int32_t) * 4 * 2 * nscenes);
  t.sk = off;
  off = up256(off + sizeof(SceneK<double>) * nscenes);
  t.grid = off;
  return t;
}

struct BatchLayout {
  size_t off_scenes, off_poffs, off_noffs, off_boxes, off_gridA, off_gridB, total;
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
  const TableOffsets t = table_offsets(nscenes);
  L->off_scenes = t.scenes;
  L->off_poffs = t.poffs;
  L->off_noffs = t.noffs;
  L->off_boxes = t.boxes;
  L->off_gridA = t.grid;
  size_t off = up256(t.grid + size_t(4) * real_bytes * nodes);
  L->off_gridB = off;
  off = up256(off + size_t(4) * real_bytes * nodes);
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
__device__ __forceinline__ KParams<T> scene_kparams(const SceneK<T>& s) {
  KParams<T> k;
  k.dx = s.dx;
  k.inv_dx = s.inv_dx;
  k.dt = s.dt;
  k.gravity = s.gravity;
  k.volume = s.volume;
  k.hardening = s.hardening;
  k.mass = s.mass;
  k.mu0 = s.mu0;
  k.lam0 = s.lam0;
  k.v_allowed = s.v_allowed;
  k.res = s.res;
  k.model = s.model;
  k.wall_mode = s.wall_mode;
  k.wall_lo = s.wall_lo;
  k.wall_hi = s.wall_hi;
  k.variant = 0;
  return k;
}

constexpr int kBatchMaxThreads = 512;

// Widen a scene's node box; the plain L2 read first skips the atomics that would change nothing
// (boxes only grow within a pass, so a stale read can only cost an atomic, never lose one).
__device__ __forceinline__ void widen_box(int* bx, int lo0, int lo1, int hi0, int hi1) {
  if (lo0 < __ldcg(bx + 0)) atomicMin(bx + 0, lo0);
  if (lo1 < __ldcg(bx + 1)) atomicMin(bx + 1, lo1);
  if (hi0 > __ldcg(bx + 2)) atomicMax(bx + 2, hi0);
  if (hi1 > __ldcg(bx + 3)) atomicMax(bx + 3, hi1);
}

// P2G of one particle per lane of a whole warp (every lane calls it).  Lanes that hold a run of
// consecutive particles with the same base node (the batch keeps each scene's particles ordered by
// base cell) sum their 27 node contributions with shuffles; the run's first lane then adds the 9
// sums to the grid, one vector atomic per node instead of one per (particle, node).  The scene's
// box of touched nodes is widened by one atomic per bound per warp where the warp holds one scene.
template <typename T>
__device__ __forceinline__ void scatter_warp(Node4<T>* A, int64_t noff, int* boxes, int si, bool ok, const int b[2],
                                             const T fx[2], const T v[2], const T A2[4], const KParams<T>& kp,
                                             int lane) {
  constexpr unsigned kFull = 0xffffffffu;
  T w[3][2];
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    T ww[3];
    bspline(ok ? fx[d] : T(0), ww);
    w[0][d] = ww[0];
    w[1][d] = ww[1];
    w[2][d] = ww[2];
  }
  const int R = kp.res + 1;
  // runs: a lane starts one when its base node differs from the previous lane's (or it holds no
  // particle); lanes of one run carry the same run number
  const int64_t key = ok ? noff + (int64_t)b[0] * R + b[1] : -1 - (int64_t)lane;
  const int64_t prev = __shfl_up_sync(kFull, key, 1);
  const bool head = lane == 0 || key != prev;
  const unsigned heads = __ballot_sync(kFull, head);
  const int run = __popc(heads & (kFull >> (31 - lane)));  // heads at or below this lane
  const bool shared = heads != kFull;                         // some run holds more than one particle
  bool same[5];
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int off = 1 << s;
    const int other = __shfl_down_sync(kFull, run, off);
    same[s] = lane + off < 32 && other == run;
  }
  Node4<T>* grid = A + noff;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const T d0 = (T(i) - fx[0]) * kp.dx;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const T d1 = (T(j) - fx[1]) * kp.dx;
      const T wt = w[i][0] * w[j][1];
      T qx = ok ? wt * (v[0] * kp.mass + (A2[0] * d0 + A2[1] * d1)) : T(0);
      T qy = ok ? wt * (v[1] * kp.mass + (A2[2] * d0 + A2[3] * d1)) : T(0);
      T qm = ok ? wt * kp.mass : T(0);
      if (shared) {
        // suffix sums within each run: after the five steps the run's first lane holds its total
#pragma unroll
        for (int s = 0; s < 5; ++s) {
          const int off = 1 << s;
          const T tx = __shfl_down_sync(kFull, qx, off);
          const T ty = __shfl_down_sync(kFull, qy, off);
          const T tm = __shfl_down_sync(kFull, qm, off);
          if (same[s]) {
            qx += tx;
            qy += ty;
            qm += tm;
          }
        }
      }
      if (ok && head) InternalSink<T>{grid}.add((int64_t)(b[0] + i) * R + (b[1] + j), qx, qy, T(0), qm);
    }
  }
  int lo0 = ok ? b[0] : kEmptyLo, lo1 = ok ? b[1] : kEmptyLo;
  int hi0 = ok ? b[0] + 2 : kEmptyHi, hi1 = ok ? b[1] + 2 : kEmptyHi;
  const int si0 = __shfl_sync(kFull, si, 0);
  if (__all_sync(kFull, !ok || si == si0)) {
    lo0 = __reduce_min_sync(kFull, lo0);
    lo1 = __reduce_min_sync(kFull, lo1);
    hi0 = __reduce_max_sync(kFull, hi0);
    hi1 = __reduce_max_sync(kFull, hi1);
    if (lane == 0 && lo0 != kEmptyLo) widen_box(boxes + 4 * si0, lo0, lo1, hi0, hi1);
  } else if (ok) {
    widen_box(boxes + 4 * si, lo0, lo1, hi0, hi1);
  }
}

// Every scene's box of one slot into shared memory (clipped to the grid), with the exclusive scan
// of the boxes' node counts in s_boff (warp 0; nscenes <= 256).  Ends with __syncthreads.
template <typename T>
__device__ __forceinline__ void load_boxes(const int* box, const SceneK<T>* s_sc, int nscenes, int64_t* s_boff,
                                           int* s_blo0, int* s_blo1, int* s_bw) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int64_t carry = 0;
    for (int c0 = 0; c0 < nscenes; c0 += 32) {
      const int i = c0 + lane;
      int64_t cnt = 0;
      if (i < nscenes) {
        const int res = s_sc[i].res;
        const int lo0 = max(__ldcg(box + 4 * i + 0), 0), lo1 = max(__ldcg(box + 4 * i + 1), 0);
        const int hi0 = min(__ldcg(box + 4 * i + 2), res), hi1 = min(__ldcg(box + 4 * i + 3), res);
        const bool any = lo0 <= hi0 && lo1 <= hi1;
        s_blo0[i] = lo0;
        s_blo1[i] = lo1;
        s_bw[i] = any ? hi1 - lo1 + 1 : 1;
        cnt = any ? (int64_t)(hi0 - lo0 + 1) * (hi1 - lo1 + 1) : 0;
      }
      int64_t inc = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
      }
      if (i < nscenes) s_boff[i] = carry + inc - cnt;
      carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) s_boff[nscenes] = carry;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batch2d_substeps(unsigned char* ws, PView<T> P, int nscenes,
                                                                        int nsteps) {
  BatchHeader* h = reinterpret_cast<BatchHeader*>(ws);
  __shared__ SceneK<T> s_sc[kMaxScenes];
  __shared__ int64_t s_poff[kMaxScenes + 1];
  __shared__ int64_t s_noff[kMaxScenes + 1];
  __shared__ int64_t s_boff[kMaxScenes + 1];
  __shared__ int s_blo0[kMaxScenes], s_blo1[kMaxScenes], s_bw[kMaxScenes];
  __shared__ int s_fail;
  if (nsteps <= 0) return;
  const TableOffsets to = table_offsets(nscenes);
  const SceneK<T>* g_sc = reinterpret_cast<const SceneK<T>*>(ws + to.sk);
  const int64_t* g_poff = reinterpret_cast<const int64_t*>(ws + to.poffs);
  const int64_t* g_noff = reinterpret_cast<const int64_t*>(ws + to.noffs);
  int* boxes = reinterpret_cast<int*>(ws + to.boxes);
  const int64_t ntot = g_poff[nscenes], nnodes = g_noff[nscenes];
  Node4<T>* A = reinterpret_cast<Node4<T>*>(ws + to.grid);
  Node4<T>* B = A + up256(nnodes * sizeof(Node4<T>)) / sizeof(Node4<T>);
  for (int i = threadIdx.x; i < nscenes; i += blockDim.x) s_sc[i] = g_sc[i];
  for (int i = threadIdx.x; i <= nscenes; i += blockDim.x) {
    s_poff[i] = g_poff[i];
    s_noff[i] = g_noff[i];
  }
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  const uint32_t limit = h->wait_limit ? h->wait_limit : kBarrierSpins;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  // whole warps step through the particles together (the P2G scatter works on whole warps)
  const int64_t warp0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  // ---- P2G of the particles as they are, boxes into slot 0
  for (int64_t gbase = warp0; gbase < ntot; gbase += stride) {
    const int64_t gp = gbase + lane;
    bool ok = gp < ntot;
    const int si = ok ? find_scene(s_poff, nscenes, gp) : 0;
    const KParams<T> kp = scene_kparams<T>(s_sc[si]);
    const uint32_t p = (uint32_t)(ok ? gp : 0);
    T fx[2] = {T(0), T(0)};
    int b[2] = {0, 0};
    if (ok) {
#pragma unroll
      for (int d = 0; d < 2; ++d) ok = ok && base_of(P.x[P.at(p, d, 2)], kp.inv_dx, kp.res, b[d], fx[d]);
      if (!ok) raise_status(&h->status, FFMPM_STATUS_OOB);
    }
    T A2[4] = {T(0), T(0), T(0), T(0)}, v[2] = {T(0), T(0)};
    if (ok) {
      T F[4], C[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        F[i] = P.F[P.at(p, i, 4)];
        C[i] = P.C[P.at(p, i, 4)];
      }
      v[0] = P.v[P.at(p, 0, 2)];
      v[1] = P.v[P.at(p, 1, 2)];
      const T e = kp.model == FFMPM_MODEL_SNOW ? ffexp(kp.hardening * (T(1) - P.Jp[p])) : kp.hardening;
      affine_of<2, T>(kp, F, C, kp.mass, kp.mu0 * e, kp.lam0 * e, A2, nullptr);
    }
    scatter_warp<T>(A, s_noff[si], boxes, si, ok, b, fx, v, A2, kp, lane);
  }
  // (fault injection for tests: CTA 0 never arrives, so the first barrier can only end by running out)
  if ((h->inject & FFMPM_INJECT_BARRIER_ABSENT) && blockIdx.x == 0) return;
  for (int k = 0; k < nsteps; ++k) {
    int* box = boxes + 4 * nscenes * (k & 1);         // nodes the P2G of substep k touched
    int* nbox = boxes + 4 * nscenes * ((k + 1) & 1);  // filled by the P2G of substep k + 1
    if (!grid_barrier(h, &s_fail, limit)) return;
    // ---- grid update over every scene's box
    load_boxes<T>(box, s_sc, nscenes, s_boff, s_blo0, s_blo1, s_bw);
    const int64_t nbox_nodes = s_boff[nscenes];
    for (int64_t gn = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gn < nbox_nodes; gn += stride) {
      const int si = find_scene(s_boff, nscenes, gn);
      const KParams<T> kp = scene_kparams<T>(s_sc[si]);
      const int li = (int)(gn - s_boff[si]);  // node within the box: at most 4097^2
      const int w = s_bw[si];
      int I[2] = {s_blo0[si] + li / w, s_blo1[si] + li % w};
      const int64_t node = s_noff[si] + (int64_t)I[0] * (kp.res + 1) + I[1];
      const Node4<T> a = A[node];
      T vel[3] = {a.x, a.y, a.z};
      grid_node<2, T>(kp, I, vel, a.w);
      B[node] = Node4<T>{vel[0], vel[1], T(0), a.w};
      A[node] = Node4<T>{T(0), T(0), T(0), T(0)};
    }
    if (!grid_barrier(h, &s_fail, limit)) return;
    // this substep's boxes were read by the grid update only: empty them for the substep after next
    if (blockIdx.x == 0)
      for (int i = threadIdx.x; i < 4 * nscenes; i += blockDim.x) box[i] = (i & 3) < 2 ? kEmptyLo : kEmptyHi;
    const bool next = k + 1 < nsteps;
    // ---- G2P, then (but after the last substep) the next substep's P2G of the new state
    for (int64_t gbase = warp0; gbase < ntot; gbase += stride) {
      const int64_t gp = gbase + lane;
      const bool live = gp < ntot;
      const int si = live ? find_scene(s_poff, nscenes, gp) : 0;
      const KParams<T> kp = scene_kparams<T>(s_sc[si]);
      const uint32_t p = (uint32_t)(live ? gp : 0);
      T xp[2] = {T(0), T(0)}, fx[2] = {T(0), T(0)};
      int b[2] = {0, 0};
      bool ok = live;
      if (live) {
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          xp[d] = P.x[P.at(p, d, 2)];
          ok = ok && base_of(xp[d], kp.inv_dx, kp.res, b[d], fx[d]);
        }
      }
      T v[2] = {T(0), T(0)}, Cn[4] = {T(0), T(0), T(0), T(0)}, Fn[4] = {T(1), T(0), T(0), T(1)};
      T xn[2] = {T(0), T(0)}, Jpn = T(1);
      if (ok) {
        T w[3][2];
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          T ww[3];
          bspline(fx[d], ww);
          w[0][d] = ww[0];
          w[1][d] = ww[1];
          w[2][d] = ww[2];
        }
        const int R = kp.res + 1;
        const Node4<T>* grid = B + s_noff[si];
        // node velocities relative to the stencil's centre node (the bulk velocity cancels exactly in C)
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
            for (int j = 0; j < 2; ++j)
              Fn[i * 2 + j] = U[i * 2] * s2[0] * V[j * 2] + U[i * 2 + 1] * s2[1] * V[j * 2 + 1];
        }
        const T det = (Fn[0] * Fn[3] - Fn[1] * Fn[2]) + T(1e-10);
        Jpn = ffclamp(P.Jp[p] * oldJ / det, T(0.6), T(20.0));
        P.Jp[p] = Jpn;
        xn[0] = xp[0] + kp.dt * v[0];
        xn[1] = xp[1] + kp.dt * v[1];
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
      if (next) {  // warp-uniform
        // a particle already outside its grid stays there (G2P left it): its P2G fails as before
        bool ok2 = ok;
        T fx2[2] = {T(0), T(0)};
        int b2[2] = {0, 0};
        if (ok) {
#pragma unroll
          for (int d = 0; d < 2; ++d) ok2 = ok2 && base_of(xn[d], kp.inv_dx, kp.res, b2[d], fx2[d]);
        }
        if (live && !ok2) raise_status(&h->status, FFMPM_STATUS_OOB);
        T A2[4] = {T(0), T(0), T(0), T(0)};
        if (ok2) {
          const T e = kp.model == FFMPM_MODEL_SNOW ? ffexp(kp.hardening * (T(1) - Jpn)) : kp.hardening;
          affine_of<2, T>(kp, Fn, Cn, kp.mass, kp.mu0 * e, kp.lam0 * e, A2, nullptr);
        }
        scatter_warp<T>(A, s_noff[si], nbox, si, ok2, b2, fx2, v, A2, kp, lane);
      }
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
  int32_t* box = reinterpret_cast<int32_t*>(img.data() + L.off_boxes);
  for (int i = 0; i < 8 * nscenes; ++i) box[i] = (i & 3) < 2 ? kEmptyLo : kEmptyHi;
  for (int i = 0; i < nscenes; ++i) {
    unsigned char* dst = img.data() + table_offsets(nscenes).sk;
    if (real_bytes == 4)
      reinterpret_cast<SceneK<float>*>(dst)[i] = scene_k<float>(scenes[i]);
    else
      reinterpret_cast<SceneK<double>*>(dst)[i] = scene_k<double>(scenes[i]);
  }
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
  if (nsteps == 0) return FFMPM_OK;
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
    int ns = nscenes, nst = nsteps;
    void* args[] = {&wsp, &view, &ns, &nst};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(nt);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
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
    return launch(k_batch2d_substeps<float>, v);
  }
  PView<double> v{};
  v.x = static_cast<double*>(P->x);
  v.v = static_cast<double*>(P->v);
  v.F = static_cast<double*>(P->F);
  v.C = static_cast<double*>(P->C);
  v.Jp = static_cast<double*>(P->Jp);
  v.soa = P->stride;
  return launch(k_batch2d_substeps<double>, v);
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
