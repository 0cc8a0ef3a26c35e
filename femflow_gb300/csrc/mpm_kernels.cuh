// MLS-MPM substep kernels, templated on dimension (2, 3) and precision (float, double).
//
// Pipeline of one substep (all on one stream):
//   k_keys         block key of every particle (three_d/p2g.py:50 base rule) + block histogram
//   radix sort     stable, bit-exact permutation by key (sort.cu)
//   k_plan_*       block offsets, work chunks, touched-block list (three launches)
//   k_p2g_cells    stress + 3^d-node scatter by cell runs into a shared-memory tile per block, one
//                  vector atomic per touched node on flush   (three_d/p2g.py:14-80)
//   k_grid_update  momentum -> velocity, gravity, clamp, walls, planar colliders over touched
//                  blocks only                               (three_d/grid_op.py:5-67)
//   k_g2p          TMA-staged tile of grid velocities, gather v and APIC C, advect, update F
//                                                            (three_d/g2p.py:9-59)
//   k_g2p2g        G2P of one substep fused with P2G of the next (resident solver)
// Sorting and planning run on the substeps that re-sort; the others keep the plan.
#pragma once

#include <algorithm>
#include <cmath>
#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace ffmpm {

template <typename T>
struct KParams {
  T dx, inv_dx, dt, gravity, volume, hardening, mass, mu0, lam0, v_allowed;
  int res, model, wall_mode, variant;
  // 2D reference walls as node-index bounds (wall_band_2d): I / res < 0.05 <=> I < wall_lo and
  // I / res > 1 - 0.05 <=> I > wall_hi
  int wall_lo = 0, wall_hi = 0;
  // planar colliders: {point, normal'} in float64 with the plane rule already applied to the normal
  int n_planes = 0;
  double dx64 = 0.0;
  double planes[FFMPM_MAX_PLANES][6] = {};
};

// normal' of plane q of the params under the plane rule (three_d/grid_op.py:59-60)
inline void plane_normal(const ffmpm_params& p, int q, double out[3]) {
  const double* nr = p.planes[q] + 3;
  const int dim = p.dim;
  double ss = 0.0;
  for (int d = 0; d < dim; ++d) ss += nr[d] * nr[d];
  const double add = p.plane_rule == FFMPM_PLANES_REFERENCE_LITERAL ? 1.0 / std::sqrt(ss) : 0.0;
  for (int d = 0; d < 3; ++d) out[d] = d < dim ? nr[d] + add : 0.0;
}

// True when node I lies strictly on the negative side of plane q: (I dx - point) . normal' < 0,
// products and sums rounded one at a time in float64 as numpy computes them.
template <int DIM, typename T>
__device__ __forceinline__ bool behind_plane(const KParams<T>& kp, const int I[DIM], int q) {
  double dot = 0.0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const double off = __dsub_rn(__dmul_rn(double(I[d]), kp.dx64), kp.planes[q][d]);
    dot = __dadd_rn(dot, __dmul_rn(off, kp.planes[q][3 + d]));
  }
  return dot < 0.0;
}

// Variant flags (ffmpm_params.variant).
constexpr int kVariantP2GDirect = 1;  // P2G scatters straight to L2 with vector reds (no smem tile)
constexpr int kVariantP2GLanes = 2;   // P2G lane-per-particle shared-tile atomics (no cell runs)
constexpr int kVariantNoFuse = 4;     // sorted solver: separate G2P and P2G launches every substep
constexpr int kVariantSortShift = 8;  // bits 8..15: substeps between re-sorts of the sorted solver

template <typename T>
struct PView {
  T *x, *v, *F, *C, *Jp;
  T *mass, *mu0, *lam0;  // nullable: scalar material from KParams
  int64_t soa;           // 0: row-major [n][k] (the reference's layout); > 0: component-major stride
  // index of component c (of k) of particle p
  __device__ __forceinline__ size_t at(uint32_t p, int c, int k) const {
    return soa ? (size_t)c * (size_t)soa + p : (size_t)p * k + c;
  }
};

// The 2D reference walls (two_d/grid_op.py:13-19) compare the node coordinate I / res, computed in
// float64, with 0.05 and 1 - 0.05.  Correctly rounded I / res grows with I, so each comparison
// holds on a prefix or a suffix of 0..res: the first index with I / res >= 0.05 and the last with
// I / res <= 1 - 0.05, found here with the same float64 arithmetic, replace the two divisions per
// node.
__host__ __device__ inline void wall_band_2d(int res, int* lo, int* hi) {
  *lo = res + 1;
  for (int i = 0; i <= res; ++i)
    if (!(double(i) / double(res) < 0.05)) {
      *lo = i;
      break;
    }
  *hi = -1;
  for (int i = res; i >= 0; --i)
    if (!(double(i) / double(res) > 1.0 - 0.05)) {
      *hi = i;
      break;
    }
}

// Kernel parameters and particle view of the C-ABI structs (host side).
template <typename T>
inline KParams<T> kparams(const ffmpm_params& p) {
  KParams<T> k;
  k.dx = T(p.dx);
  k.inv_dx = T(p.inv_dx);
  k.dt = T(p.dt);
  k.gravity = T(p.gravity);
  k.volume = T(p.volume);
  k.hardening = T(p.hardening);
  k.mass = T(p.mass);
  k.mu0 = T(p.mu_0);
  k.lam0 = T(p.lambda_0);
  k.v_allowed = T(p.dx * 0.9 / p.dt);  // three_d/grid_op.py:25, computed in double as the reference
  k.res = p.res;
  k.model = p.model;
  k.wall_mode = p.wall_mode;
  k.variant = p.variant;
  wall_band_2d(p.res, &k.wall_lo, &k.wall_hi);
  k.n_planes = std::max(0, std::min(int(p.n_planes), FFMPM_MAX_PLANES));
  k.dx64 = p.dx;
  for (int q = 0; q < k.n_planes; ++q) {
    double nrm[3];
    plane_normal(p, q, nrm);
    for (int d = 0; d < 3; ++d) {
      k.planes[q][d] = d < p.dim ? p.planes[q][d] : 0.0;
      k.planes[q][3 + d] = nrm[d];
    }
  }
  return k;
}

template <typename T>
inline PView<T> pview(const ffmpm_particles& P) {
  PView<T> v;
  v.x = static_cast<T*>(P.x);
  v.v = static_cast<T*>(P.v);
  v.F = static_cast<T*>(P.F);
  v.C = static_cast<T*>(P.C);
  v.Jp = static_cast<T*>(P.Jp);
  v.mass = static_cast<T*>(const_cast<void*>(P.mass));
  v.mu0 = static_cast<T*>(const_cast<void*>(P.mu_0));
  v.lam0 = static_cast<T*>(const_cast<void*>(P.lambda_0));
  v.soa = P.stride;
  return v;
}


template <int DIM>
__device__ __forceinline__ void block_coords(const Geom<DIM>& g, int blk, int c[DIM]) {
  if constexpr (DIM == 3) {
    c[2] = blk % g.nb;
    c[1] = (blk / g.nb) % g.nb;
    c[0] = blk / (g.nb * g.nb);
  } else {
    c[1] = blk % g.nb;
    c[0] = blk / g.nb;
  }
}

template <int DIM>
__device__ __forceinline__ int64_t node_index(int R, const int I[DIM]) {
  if constexpr (DIM == 3)
    return ((int64_t)I[0] * R + I[1]) * (int64_t)R + I[2];
  else
    return (int64_t)I[0] * R + I[1];
}

// Key of a particle: block id (and, with cell_bits > 0, the cell inside the block in the low bits).
template <int DIM, typename T>
__device__ __forceinline__ bool particle_key(const T* xp, const KParams<T>& kp, const Geom<DIM>& g, int cell_bits,
                                             uint32_t& key, uint32_t& blk) {
  int b[DIM];
  bool ok = true;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    T fx;
    ok = ok && base_of(xp[d], kp.inv_dx, kp.res, b[d], fx);
  }
  if (!ok) {
    key = kInvalidKey;
    blk = 0;
    return false;
  }
  uint32_t bid = 0, cell = 0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    bid = bid * g.nb + (uint32_t)(b[d] >> g.bs_shift);
    cell = (cell << g.bs_shift) | (uint32_t)(b[d] & (g.bs - 1));
  }
  blk = bid;
  key = cell_bits ? ((bid << cell_bits) | cell) : bid;
  return true;
}

template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_keys(KParams<T> kp, Geom<DIM> g, PView<T> P, uint32_t n,
                                                   int cell_bits, uint32_t* __restrict__ keys,
                                                   uint32_t* __restrict__ block_count, int32_t* status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = false;
  uint32_t key = kInvalidKey, blk = 0;
  if (i < n) {
    T xp[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) xp[d] = P.x[P.at(i, d, DIM)];
    valid = particle_key<DIM, T>(xp, kp, g, cell_bits, key, blk);
    if (!valid) raise_status(status, FFMPM_STATUS_OOB);
    keys[i] = key;
  }
  if (block_count) warp_count(block_count, blk, valid);
}

// ----------------------------------------------------------------------------------------------
// The plan: block starts (exclusive scan of the histogram), chunks of at most kChunk particles, the
// list of occupied blocks, and the touched blocks (occupied blocks dilated by +1 along every axis,
// because a stencil based in block b reaches 2 nodes into block b+1; by +-1 when the plan is kept
// over several substeps).  Three launches over CTAs of 1024 blocks (k_plan_local: values and local
// prefixes; k_plan_offsets: prefixes of the CTA totals; k_plan_write: final offsets and lists), so
// that no CTA waits on another.  The last one re-zeroes the histogram for the next substep.
struct Scan4 {
  uint32_t a, b, c, d;
};

// Exclusive scan of KB Scan4 values per thread over the CTA, part j of every thread before part
// j + 1 (the thread's parts cover blocks j * blockDim + threadIdx): ex[j] is the prefix of part j
// of this thread, *total the sum of everything.  One set of barriers for all KB parts.
template <int KB>
__device__ __forceinline__ void block_exclusive_scan4_parts(const Scan4 (&v)[KB], Scan4 (&ex)[KB], Scan4* total,
                                                            Scan4 (*warp_buf)[32]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  Scan4 inc[KB];
#pragma unroll
  for (int j = 0; j < KB; ++j) {
    inc[j] = v[j];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ta = __shfl_up_sync(0xffffffffu, inc[j].a, o), tb = __shfl_up_sync(0xffffffffu, inc[j].b, o);
      const uint32_t tc = __shfl_up_sync(0xffffffffu, inc[j].c, o), td = __shfl_up_sync(0xffffffffu, inc[j].d, o);
      if (lane >= o) {
        inc[j].a += ta; inc[j].b += tb; inc[j].c += tc; inc[j].d += td;
      }
    }
    if (lane == 31) warp_buf[j][warp] = inc[j];
  }
  __syncthreads();
  if (warp == 0) {
    // scan the KB x nwarps warp totals in part-major order
    Scan4 carry{0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < KB; ++j) {
      Scan4 w = lane < nwarps ? warp_buf[j][lane] : Scan4{0, 0, 0, 0};
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ta = __shfl_up_sync(0xffffffffu, w.a, o), tb = __shfl_up_sync(0xffffffffu, w.b, o);
        const uint32_t tc = __shfl_up_sync(0xffffffffu, w.c, o), td = __shfl_up_sync(0xffffffffu, w.d, o);
        if (lane >= o) {
          w.a += ta; w.b += tb; w.c += tc; w.d += td;
        }
      }
      w.a += carry.a; w.b += carry.b; w.c += carry.c; w.d += carry.d;
      if (lane < nwarps) warp_buf[j][lane] = w;  // inclusive over parts < j and warps <= lane
      carry.a = __shfl_sync(0xffffffffu, w.a, nwarps - 1);
      carry.b = __shfl_sync(0xffffffffu, w.b, nwarps - 1);
      carry.c = __shfl_sync(0xffffffffu, w.c, nwarps - 1);
      carry.d = __shfl_sync(0xffffffffu, w.d, nwarps - 1);
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < KB; ++j) {
    Scan4 prev;
    if (warp > 0) prev = warp_buf[j][warp - 1];
    else if (j > 0) prev = warp_buf[j - 1][nwarps - 1];
    else prev = Scan4{0, 0, 0, 0};
    ex[j] = Scan4{prev.a + inc[j].a - v[j].a, prev.b + inc[j].b - v[j].b, prev.c + inc[j].c - v[j].c,
                  prev.d + inc[j].d - v[j].d};
  }
  *total = warp_buf[KB - 1][nwarps - 1];
  __syncthreads();
}

// Touched test of block b, gather form: any block b - o, o in {0,1}^DIM, holds particles; with `sym`
// any block b + o, o in {-1,0,1}^DIM (the histogram is small and stays in L2).
template <int DIM>
__device__ __forceinline__ uint32_t plan_touched(const Geom<DIM>& g, const uint32_t* __restrict__ block_count, int b,
                                                 int sym) {
  int bc[DIM];
  block_coords<DIM>(g, b, bc);
  if (!sym) {
#pragma unroll
    for (int o = 0; o < (1 << DIM); ++o) {
      int nb_id = 0;
      bool ok = true;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int cc = bc[d] - ((o >> (DIM - 1 - d)) & 1);
        ok = ok && cc >= 0;
        nb_id = nb_id * g.nb + cc;
      }
      if (ok && block_count[nb_id] > 0) return 1u;
    }
    return 0u;
  }
  constexpr int NO = DIM == 3 ? 27 : 9;
#pragma unroll
  for (int o = 0; o < NO; ++o) {
    int nb_id = 0, r = o;
    bool ok = true;
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
      const int cc = bc[d] + (r % 3) - 1;
      r /= 3;
      ok = ok && cc >= 0 && cc < g.nb;
    }
    if (!ok) continue;
    r = o;
    int mul = 1;
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
      nb_id += (bc[d] + (r % 3) - 1) * mul;
      mul *= g.nb;
      r /= 3;
    }
    if (block_count[nb_id] > 0) return 1u;
  }
  return 0u;
}

constexpr int kPlanCta = 1024;  // blocks per CTA of the plan kernels

// Per block: count, touched mark, and the prefixes of (particles, chunks, touched, occupied) within
// its CTA's 1024 blocks (particles in block_start, the others in pref[0..2][nblocks]); per CTA: the
// totals.  Nothing is done on a substep that keeps its plan (sort_flag 0).
template <int DIM>
__global__ void __launch_bounds__(kPlanCta) k_plan_local(Geom<DIM> g, const uint32_t* __restrict__ block_count,
                                                         uint32_t* __restrict__ block_start,
                                                         uint32_t* __restrict__ block_cnt, uint32_t* __restrict__ tmark,
                                                         uint32_t* __restrict__ pref, Scan4* __restrict__ cta_tot,
                                                         const uint32_t* __restrict__ sort_flag, int sym) {
  if (sort_flag && *sort_flag == 0u) return;
  __shared__ Scan4 part_buf[1][32];
  const int b = blockIdx.x * kPlanCta + threadIdx.x;
  uint32_t c = 0, tch = 0;
  if (b < g.nblocks) {
    c = block_count[b];
    tch = plan_touched<DIM>(g, block_count, b, sym);
  }
  const Scan4 v[1] = {Scan4{c, (c + kChunk - 1) / kChunk, tch, c > 0 ? 1u : 0u}};
  Scan4 ex[1], tot;
  block_exclusive_scan4_parts<1>(v, ex, &tot, part_buf);
  if (b < g.nblocks) {
    block_start[b] = ex[0].a;
    pref[b] = ex[0].b;
    pref[g.nblocks + b] = ex[0].c;
    pref[2 * g.nblocks + b] = ex[0].d;
    block_cnt[b] = c;
    tmark[b] = tch;
  }
  if (threadIdx.x == 0) cta_tot[blockIdx.x] = tot;
}

// One CTA: exclusive prefixes of the CTA totals, and the plan's totals into the header.
static __global__ void __launch_bounds__(kPlanCta) k_plan_offsets(const Scan4* __restrict__ cta_tot, Scan4* __restrict__ cta_off,
                                                           int ncta, WsHeader* hdr, const uint32_t* __restrict__ sort_flag) {
  if (sort_flag && *sort_flag == 0u) return;
  __shared__ Scan4 part_buf[1][32];
  Scan4 carry{0, 0, 0, 0};
  for (int base = 0; base < ncta; base += kPlanCta) {
    const int i = base + threadIdx.x;
    const Scan4 v[1] = {i < ncta ? cta_tot[i] : Scan4{0, 0, 0, 0}};
    Scan4 ex[1], tot;
    block_exclusive_scan4_parts<1>(v, ex, &tot, part_buf);
    if (i < ncta) cta_off[i] = Scan4{carry.a + ex[0].a, carry.b + ex[0].b, carry.c + ex[0].c, carry.d + ex[0].d};
    carry.a += tot.a; carry.b += tot.b; carry.c += tot.c; carry.d += tot.d;
  }
  if (threadIdx.x == 0) {
    hdr->n_valid = carry.a;
    hdr->n_chunks = carry.b;
    hdr->n_touched = carry.c;
    hdr->n_occupied = carry.d;
  }
}

// Final block starts, the chunks, the touched and occupied lists; re-zeroes the histogram (also on
// substeps that keep their plan, where nothing else is written).
template <int DIM>
__global__ void __launch_bounds__(kPlanCta) k_plan_write(Geom<DIM> g, uint32_t* __restrict__ block_count,
                                                         uint32_t* __restrict__ block_start,
                                                         const uint32_t* __restrict__ block_cnt,
                                                         const uint32_t* __restrict__ tmark,
                                                         const uint32_t* __restrict__ pref,
                                                         const Scan4* __restrict__ cta_off, int4* __restrict__ chunks,
                                                         uint32_t* __restrict__ touched, int4* __restrict__ occupied,
                                                         const uint32_t* __restrict__ sort_flag) {
  const int b = blockIdx.x * kPlanCta + threadIdx.x;
  if (b >= g.nblocks) return;
  if (!(sort_flag && *sort_flag == 0u)) {
    const Scan4 off = cta_off[blockIdx.x];
    const uint32_t c = block_cnt[b], start = off.a + block_start[b];
    block_start[b] = start;
    const uint32_t nch = (c + kChunk - 1) / kChunk, ch0 = off.b + pref[b];
    for (uint32_t q = 0; q < nch; ++q)
      chunks[ch0 + q] = make_int4(b, (int)(start + q * kChunk), (int)min((uint32_t)kChunk, c - q * kChunk), 0);
    if (tmark[b]) touched[off.c + pref[g.nblocks + b]] = (uint32_t)b;
    if (c > 0) occupied[off.d + pref[2 * g.nblocks + b]] = make_int4(b, (int)start, (int)c, 0);
  }
  block_count[b] = 0;
}

// ----------------------------------------------------------------------------------------------
// Grid-side scatter targets of P2G.
template <typename T>
struct InternalSink {  // workspace grid of Node4 {momentum xyz, mass}
  Node4<T>* A;
  __device__ __forceinline__ void add(int64_t node, T a, T b, T c, T m) const {
    if constexpr (sizeof(T) == 4) {
      atomicAdd(reinterpret_cast<float4*>(A + node), make_float4(a, b, c, m));
    } else {
      atomic_add4(A + node, a, b, c, m);
    }
  }
};

template <typename T, int DIM>
struct UserSink {  // caller's grid_velocity [nodes][DIM] and grid_mass [nodes]
  T* gv;
  T* gm;
  __device__ __forceinline__ void add(int64_t node, T a, T b, T c, T m) const {
    atomicAdd(&gv[node * DIM + 0], a);
    atomicAdd(&gv[node * DIM + 1], b);
    if constexpr (DIM == 3) atomicAdd(&gv[node * DIM + 2], c);
    atomicAdd(&gm[node], m);
  }
};

template <int DIM>
__device__ __forceinline__ int tile_nodes(const Geom<DIM>& g) {
  return DIM == 3 ? g.tile * g.tile * g.tile : g.tile * g.tile;
}

// Stress + APIC affine matrix of one particle (utils.py:95-135 / 52-92):
//   A = -(dt*vol) * (4*inv_dx^2 * PF) + m*C,  PF = 2mu(F-R)F^T + lam(J-1)J  (scalar on all entries;
//   on the diagonal only for FFMPM_MODEL_FIXED_COROTATED)
// F - R for F close to a rotation, without forming R: with S = sqrt(F^T F) = I + Y,
// F - R = F (I - S^-1) = F Y (I + Y)^-1, and Y = S - I is the fixed point of Y = (E - Y^2) / 2 with
// E = F^T F - I = H + H^T + H^T H, H = F - I.  Every quantity is of the size of the strain, so F - R
// keeps float's relative precision; Newton's R has an absolute error of ~1e-7, which at strain 1e-4
// leaves F - R with three correct digits.  Applies when max |E| <= 0.05 (then |Y|_F < 0.08, the
// iteration contracts by that factor, and six iterations reach float precision); returns false
// otherwise.
template <typename T>
__device__ __forceinline__ bool f_minus_r_small_strain3(const T F[9], T FmR[9]) {
  T H[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) H[i] = F[i] - (i % 4 == 0 ? T(1) : T(0));
  // E and Y are symmetric (every entry (a, b) is formed exactly like (b, a)), so only the six
  // entries a <= b are computed and mirrored: bit-identical to the full products
  T E[9], emax = T(0);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      const T e = H[a * 3 + b] + H[b * 3 + a] + H[0 * 3 + a] * H[0 * 3 + b] + H[1 * 3 + a] * H[1 * 3 + b] +
                  H[2 * 3 + a] * H[2 * 3 + b];
      E[a * 3 + b] = E[b * 3 + a] = e;
      emax = ffabs(e) > emax ? ffabs(e) : emax;
    }
  if (!(emax <= T(0.05))) return false;
  T Y[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) Y[i] = T(0.5) * E[i];
  // at most six iterations; an iteration that returns Y unchanged is a fixed point (every later one
  // would return the same Y), so stopping there gives the six-iteration result bit for bit
#pragma unroll 1
  for (int it = 0; it < 6; ++it) {
    T Yn[9];
    bool same = true;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a; b < 3; ++b) {
        const T y = T(0.5) * (E[a * 3 + b] - (Y[a * 3 + 0] * Y[0 * 3 + b] + Y[a * 3 + 1] * Y[1 * 3 + b] +
                                              Y[a * 3 + 2] * Y[2 * 3 + b]));
        Yn[a * 3 + b] = Yn[b * 3 + a] = y;
        same = same && y == Y[a * 3 + b];
      }
#pragma unroll
    for (int i = 0; i < 9; ++i) Y[i] = Yn[i];
    if (same) break;
  }
  T M[9], Mc[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) M[i] = Y[i] + (i % 4 == 0 ? T(1) : T(0));
  cofactor3(M, Mc);
  const T inv_det = T(1) / (M[0] * Mc[0] + M[1] * Mc[1] + M[2] * Mc[2]);
  T FY[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      FY[a * 3 + b] = F[a * 3 + 0] * Y[0 * 3 + b] + F[a * 3 + 1] * Y[1 * 3 + b] + F[a * 3 + 2] * Y[2 * 3 + b];
  // (I + Y)^-1 = cof(I + Y)^T / det, and cof of a symmetric matrix is symmetric
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      FmR[a * 3 + b] = (FY[a * 3 + 0] * Mc[0 * 3 + b] + FY[a * 3 + 1] * Mc[1 * 3 + b] + FY[a * 3 + 2] * Mc[2 * 3 + b]) *
                       inv_det;
  return true;
}

template <int DIM, typename T>
__device__ __forceinline__ void affine_of(const KParams<T>& kp, const T* F, const T* C, T m, T mu, T lam, T* A,
                                          uint32_t* fallbacks) {
  const T Dinv = T(4) * kp.inv_dx * kp.inv_dx;
  const T s = -(kp.dt * kp.volume);
  if constexpr (DIM == 3) {
    T FmR[9];
    bool small = false;
    if constexpr (sizeof(T) == 4) small = f_minus_r_small_strain3(F, FmR);
    if (!small) {
      T R[9];
      polar3<T>(F, R, fallbacks);
#pragma unroll
      for (int i = 0; i < 9; ++i) FmR[i] = F[i] - R[i];
    }
    const T J = det3(F);
    const T sc = lam * (J - T(1)) * J;
#pragma unroll
    for (int i = 0; i < 9; ++i) FmR[i] *= T(2) * mu;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T pf = FmR[i * 3 + 0] * F[j * 3 + 0] + FmR[i * 3 + 1] * F[j * 3 + 1] + FmR[i * 3 + 2] * F[j * 3 + 2] +
                     ((i == j || kp.model != FFMPM_MODEL_FIXED_COROTATED) ? sc : T(0));
        A[i * 3 + j] = s * (Dinv * pf) + m * C[i * 3 + j];
      }
  } else {
    T R[4];
    polar2<T>(F, R);
    const T J = F[0] * F[3] - F[1] * F[2];
    const T sc = lam * (J - T(1)) * J;
    T FmR[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) FmR[i] = T(2) * mu * (F[i] - R[i]);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const T pf = FmR[i * 2 + 0] * F[j * 2 + 0] + FmR[i * 2 + 1] * F[j * 2 + 1] +
                     ((i == j || kp.model != FFMPM_MODEL_FIXED_COROTATED) ? sc : T(0));
        A[i * 2 + j] = s * (Dinv * pf) + m * C[i * 2 + j];
      }
  }
}

template <typename T>
__device__ __forceinline__ void lame_of(const KParams<T>& kp, const PView<T>& P, uint32_t p, T& m, T& mu, T& lam) {
  m = P.mass ? P.mass[p] : kp.mass;
  const T mu0 = P.mu0 ? P.mu0[p] : kp.mu0;
  const T lam0 = P.lam0 ? P.lam0[p] : kp.lam0;
  const T e = (kp.model == FFMPM_MODEL_SNOW) ? ffexp(kp.hardening * (T(1) - P.Jp[p])) : kp.hardening;
  mu = mu0 * e;
  lam = lam0 * e;
}

// Shared-memory float add whose result is not needed: a reduction (red), not a read-modify-write
// that returns the old value.
__device__ __forceinline__ void smem_add(float* p, float v) {
  asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(p))), "f"(v)
               : "memory");
}
__device__ __forceinline__ void smem_add(double* p, double v) { atomicAdd(p, v); }

// Accumulation targets of one particle's 3^DIM contributions, addressed by node coordinates
// relative to the block origin.

template <int DIM, typename T>
struct TileAdder {  // shared tile, SoA: 4 arrays of TN values
  T* tile;
  int TN, T1;
  __device__ __forceinline__ void add(int li, int lj, int lk, T a, T b, T c, T m) const {
    const int idx = DIM == 3 ? (li * T1 + lj) * T1 + lk : li * T1 + lj;
    smem_add(&tile[idx], a);
    smem_add(&tile[TN + idx], b);
    if constexpr (DIM == 3) smem_add(&tile[2 * TN + idx], c);
    smem_add(&tile[3 * TN + idx], m);
  }
};

template <int DIM, typename T, typename Sink>
struct DirectAdder {  // global grid through the sink (one vector red per node)
  Sink sink;
  int R;
  int org[DIM];
  __device__ __forceinline__ void add(int li, int lj, int lk, T a, T b, T c, T m) const {
    int I[DIM];
    I[0] = org[0] + li;
    I[1] = org[1] + lj;
    if constexpr (DIM == 3) I[2] = org[2] + lk;
    sink.add(node_index<DIM>(R, I), a, b, c, m);
  }
};

// Scatter one particle: stress, APIC affine, 3^DIM weighted contributions into `acc`.
template <int DIM, typename T, typename Adder>
__device__ __forceinline__ void p2g_particle(const KParams<T>& kp, const Geom<DIM>& g, const PView<T>& P, uint32_t p,
                                             const int org[DIM], const Adder& acc, int32_t* status,
                                             uint32_t* fallbacks) {
  constexpr int DD = DIM * DIM;
  T fx[DIM], w[3][DIM];
  int lb[DIM];
  bool ok = true;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    int b;
    ok = ok && base_of(P.x[P.at(p, d, DIM)], kp.inv_dx, kp.res, b, fx[d]);
    lb[d] = b - org[d];
    ok = ok && lb[d] >= 0 && lb[d] + 2 < g.tile;
    T ww[3];
    bspline(fx[d], ww);
    w[0][d] = ww[0];
    w[1][d] = ww[1];
    w[2][d] = ww[2];
  }
  if (!ok) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T m, mu, lam;
  lame_of(kp, P, p, m, mu, lam);
  T F[DD], C[DD], A[DD], v[DIM];
#pragma unroll
  for (int i = 0; i < DD; ++i) {
    F[i] = P.F[P.at(p, i, DD)];
    C[i] = P.C[P.at(p, i, DD)];
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) v[d] = P.v[P.at(p, d, DIM)];
  affine_of<DIM, T>(kp, F, C, m, mu, lam, A, fallbacks);
  const T dx = kp.dx;
  T mv[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) mv[d] = v[d] * m;
  if constexpr (DIM == 3) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T d0 = (T(i) - fx[0]) * dx;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T d1 = (T(j) - fx[1]) * dx;
        const T wij = w[i][0] * w[j][1];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const T d2 = (T(k) - fx[2]) * dx;
          const T weight = wij * w[k][2];
          acc.add(lb[0] + i, lb[1] + j, lb[2] + k, weight * (mv[0] + (A[0] * d0 + A[1] * d1 + A[2] * d2)),
                  weight * (mv[1] + (A[3] * d0 + A[4] * d1 + A[5] * d2)),
                  weight * (mv[2] + (A[6] * d0 + A[7] * d1 + A[8] * d2)), weight * m);
        }
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T d0 = (T(i) - fx[0]) * dx;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T d1 = (T(j) - fx[1]) * dx;
        const T weight = w[i][0] * w[j][1];
        acc.add(lb[0] + i, lb[1] + j, 0, weight * (mv[0] + (A[0] * d0 + A[1] * d1)),
                weight * (mv[1] + (A[2] * d0 + A[3] * d1)), T(0), weight * m);
      }
    }
  }
}

template <int DIM, typename T, typename Sink>
__device__ __forceinline__ void p2g_flush(const T* tile, int TN, const Geom<DIM>& g, const int org[DIM],
                                          const Sink& sink) {
  const int T1 = g.tile;
  for (int t = threadIdx.x; t < TN; t += blockDim.x) {
    const T a = tile[t], b = tile[TN + t], c = tile[2 * TN + t], m = tile[3 * TN + t];
    if (a == T(0) && b == T(0) && c == T(0) && m == T(0)) continue;
    int I[DIM];
    if constexpr (DIM == 3) {
      I[0] = org[0] + t / (T1 * T1);
      I[1] = org[1] + (t / T1) % T1;
      I[2] = org[2] + t % T1;
    } else {
      I[0] = org[0] + t / T1;
      I[1] = org[1] + t % T1;
    }
    bool in = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) in = in && I[d] < g.R;
    if (in) sink.add(node_index<DIM>(g.R, I), a, b, c, m);
  }
}

// ----------------------------------------------------------------------------------------------
// Cell-run P2G.  Particles arrive sorted by cell inside their block, so a chunk holds runs of
// particles that share a base cell and therefore all 3^DIM stencil nodes.  Phase 1 (one thread per
// particle) computes each particle's record once.  Phase 2 finds the runs.  Phase 3 gives each run
// to a warp whose lanes are the stencil nodes: every lane sums its node's contributions over the
// run's particles in registers and adds the sum to the shared tile once, so the tile sees one
// atomic per (node, run) instead of one per (node, particle).
//
// Record (floats): [m, q (DIM), a = dx A (DIM^2, row-major), wx0..2, wy0..2 (, wz0..2)] with
// q = m v - dx A fx; the contribution to node o is w_o (q + a o, m), algebraically the reference's
// w (m v + A (o - fx) dx, m).
template <int DIM>
struct RecLayout {
  static constexpr int kFloats = DIM == 3 ? 22 : 13;  // m, q (DIM), dx A (DIM^2), weights (3 DIM)
  // 7 (3D) / 5 (2D) float4 per record: 16-byte aligned vector accesses, and the per-thread vector
  // stores of phase 1 fall on distinct bank groups (stride 112 B / 80 B).
  static constexpr int kStride = DIM == 3 ? 28 : 20;
  static constexpr int kW = DIM == 3 ? 13 : 7;  // first weight
  static_assert(kFloats == 1 + DIM + DIM * DIM + 3 * DIM, "record size");
};

// The state P2G reads of one particle (loaded ahead of the arithmetic so that the loads of
// several particles are in flight together).
template <int DIM, typename T>
struct P2GIn {
  T x[DIM], v[DIM], F[DIM * DIM], C[DIM * DIM];
  T m, mu0, lam0, jp;
};

template <int DIM, typename T>
__device__ __forceinline__ void p2g_load(const KParams<T>& kp, const PView<T>& P, uint32_t p, P2GIn<DIM, T>& in) {
  constexpr int DD = DIM * DIM;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    in.x[d] = P.x[P.at(p, d, DIM)];
    in.v[d] = P.v[P.at(p, d, DIM)];
  }
#pragma unroll
  for (int i = 0; i < DD; ++i) {
    in.F[i] = P.F[P.at(p, i, DD)];
    in.C[i] = P.C[P.at(p, i, DD)];
  }
  in.m = P.mass ? P.mass[p] : kp.mass;
  in.mu0 = P.mu0 ? P.mu0[p] : kp.mu0;
  in.lam0 = P.lam0 ? P.lam0[p] : kp.lam0;
  in.jp = kp.model == FFMPM_MODEL_SNOW ? P.Jp[p] : T(1);
}

// Record of one particle.  Returns kRecTile when its stencil lies in the chunk block's tile,
// kRecStray when it is inside the grid but its stencil left that tile (possible between re-sorts;
// the record is complete and base[] holds its base node), kRecOut when it is outside the grid.
constexpr int kRecOut = 0, kRecTile = 1, kRecStray = 2;

template <int DIM, typename T>
__device__ __forceinline__ int p2g_record(const KParams<T>& kp, const Geom<DIM>& g, const P2GIn<DIM, T>& in,
                                          const int org[DIM], T* rec, int& cell, int32_t* status,
                                          uint32_t* fallbacks, int base[DIM]) {
  constexpr int DD = DIM * DIM;
  T fx[DIM];
  int lb[DIM];
  bool ok = true, in_tile = true;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    int b;
    ok = ok && base_of(in.x[d], kp.inv_dx, kp.res, b, fx[d]);
    base[d] = b;
    lb[d] = b - org[d];
    in_tile = in_tile && lb[d] >= 0 && lb[d] + 2 < g.tile;
  }
  if (!ok) {
    raise_status(status, FFMPM_STATUS_OOB);
    return kRecOut;
  }
  cell = in_tile ? (DIM == 3 ? (lb[0] * g.bs + lb[1]) * g.bs + lb[2] : lb[0] * g.bs + lb[1]) : -1;
  const T m = in.m;
  const T e = (kp.model == FFMPM_MODEL_SNOW) ? ffexp(kp.hardening * (T(1) - in.jp)) : kp.hardening;
  T A[DD];
  affine_of<DIM, T>(kp, in.F, in.C, m, in.mu0 * e, in.lam0 * e, A, fallbacks);
  const T dx = kp.dx;
  rec[0] = m;
#pragma unroll
  for (int r = 0; r < DIM; ++r) {
    T af = T(0);
#pragma unroll
    for (int c = 0; c < DIM; ++c) af += A[r * DIM + c] * fx[c];
    rec[1 + r] = in.v[r] * m - dx * af;
  }
  constexpr int a0 = DIM == 3 ? 4 : 3;
#pragma unroll
  for (int i = 0; i < DD; ++i) rec[a0 + i] = dx * A[i];
  // the weights last: they are not live during the stress
  constexpr int w0 = RecLayout<DIM>::kW;
#pragma unroll
  for (int d = 0; d < DIM; ++d) bspline(fx[d], rec + w0 + 3 * d);
  return in_tile ? kRecTile : kRecStray;
}

// Scatter one record (in shared memory) straight to the global grid through the sink: a particle
// whose stencil left its chunk block's tile.  Its base node is in the record's padding,
// rec[kFloats + d] (exact: node indices are far below 2^24).  Node (i, j[, k]) gets
// w (q + dx A (i, j[, k])) and w m.
template <int DIM, typename T, typename Sink>
__device__ void p2g_scatter_record(const T* rec, int R, const Sink& sink) {
  constexpr int a0 = 1 + DIM;
  constexpr int w0 = RecLayout<DIM>::kW;
  int base[DIM];
  for (int d = 0; d < DIM; ++d) base[d] = static_cast<int>(rec[RecLayout<DIM>::kFloats + d]);
  const T m = rec[0];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < (DIM == 3 ? 3 : 1); ++k) {
        const int o[3] = {i, j, k};
        T wt = rec[w0 + i] * rec[w0 + 3 + j];
        if constexpr (DIM == 3) wt *= rec[w0 + 6 + k];
        T q[3] = {T(0), T(0), T(0)};
        for (int r = 0; r < DIM; ++r) {
          T a = rec[1 + r];
          for (int c = 0; c < DIM; ++c) a += rec[a0 + r * DIM + c] * T(o[c]);
          q[r] = wt * a;
        }
        int I[DIM];
        for (int d = 0; d < DIM; ++d) I[d] = base[d] + o[d];
        sink.add(node_index<DIM>(R, I), q[0], q[1], DIM == 3 ? q[2] : T(0), wt * m);
      }
}

// Shared-memory arrays of the cell-run P2G (phases 2 and 3).
template <typename T>
struct CellRunSmem {
  T* recs;     // [kChunk][RecLayout::kStride]
  int* cells;  // [kChunk] cell of each record (negative: no tile contribution)
  int* rank;   // [kChunk]
  int* order;  // [kChunk]
  int* runs;   // [max(kChunk, ncell) + 1]
  int* hist;   // [ncell]
  int* nruns;  // 1
  int* warp_cnt;
  int* warp_nz;  // [kThreads / 32] each
};

// Bytes of the cell-run arrays (records + the int arrays) after the tile, for block side bs.
template <int DIM, typename T>
__host__ __device__ constexpr size_t cell_run_smem_bytes(int bs) {
  const int ncell = DIM == 3 ? bs * bs * bs : bs * bs;
  return size_t(kChunk) * RecLayout<DIM>::kStride * sizeof(T) +
         sizeof(int) * (3 * kChunk + (kChunk > ncell ? kChunk : ncell) + 1 + ncell);
}

template <int DIM, typename T>
__device__ __forceinline__ CellRunSmem<T> cell_run_smem(unsigned char* at, const Geom<DIM>& g, int* nruns,
                                                        int* warp_cnt, int* warp_nz) {
  const int ncell = DIM == 3 ? g.bs * g.bs * g.bs : g.bs * g.bs;
  CellRunSmem<T> cr;
  cr.recs = reinterpret_cast<T*>(at);
  cr.cells = reinterpret_cast<int*>(cr.recs + (size_t)kChunk * RecLayout<DIM>::kStride);
  cr.rank = cr.cells + kChunk;
  cr.order = cr.rank + kChunk;
  cr.runs = cr.order + kChunk;
  cr.hist = cr.runs + max(kChunk, ncell) + 1;
  cr.nruns = nruns;
  cr.warp_cnt = warp_cnt;
  cr.warp_nz = warp_nz;
  return cr;
}

// Phase-1 tail: store record `rec` (of kind kRecTile / kRecStray / kRecOut) as record l.  Cell -1
// marks a particle outside the grid, -2 one whose stencil left the block's tile (scattered to the
// global grid after the phase; its base node rides in the record's padding).
template <int DIM, typename T>
__device__ __forceinline__ void p2g_store_record(const CellRunSmem<T>& cr, int l, T* rec, int kind, int cell,
                                                 const int base[DIM]) {
  constexpr int RF = RecLayout<DIM>::kFloats;
  constexpr int RS = RecLayout<DIM>::kStride;
#pragma unroll
  for (int i = RF; i < RS; ++i) rec[i] = T(0);
  if (kind == kRecStray) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) rec[RF + d] = T(base[d]);
    cell = -2;
  } else if (kind != kRecTile) {
    cell = -1;
  }
  Node4<T>* dst = reinterpret_cast<Node4<T>*>(cr.recs + (size_t)l * RS);
#pragma unroll
  for (int i = 0; i < RS / 4; ++i) dst[i] = Node4<T>{rec[4 * i], rec[4 * i + 1], rec[4 * i + 2], rec[4 * i + 3]};
  cr.cells[l] = cell;
}

// Phases 2 and 3 of the cell-run P2G over the nrec records of one chunk (phase 1 has filled
// recs/cells and synchronised): group the records by cell, then add every cell's run to the tile.
// Ends with the tile adds issued (no trailing barrier).
template <int DIM, typename T>
__device__ __forceinline__ void p2g_cell_runs(const CellRunSmem<T>& cr, const Geom<DIM>& g, int nrec,
                                              const TileAdder<DIM, T>& tacc) {
  constexpr int RS = RecLayout<DIM>::kStride;
  const int ncell = DIM == 3 ? g.bs * g.bs * g.bs : g.bs * g.bs;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* const recs = cr.recs;
  int* const cells = cr.cells;
  int* const rank = cr.rank;
  int* const order = cr.order;
  int* const runs = cr.runs;
  int* const hist = cr.hist;
  int* const warp_cnt = cr.warp_cnt;
  int* const warp_nz = cr.warp_nz;
  // phase 2: group the chunk's particles by cell with a counting sort in shared memory (the
  // chunk's order can come from a re-sort several substeps old, so equal cells need not be
  // adjacent).  Run r is order[runs[r] .. runs[r + 1]): the particles of one cell.  Particles
  // with cell -1 (outside the grid, or strays handled in phase 1) are left out.
  {
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) hist[c] = 0;
    __syncthreads();
    // one shared atomic per distinct cell of a warp (neighbouring particles mostly share a cell)
    for (int l = threadIdx.x; l < nrec; l += blockDim.x) {
      const int c = cells[l];
      const unsigned act = __activemask();
      const unsigned peers = __match_any_sync(act, c);
      const int leader = __ffs(peers) - 1;
      int first = 0;
      if (c >= 0 && lane == leader) first = atomicAdd(&hist[c], __popc(peers));
      first = __shfl_sync(peers, first, leader);
      rank[l] = c >= 0 ? first + __popc(peers & lanemask_lt()) : -1;
    }
    __syncthreads();
    const int per_t = (ncell + blockDim.x - 1) / blockDim.x;
    const int beg = threadIdx.x * per_t;
    const int end = min(ncell, beg + per_t);
    int cnt = 0, nz = 0;
    for (int c = beg; c < end; ++c) {
      cnt += hist[c];
      nz += hist[c] > 0;
    }
    int icnt = cnt, inz = nz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int tc = __shfl_up_sync(0xffffffffu, icnt, o), tz = __shfl_up_sync(0xffffffffu, inz, o);
      if (lane >= o) {
        icnt += tc;
        inz += tz;
      }
    }
    if (lane == 31) {
      warp_cnt[warp] = icnt;
      warp_nz[warp] = inz;
    }
    __syncthreads();
    int pos = 0, r = 0, tot_cnt = 0, tot_nz = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
      pos += w < warp ? warp_cnt[w] : 0;
      r += w < warp ? warp_nz[w] : 0;
      tot_cnt += warp_cnt[w];
      tot_nz += warp_nz[w];
    }
    pos += icnt - cnt;
    r += inz - nz;
    for (int c = beg; c < end; ++c) {
      const int h = hist[c];
      if (h > 0) runs[r++] = pos;
      hist[c] = pos;  // start of cell c in order[]
      pos += h;
    }
    if (threadIdx.x == 0) {
      *cr.nruns = tot_nz;
      runs[tot_nz] = tot_cnt;
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nrec; l += blockDim.x) {
      const int c = cells[l];
      if (c >= 0) order[hist[c] + rank[l]] = l;
    }
  }
  __syncthreads();
  const int nruns = *cr.nruns;
  // phase 3: a warp per run.  A particle is served by LP lanes (3D: 9, one per (j, k); 2D: 3, one
  // per j); each lane accumulates the 3 nodes along x (i = 0, 1, 2) of its (j, k), and the warp
  // takes NG particles of the run per step.  The NG partial sums are then folded onto group 0.
  constexpr int LP = DIM == 3 ? 9 : 3;
  constexpr int NG = 32 / LP;  // 3 (3D) or 10 (2D) particles per step
  const int grp = lane / LP;
  const int jk = lane - grp * LP;
  const bool active = grp < NG;
  const int oj = DIM == 3 ? jk / 3 : jk, ok = DIM == 3 ? jk % 3 : 0;
  constexpr int a0 = 1 + DIM;
  constexpr int w0 = RecLayout<DIM>::kW;
  for (int r = warp; r < nruns; r += kThreads / 32) {
    const int l0 = runs[r], l1 = runs[r + 1];
    T acc[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = T(0);
    if (active) {
      // a lane needs m, q, dx A and the x weights (the first RU floats: whole float4s) and its own
      // y (and z) weight; two records per step, both loaded before either is accumulated
      constexpr int RU = DIM == 3 ? 16 : 12;
      struct Rv {
        T v[RU];
        T wjk;
      };
      auto load = [&](int ll, Rv& rv) {
        const T* rc = recs + (size_t)order[ll] * RS;
        const Node4<T>* src = reinterpret_cast<const Node4<T>*>(rc);
#pragma unroll
        for (int i = 0; i < RU / 4; ++i) {
          const Node4<T> q4 = src[i];
          rv.v[4 * i] = q4.x;
          rv.v[4 * i + 1] = q4.y;
          rv.v[4 * i + 2] = q4.z;
          rv.v[4 * i + 3] = q4.w;
        }
        if constexpr (DIM == 3)
          rv.wjk = rc[w0 + 3 + oj] * rc[w0 + 6 + ok];
        else
          rv.wjk = rc[w0 + 3 + oj];
      };
      auto accum = [&](const Rv& r) {
        const T* rv = r.v;
        const T m = rv[0];
        const T wjk = r.wjk;
        // base_r = q_r + a_r1 j (+ a_r2 k); node i adds i * a_r0
        T base[DIM], step[DIM];
#pragma unroll
        for (int rr = 0; rr < DIM; ++rr) {
          T b = rv[1 + rr] + rv[a0 + rr * DIM + 1] * T(oj);
          if constexpr (DIM == 3) b += rv[a0 + rr * DIM + 2] * T(ok);
          base[rr] = b;
          step[rr] = rv[a0 + rr * DIM];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const T wgt = rv[w0 + i] * wjk;
#pragma unroll
          for (int rr = 0; rr < DIM; ++rr) acc[i][rr] += wgt * (base[rr] + T(i) * step[rr]);
          acc[i][3] += wgt * m;
        }
      };
      int ll = l0 + grp;
      for (; ll + NG < l1; ll += 2 * NG) {
        Rv ra, rb;
        load(ll, ra);
        load(ll + NG, rb);
        accum(ra);
        accum(rb);
      }
      if (ll < l1) {
        Rv ra;
        load(ll, ra);
        accum(ra);
      }
    }
    // fold the NG groups onto group 0 (lanes 0..LP-1)
#pragma unroll
    for (int off = 1; off < NG; off <<= 1) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const T t = __shfl_down_sync(0xffffffffu, acc[i][c], off * LP);
          if (grp % (2 * off) == 0 && grp + off < NG) acc[i][c] += t;
        }
    }
    if (grp == 0) {
      const int cl = cells[order[l0]];
      int lb[DIM];
      if constexpr (DIM == 3) {
        lb[2] = cl & (g.bs - 1);
        lb[1] = (cl >> g.bs_shift) & (g.bs - 1);
        lb[0] = cl >> (2 * g.bs_shift);
#pragma unroll
        for (int i = 0; i < 3; ++i)
          tacc.add(lb[0] + i, lb[1] + oj, lb[2] + ok, acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
      } else {
        lb[1] = cl & (g.bs - 1);
        lb[0] = cl >> g.bs_shift;
#pragma unroll
        for (int i = 0; i < 3; ++i) tacc.add(lb[0] + i, lb[1] + oj, 0, acc[i][0], acc[i][1], T(0), acc[i][3]);
      }
    }
  }
}

template <int DIM, typename T, typename Sink>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1) k_p2g_cells(KParams<T> kp, Geom<DIM> g, PView<T> P,
                                                        const uint32_t* __restrict__ perm,
                                                        const int4* __restrict__ chunks,
                                                        const WsHeader* __restrict__ hdr, Sink sink, int32_t* status,
                                                        uint32_t* fallbacks, const uint32_t* __restrict__ sort_flag) {
  if (sort_flag && *sort_flag == 0u) perm = nullptr;  // plan kept from an earlier substep: identity order
  if (perm && wait_gave_up(status)) return;
  constexpr int RS = RecLayout<DIM>::kStride;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int TN = tile_nodes<DIM>(g);
  T* tile = reinterpret_cast<T*>(smem_raw);
  __shared__ int nruns_s;
  __shared__ int warp_cnt[kThreads / 32];
  __shared__ int warp_nz[kThreads / 32];
  const CellRunSmem<T> cr = cell_run_smem<DIM, T>(reinterpret_cast<unsigned char*>(tile + 4 * TN), g, &nruns_s,
                                                  warp_cnt, warp_nz);
  const uint32_t nch = hdr->n_chunks;
  const uint32_t per = (nch + gridDim.x - 1) / gridDim.x;
  const uint32_t c0 = blockIdx.x * per;
  const uint32_t c1 = min(nch, c0 + per);
  const TileAdder<DIM, T> tacc{tile, TN, g.tile};
  int cur = -1;
  int org[DIM];
  for (uint32_t c = c0; c < c1; ++c) {
    const int4 ch = chunks[c];
    if (ch.x != cur) {
      if (cur >= 0) {
        __syncthreads();
        p2g_flush<DIM, T, Sink>(tile, TN, g, org, sink);
      }
      __syncthreads();
      for (int t = threadIdx.x; t < 4 * TN; t += blockDim.x) tile[t] = T(0);
      cur = ch.x;
      int bc[DIM];
      block_coords<DIM>(g, cur, bc);
#pragma unroll
      for (int d = 0; d < DIM; ++d) org[d] = bc[d] * g.bs;
    }
    // phase 1: one record per particle and thread.  One particle at a time: two in flight per
    // thread cost more registers than their overlapped loads gain.
    for (int l = threadIdx.x; l < ch.z; l += blockDim.x) {
      const uint32_t s = ch.y + l;
      P2GIn<DIM, T> in;
      p2g_load<DIM, T>(kp, P, perm ? perm[s] : s, in);
      T rec[RS];
      int cell = -1, base[DIM];
      const int kind = p2g_record<DIM, T>(kp, g, in, org, rec, cell, status, fallbacks, base);
      p2g_store_record<DIM, T>(cr, l, rec, kind, cell, base);
    }
    __syncthreads();
    // particles whose stencil left the block's tile (only between re-sorts): direct global adds
    for (int l = threadIdx.x; l < ch.z; l += blockDim.x)
      if (cr.cells[l] == -2) p2g_scatter_record<DIM, T, Sink>(cr.recs + (size_t)l * RS, g.R, sink);
    p2g_cell_runs<DIM, T>(cr, g, ch.z, tacc);
    __syncthreads();  // records and runs are rewritten by the next chunk
  }
  if (cur >= 0) {
    __syncthreads();
    p2g_flush<DIM, T, Sink>(tile, TN, g, org, sink);
  }
}

// ----------------------------------------------------------------------------------------------
// Deterministic P2G.  One CTA sums each occupied block.  Runs (as in k_p2g_cells) go to warps by a fixed
// rule (run r of a chunk -> warp r mod 8) and every warp adds its runs' node sums, in run order,
// into its own shared tile without atomics; the eight tiles are summed in warp order into the
// block's staging tile.  The grid update then sums the (at most 2^DIM) staged tiles that cover a
// node in a fixed block order.  Every floating-point sum therefore has a fixed order and the
// result is bit-identical from run to run.
template <int DIM, typename T>
__host__ __device__ constexpr size_t p2g_det_smem_bytes(int TN) {
  return size_t(kThreads / 32) * 4 * TN * sizeof(T) + size_t(kChunk) * RecLayout<DIM>::kStride * sizeof(T) +
         sizeof(int) * (2 * kChunk + 1);
}

template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_p2g_det(KParams<T> kp, Geom<DIM> g, PView<T> P,
                                                      const uint32_t* __restrict__ perm,
                                                      const int4* __restrict__ occupied,
                                                      const WsHeader* __restrict__ hdr, Node4<T>* __restrict__ stage,
                                                      int32_t* status, uint32_t* fallbacks, uint32_t* next) {
  if (wait_gave_up(status)) return;
  constexpr int RF = RecLayout<DIM>::kFloats;
  constexpr int RS = RecLayout<DIM>::kStride;
  constexpr int NW = kThreads / 32;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int TN = tile_nodes<DIM>(g);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* wtiles = reinterpret_cast<T*>(smem_raw);           // [NW][4][TN]
  T* recs = wtiles + (size_t)NW * 4 * TN;                // [kChunk][RS]
  int* cells = reinterpret_cast<int*>(recs + (size_t)kChunk * RS);
  int* runs = cells + kChunk;                            // [kChunk + 1]
  __shared__ int nruns_s;
  __shared__ int warp_cnt[kThreads / 32];
  T* mytile = wtiles + (size_t)warp * 4 * TN;
  const int T1 = g.tile;
  constexpr int LP = DIM == 3 ? 9 : 3;
  constexpr int NG = 32 / LP;
  const int grp = lane / LP;
  const int jk = lane - grp * LP;
  const bool active = grp < NG;
  const int oj = DIM == 3 ? jk / 3 : jk, ok = DIM == 3 ? jk % 3 : 0;
  constexpr int a0 = 1 + DIM;
  constexpr int w0 = RecLayout<DIM>::kW;
  const uint32_t nocc = hdr->n_occupied;
  __shared__ uint32_t next_s;
  // Blocks go to CTAs through two shared counters (zeroed before the launch): the first pass takes
  // the blocks of at least two full chunks, the second the rest, so that the large work items
  // start first and the CTAs finish close together.  Which CTA sums a block changes no sum: each
  // block is summed by one CTA, in the fixed order below, into its own staging tile.
  int pass = 0;
  for (;;) {
    __syncthreads();  // every thread has read next_s and finished the previous block
    if (threadIdx.x == 0) next_s = atomicAdd(&next[pass], 1u);
    __syncthreads();
    const uint32_t ob = next_s;
    if (ob >= nocc) {
      if (++pass == 2) break;
      continue;
    }
    const int4 occ = occupied[ob];
    if ((occ.z >= 2 * kChunk) != (pass == 0)) continue;
    int org[DIM];
    {
      int bc[DIM];
      block_coords<DIM>(g, occ.x, bc);
#pragma unroll
      for (int d = 0; d < DIM; ++d) org[d] = bc[d] * g.bs;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < NW * 4 * TN; t += blockDim.x) wtiles[t] = T(0);
    for (int c0 = 0; c0 < occ.z; c0 += kChunk) {
      const int cz = min(kChunk, occ.z - c0);
      const uint32_t s0 = (uint32_t)(occ.y + c0);
      __syncthreads();  // tiles zeroed / previous chunk's records consumed
      // one particle per thread at a time (two in flight cost more registers than they gain)
      for (int l = threadIdx.x; l < cz; l += blockDim.x) {
        P2GIn<DIM, T> in;
        p2g_load<DIM, T>(kp, P, perm[s0 + l], in);
        T rec[RS];
        int cell = -1;
        int base[DIM];
        if (p2g_record<DIM, T>(kp, g, in, org, rec, cell, status, fallbacks, base) != kRecTile) {
          if (cell < 0) raise_status(status, FFMPM_STATUS_OOB);  // a fresh plan has no strays
          cell = -1;
        }
#pragma unroll
        for (int i = RF; i < RS; ++i) rec[i] = T(0);
        Node4<T>* dst = reinterpret_cast<Node4<T>*>(recs + (size_t)l * RS);
#pragma unroll
        for (int i = 0; i < RS / 4; ++i) dst[i] = Node4<T>{rec[4 * i], rec[4 * i + 1], rec[4 * i + 2], rec[4 * i + 3]};
        cells[l] = cell;
      }
      __syncthreads();
      {
        const int per_t = (cz + blockDim.x - 1) / blockDim.x;
        const int beg = threadIdx.x * per_t;
        int heads = 0;
        for (int l = beg; l < min(cz, beg + per_t); ++l) heads += (l == 0 || cells[l] != cells[l - 1]);
        int inc = heads;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += t;
        }
        if (lane == 31) warp_cnt[warp] = inc;
        __syncthreads();
        int before = 0, tot = 0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) {
          before += w < warp ? warp_cnt[w] : 0;
          tot += warp_cnt[w];
        }
        int r = before + inc - heads;
        for (int l = beg; l < min(cz, beg + per_t); ++l)
          if (l == 0 || cells[l] != cells[l - 1]) runs[r++] = l;
        if (threadIdx.x == 0) {
          nruns_s = tot;
          runs[tot] = cz;
        }
      }
      __syncthreads();
      const int nruns = nruns_s;
      for (int r = warp; r < nruns; r += NW) {
        const int l0 = runs[r], l1 = runs[r + 1];
        const int cl = cells[l0];
        if (cl < 0) continue;
        T acc[3][4];
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = T(0);
        if (active) {
          // as in p2g_cell_runs: a lane loads m, q, dx A and the x weights (RU floats) and its own
          // y (and z) weight; two records per step, added in the same order as one at a time
          constexpr int RU = DIM == 3 ? 16 : 12;
          struct Rv {
            T v[RU];
            T wjk;
          };
          const auto load = [&](int l, Rv& rv) {
            const T* rc = recs + (size_t)l * RS;
            const Node4<T>* src = reinterpret_cast<const Node4<T>*>(rc);
#pragma unroll
            for (int i = 0; i < RU / 4; ++i) {
              const Node4<T> q4 = src[i];
              rv.v[4 * i] = q4.x;
              rv.v[4 * i + 1] = q4.y;
              rv.v[4 * i + 2] = q4.z;
              rv.v[4 * i + 3] = q4.w;
            }
            if constexpr (DIM == 3)
              rv.wjk = rc[w0 + 3 + oj] * rc[w0 + 6 + ok];
            else
              rv.wjk = rc[w0 + 3 + oj];
          };
          const auto accum = [&](const Rv& r) {
            const T* rv = r.v;
            const T m = rv[0];
            T bse[DIM], stp[DIM];
#pragma unroll
            for (int rr = 0; rr < DIM; ++rr) {
              T b = rv[1 + rr] + rv[a0 + rr * DIM + 1] * T(oj);
              if constexpr (DIM == 3) b += rv[a0 + rr * DIM + 2] * T(ok);
              bse[rr] = b;
              stp[rr] = rv[a0 + rr * DIM];
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              const T wgt = rv[w0 + i] * r.wjk;
#pragma unroll
              for (int rr = 0; rr < DIM; ++rr) acc[i][rr] += wgt * (bse[rr] + T(i) * stp[rr]);
              acc[i][3] += wgt * m;
            }
          };
          int l = l0 + grp;
          for (; l + NG < l1; l += 2 * NG) {
            Rv ra, rb;
            load(l, ra);
            load(l + NG, rb);
            accum(ra);
            accum(rb);
          }
          if (l < l1) {
            Rv ra;
            load(l, ra);
            accum(ra);
          }
        }
#pragma unroll
        for (int off = 1; off < NG; off <<= 1) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
              const T t = __shfl_down_sync(0xffffffffu, acc[i][cc], off * LP);
              if (grp % (2 * off) == 0 && grp + off < NG) acc[i][cc] += t;
            }
        }
        if (grp == 0) {
          int lb[DIM];
          if constexpr (DIM == 3) {
            lb[2] = cl & (g.bs - 1);
            lb[1] = (cl >> g.bs_shift) & (g.bs - 1);
            lb[0] = cl >> (2 * g.bs_shift);
          } else {
            lb[1] = cl & (g.bs - 1);
            lb[0] = cl >> g.bs_shift;
          }
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const int idx = DIM == 3 ? ((lb[0] + i) * T1 + lb[1] + oj) * T1 + lb[2] + ok : (lb[0] + i) * T1 + lb[1] + oj;
            mytile[idx] += acc[i][0];
            mytile[TN + idx] += acc[i][1];
            if constexpr (DIM == 3) mytile[2 * TN + idx] += acc[i][2];
            mytile[3 * TN + idx] += acc[i][3];
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    // the block's staging tile: warp tiles summed in warp order
    Node4<T>* st = stage + (size_t)occ.x * TN;
    for (int t = threadIdx.x; t < TN; t += blockDim.x) {
      T a = T(0), b = T(0), c = T(0), m = T(0);
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const T* wt = wtiles + (size_t)w * 4 * TN;
        a += wt[t];
        b += wt[TN + t];
        c += wt[2 * TN + t];
        m += wt[3 * TN + t];
      }
      st[t] = Node4<T>{a, b, c, m};
    }
  }
}

template <int DIM, typename T, typename Sink, bool kDirect>
__global__ void __launch_bounds__(kThreads) k_p2g(KParams<T> kp, Geom<DIM> g, PView<T> P,
                                                  const uint32_t* __restrict__ perm, const int4* __restrict__ chunks,
                                                  const WsHeader* __restrict__ hdr, Sink sink, int32_t* status,
                                                  uint32_t* fallbacks) {
  if (wait_gave_up(status)) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);
  const int TN = tile_nodes<DIM>(g);
  const uint32_t nch = hdr->n_chunks;
  const uint32_t per = (nch + gridDim.x - 1) / gridDim.x;
  const uint32_t c0 = blockIdx.x * per;
  const uint32_t c1 = min(nch, c0 + per);
  if constexpr (kDirect) {
    for (uint32_t c = c0; c < c1; ++c) {
      const int4 ch = chunks[c];
      DirectAdder<DIM, T, Sink> acc;
      acc.sink = sink;
      acc.R = g.R;
      int bc[DIM];
      block_coords<DIM>(g, ch.x, bc);
#pragma unroll
      for (int d = 0; d < DIM; ++d) acc.org[d] = bc[d] * g.bs;
      for (int l = threadIdx.x; l < ch.z; l += blockDim.x)
        p2g_particle<DIM, T>(kp, g, P, perm[ch.y + l], acc.org, acc, status, fallbacks);
    }
    return;
  }
  const TileAdder<DIM, T> tacc{tile, TN, g.tile};
  int cur = -1;
  int org[DIM];
  for (uint32_t c = c0; c < c1; ++c) {
    const int4 ch = chunks[c];
    if (ch.x != cur) {
      if (cur >= 0) {
        __syncthreads();
        p2g_flush<DIM, T, Sink>(tile, TN, g, org, sink);
      }
      __syncthreads();
      for (int t = threadIdx.x; t < 4 * TN; t += blockDim.x) tile[t] = T(0);
      cur = ch.x;
      int bc[DIM];
      block_coords<DIM>(g, cur, bc);
#pragma unroll
      for (int d = 0; d < DIM; ++d) org[d] = bc[d] * g.bs;
      __syncthreads();
    }
    for (int l = threadIdx.x; l < ch.z; l += blockDim.x)
      p2g_particle<DIM, T>(kp, g, P, perm[ch.y + l], org, tacc, status, fallbacks);
  }
  if (cur >= 0) {
    __syncthreads();
    p2g_flush<DIM, T, Sink>(tile, TN, g, org, sink);
  }
}

// ----------------------------------------------------------------------------------------------
// Grid node rule (three_d/grid_op.py:22-47, two_d/grid_op.py:13-24).  vel holds momentum on
// entry (or, for the per-phase API, whatever the caller's grid held) and velocity on exit.
template <int DIM, typename T>
__device__ __forceinline__ void grid_node(const KParams<T>& kp, const int I[DIM], T vel[3], T m) {
  if constexpr (DIM == 3) {
    if (m > T(0)) {
      vel[0] = vel[0] / m;
      vel[1] = vel[1] / m;
      vel[2] = vel[2] / m;
      vel[1] += kp.dt * kp.gravity;
#pragma unroll
      for (int d = 0; d < 3; ++d) vel[d] = ffclamp(vel[d], -kp.v_allowed, kp.v_allowed);
    }
    if (kp.wall_mode == FFMPM_WALLS_REFERENCE) {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (I[d] < 1 || I[d] >= kp.res - 1) vel[d] = T(0);
    } else {
      bool near = false;
#pragma unroll
      for (int d = 0; d < 3; ++d) near = near || I[d] < 3 || I[d] > kp.res - 3;
      if (near) vel[0] = vel[1] = vel[2] = T(0);
    }
  } else {
    if (m > T(0)) {
      vel[0] = vel[0] / m;
      vel[1] = vel[1] / m;
      vel[1] += kp.dt * kp.gravity;
      if (kp.wall_mode == FFMPM_WALLS_REFERENCE) {
        // x = I0 / res, y = I1 / res: x < 0.05, x > 0.95 or y > 0.95 stop the node; y < 0.05 keeps
        // only an upward velocity
        if (I[0] < kp.wall_lo || I[0] > kp.wall_hi || I[1] > kp.wall_hi) vel[0] = vel[1] = T(0);
        if (I[1] < kp.wall_lo) vel[1] = vel[1] > T(0) ? vel[1] : T(0);
      } else {
        bool near = I[0] < 3 || I[0] > kp.res - 3 || I[1] < 3 || I[1] > kp.res - 3;
        if (near) vel[0] = vel[1] = T(0);
      }
    }
    vel[2] = T(0);
  }
  // planar colliders (sticky), after the walls
  for (int q = 0; q < kp.n_planes; ++q)
    if (behind_plane<DIM, T>(kp, I, q)) vel[0] = vel[1] = vel[2] = T(0);
}

template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_grid_update(KParams<T> kp, Geom<DIM> g,
                                                          const uint32_t* __restrict__ touched,
                                                          const WsHeader* __restrict__ hdr, Node4<T>* __restrict__ A,
                                                          Node4<T>* __restrict__ B) {
  const uint32_t nt = hdr->n_touched;
  const int per_block = DIM == 3 ? g.bs * g.bs * g.bs : g.bs * g.bs;
  for (uint32_t tb = blockIdx.x; tb < nt; tb += gridDim.x) {
    int bc[DIM];
    block_coords<DIM>(g, (int)touched[tb], bc);
    for (int t = threadIdx.x; t < per_block; t += blockDim.x) {
      int I[DIM];
      if constexpr (DIM == 3) {
        I[0] = bc[0] * g.bs + (t >> (2 * g.bs_shift));
        I[1] = bc[1] * g.bs + ((t >> g.bs_shift) & (g.bs - 1));
        I[2] = bc[2] * g.bs + (t & (g.bs - 1));
      } else {
        I[0] = bc[0] * g.bs + (t >> g.bs_shift);
        I[1] = bc[1] * g.bs + (t & (g.bs - 1));
      }
      bool in = true;
#pragma unroll
      for (int d = 0; d < DIM; ++d) in = in && I[d] < g.R;
      if (!in) continue;
      const int64_t node = node_index<DIM>(g.R, I);
      const Node4<T> a = A[node];
      T vel[3] = {a.x, a.y, a.z};
      grid_node<DIM, T>(kp, I, vel, a.w);
      B[node] = Node4<T>{vel[0], vel[1], vel[2], a.w};
      // re-zero A for the next P2G (a node that received nothing is zero already)
      if (a.x != T(0) || a.y != T(0) || a.z != T(0) || a.w != T(0)) A[node] = Node4<T>{T(0), T(0), T(0), T(0)};
    }
  }
}

// Grid update of the deterministic mode: node momentum/mass = staged tiles of the blocks whose
// tiles cover the node, summed in a fixed order; then the grid rule (grid_node).
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_grid_update_det(KParams<T> kp, Geom<DIM> g,
                                                              const uint32_t* __restrict__ touched,
                                                              const uint32_t* __restrict__ block_cnt,
                                                              const WsHeader* __restrict__ hdr,
                                                              const Node4<T>* __restrict__ stage,
                                                              Node4<T>* __restrict__ B, T* user_gv, T* user_gm) {
  const uint32_t nt = hdr->n_touched;
  const int per_block = DIM == 3 ? g.bs * g.bs * g.bs : g.bs * g.bs;
  const int TN = tile_nodes<DIM>(g);
  const int T1 = g.tile;
  for (uint32_t tb = blockIdx.x; tb < nt; tb += gridDim.x) {
    int bc[DIM];
    block_coords<DIM>(g, (int)touched[tb], bc);
    for (int t = threadIdx.x; t < per_block; t += blockDim.x) {
      int loc[DIM], I[DIM];
      if constexpr (DIM == 3) {
        loc[0] = t >> (2 * g.bs_shift);
        loc[1] = (t >> g.bs_shift) & (g.bs - 1);
        loc[2] = t & (g.bs - 1);
      } else {
        loc[0] = t >> g.bs_shift;
        loc[1] = t & (g.bs - 1);
      }
      bool in = true;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        I[d] = bc[d] * g.bs + loc[d];
        in = in && I[d] < g.R;
      }
      if (!in) continue;
      T a = T(0), b = T(0), c = T(0), m = T(0);
#pragma unroll
      for (int o = 0; o < (1 << DIM); ++o) {
        int src[DIM], tl[DIM];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const int od = (o >> (DIM - 1 - d)) & 1;
          src[d] = bc[d] - od;
          tl[d] = loc[d] + od * g.bs;
          ok = ok && src[d] >= 0 && tl[d] < T1;
        }
        if (!ok) continue;
        int sb = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) sb = sb * g.nb + src[d];
        if (block_cnt[sb] == 0) continue;
        const int ti = DIM == 3 ? (tl[0] * T1 + tl[1]) * T1 + tl[2] : tl[0] * T1 + tl[1];
        const Node4<T> v = stage[(size_t)sb * TN + ti];
        a += v.x;
        b += v.y;
        c += v.z;
        m += v.w;
      }
      const int64_t node = node_index<DIM>(g.R, I);
      if (user_gv) {
        // per-phase API: add the deterministic node sums into the caller's grid
        user_gv[node * DIM + 0] += a;
        user_gv[node * DIM + 1] += b;
        if constexpr (DIM == 3) user_gv[node * DIM + 2] += c;
        user_gm[node] += m;
      } else {
        T vel[3] = {a, b, c};
        grid_node<DIM, T>(kp, I, vel, m);
        B[node] = Node4<T>{vel[0], vel[1], vel[2], m};
      }
    }
  }
}

// Dense per-phase grid_op on the caller's arrays (every node, as the reference sweeps).
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_grid_op_dense(KParams<T> kp, int R, T* __restrict__ gv,
                                                            const T* __restrict__ gm) {
  const int64_t nn = DIM == 3 ? (int64_t)R * R * R : (int64_t)R * R;
  for (int64_t node = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; node < nn;
       node += (int64_t)gridDim.x * blockDim.x) {
    int I[DIM];
    if constexpr (DIM == 3) {
      I[0] = (int)(node / ((int64_t)R * R));
      I[1] = (int)((node / R) % R);
      I[2] = (int)(node % R);
    } else {
      I[0] = (int)(node / R);
      I[1] = (int)(node % R);
    }
    T vel[3] = {gv[node * DIM + 0], gv[node * DIM + 1], DIM == 3 ? gv[node * DIM + DIM - 1] : T(0)};
    grid_node<DIM, T>(kp, I, vel, gm[node]);
#pragma unroll
    for (int d = 0; d < DIM; ++d) gv[node * DIM + d] = vel[d];
  }
}

// ----------------------------------------------------------------------------------------------
// G2P.  The tile of grid velocities for the chunk's block ((bs+2)^DIM nodes of Node4) is staged in
// shared memory, either by one TMA bulk-tensor copy from the workspace grid (kTma) or by plain
// loads from the caller's grid (per-phase API).
struct G2PExtra {
  const int32_t* ids_in;
  int32_t* ids_out;
  uint32_t* keys_next;    // sorted mode: key of the updated position (next substep's sort input)
  uint32_t* block_count;  // sorted mode: histogram for the next substep
  int cell_bits;
  // plans kept over several substeps: the global node grid for particles whose stencil left their
  // chunk block's tile, and the flag raised when a particle's next stencil leaves the blocks within
  // +-1 of that block (the next substep must then re-sort)
  const void* grid_global;
  uint32_t* far_flag;
};

// The state G2P reads of one particle (loaded ahead of the arithmetic so that the loads of
// several particles are in flight together).
template <int DIM, typename T>
struct G2PIn {
  T x[DIM];
  T F[DIM * DIM];
  T jp;
};

template <int DIM, typename T>
__device__ __forceinline__ void g2p_load(const PView<T>& Pin, uint32_t p, bool need_jp, G2PIn<DIM, T>& in) {
#pragma unroll
  for (int d = 0; d < DIM; ++d) in.x[d] = Pin.x[Pin.at(p, d, DIM)];
#pragma unroll
  for (int i = 0; i < DIM * DIM; ++i) in.F[i] = Pin.F[Pin.at(p, i, DIM * DIM)];
  in.jp = need_jp ? Pin.Jp[p] : T(1);
}

// G2P of one particle p, written to slot q of Pout.  With kNext (fused G2P + P2G) the updated
// particle also goes to *next (the input of the next substep's P2G), and v and C are not stored:
// the next substep's G2P rebuilds them from the grid.  Returns false for a particle outside the grid
// or off its tile without a global grid (nothing written).
template <int DIM, typename T, bool kNext = false>
__device__ __forceinline__ bool g2p_particle(const KParams<T>& kp, const Geom<DIM>& g, const PView<T>& Pin,
                                             const PView<T>& Pout, uint32_t p, uint32_t q, const int org[DIM],
                                             const Node4<T>* tile, int32_t* status, bool sorted,
                                             const G2PExtra& ex, const G2PIn<DIM, T>& in,
                                             P2GIn<DIM, T>* next = nullptr) {
  constexpr int DD = DIM * DIM;
  T xp[DIM], fx[DIM], w[3][DIM];
  int lb[DIM], base[DIM];
  bool ok = true, in_tile = true;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    xp[d] = in.x[d];
    ok = ok && base_of(xp[d], kp.inv_dx, kp.res, base[d], fx[d]);
    lb[d] = base[d] - org[d];
    in_tile = in_tile && lb[d] >= 0 && lb[d] + 2 < g.tile;
    T ww[3];
    bspline(fx[d], ww);
    w[0][d] = ww[0];
    w[1][d] = ww[1];
    w[2][d] = ww[2];
  }
  if (!ok || (!in_tile && !ex.grid_global)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return false;
  }
  // stencil source: the staged tile, or (a particle that left its chunk block's tile between
  // re-sorts) the global node grid.  Node (i, j[, k]) of the stencil is src[i s0 + j s1 (+ k s2)]:
  // 3D strides (W^2, W, 1), 2D strides (W, 1), W the row width of the source.
  const int W = in_tile ? g.tile : g.R;
  const int s0 = DIM == 3 ? W * W : W;
  const int s1 = DIM == 3 ? W : 1;
  const int s2 = 1;
  const Node4<T>* src = in_tile ? tile + (DIM == 3 ? (lb[0] * W + lb[1]) * W + lb[2] : lb[0] * W + lb[1])
                                : static_cast<const Node4<T>*>(ex.grid_global) + node_index<DIM>(g.R, base);
  // The gather runs on node velocities relative to the stencil's centre node u: v = u + sum w (v_i - u)
  // and C = 4 inv_dx sum w (v_i - u) (x) (i - fx), equal in exact arithmetic to the reference's
  // sums (the weights sum to 1 and sum w (i - fx) = 0).  A body's bulk velocity then cancels exactly
  // instead of leaving rounding residue of size |u| eps inv_dx in C, which in float would drift F
  // by ~1e-5 over a thousand substeps of a falling or colliding body.
  T v[DIM], Cn[DD];
#pragma unroll
  for (int d = 0; d < DIM; ++d) v[d] = T(0);
#pragma unroll
  for (int i = 0; i < DD; ++i) Cn[i] = T(0);
  T u[DIM];
  if constexpr (DIM == 3) {
    const Node4<T> c = src[s0 + s1 + s2];
    u[0] = c.x;
    u[1] = c.y;
    u[2] = c.z;
    // The weights are separable, w = wx_i wy_j wz_k, so the 27-node sums are taken one axis at a
    // time: along k for each (i, j) (the sums s0 = sum_k wz_k g and s1 = sum_k wz_k (k - fz) g),
    // then along j, then along i; 360 multiply-adds where the node-by-node form takes 513.
    T wzd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) wzd[k] = w[k][2] * (T(k) - fx[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T t0[3] = {T(0), T(0), T(0)}, t1[3] = {T(0), T(0), T(0)}, t2[3] = {T(0), T(0), T(0)};
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T sa[3] = {T(0), T(0), T(0)}, sb[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const Node4<T> gvn = src[i * s0 + j * s1 + k * s2];
          const T g0 = gvn.x - u[0], g1 = gvn.y - u[1], g2 = gvn.z - u[2];
          sa[0] += w[k][2] * g0;
          sa[1] += w[k][2] * g1;
          sa[2] += w[k][2] * g2;
          sb[0] += wzd[k] * g0;
          sb[1] += wzd[k] * g1;
          sb[2] += wzd[k] * g2;
        }
        const T wy = w[j][1], wyd = w[j][1] * (T(j) - fx[1]);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          t0[r] += wy * sa[r];
          t1[r] += wyd * sa[r];
          t2[r] += wy * sb[r];
        }
      }
      const T wx = w[i][0], wxd = w[i][0] * (T(i) - fx[0]);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        v[r] += wx * t0[r];
        Cn[r * 3 + 0] += wxd * t0[r];
        Cn[r * 3 + 1] += wx * t1[r];
        Cn[r * 3 + 2] += wx * t2[r];
      }
    }
  } else {
    const Node4<T> c = src[s0 + s1];
    u[0] = c.x;
    u[1] = c.y;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T d0 = T(i) - fx[0];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T d1 = T(j) - fx[1];
        const T weight = w[i][0] * w[j][1];
        const Node4<T> gvn = src[i * s0 + j * s1];
        const T wv0 = weight * (gvn.x - u[0]), wv1 = weight * (gvn.y - u[1]);
        v[0] += wv0;
        v[1] += wv1;
        Cn[0] += wv0 * d0; Cn[1] += wv0 * d1;
        Cn[2] += wv1 * d0; Cn[3] += wv1 * d1;
      }
    }
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) v[d] += u[d];
  const T c4 = T(4) * kp.inv_dx;
#pragma unroll
  for (int i = 0; i < DD; ++i) Cn[i] *= c4;
  T F[DD], Fn[DD];
#pragma unroll
  for (int i = 0; i < DD; ++i) F[i] = in.F[i];
  // F <- (I + dt C) F   (g2p.py:46), evaluated as F + dt (C F): the increment is formed on its own
  // and rounded once against F, where 1 + dt C would round dt C to the spacing of the numbers near
  // 1 (in float that keeps only ~3 digits of a 1e-4 increment)
#pragma unroll
  for (int r = 0; r < DIM; ++r)
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < DIM; ++k) acc += Cn[r * DIM + k] * F[k * DIM + c];
      Fn[r * DIM + c] = F[r * DIM + c] + kp.dt * acc;
    }
  const bool write_jp = (DIM == 2) || sorted || kp.model == FFMPM_MODEL_SNOW;
  T jp_new = in.jp;
  if constexpr (DIM == 2) {
    // two_d/g2p.py:37-46: SVD, clamp (snow only), rebuild, Jp update.  Without the clamp the
    // rebuild returns F itself (up to the sign convention of the SVD), so only snow rebuilds.
    const T oldJ = Fn[0] * Fn[3] - Fn[1] * Fn[2];
    if (kp.model == FFMPM_MODEL_SNOW) {
      T U[4], s[2], V[4];
      svd2<T>(Fn, U, s, V);
      s[0] = ffclamp(s[0], T(1.0 - 2.5e-2), T(1.0 + 7.5e-3));
      s[1] = ffclamp(s[1], T(1.0 - 2.5e-2), T(1.0 + 7.5e-3));
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) Fn[i * 2 + j] = U[i * 2 + 0] * s[0] * V[j * 2 + 0] + U[i * 2 + 1] * s[1] * V[j * 2 + 1];
    }
    const T det = (Fn[0] * Fn[3] - Fn[1] * Fn[2]) + T(1e-10);
    jp_new = ffclamp(jp_new * oldJ / det, T(0.6), T(20.0));
  } else {
    if (kp.model == FFMPM_MODEL_SNOW) {
      // three_d/g2p.py:48-58: clamp the singular values, rebuild F, update Jp.  The rebuild is
      // U diag(s) V^T of F = U diag(s) V^T; the reference writes U @ diag(s) @ Vh.T with numpy's Vh,
      // which depends on LAPACK's singular-vector signs and does not return F for unclamped s.
      T U[9], sv[3], V[9];
      svd3<T>(Fn, U, sv, V);
      const T oldJ = det3(Fn);
#pragma unroll
      for (int d = 0; d < 3; ++d) sv[d] = ffclamp(sv[d], T(1.0 - 2.5e-2), T(1.0 + 7.5e-3));
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          Fn[i * 3 + j] = U[i * 3 + 0] * sv[0] * V[j * 3 + 0] + U[i * 3 + 1] * sv[1] * V[j * 3 + 1] +
                          U[i * 3 + 2] * sv[2] * V[j * 3 + 2];
      const T det = det3(Fn) + T(1e-10);
      jp_new = ffclamp(jp_new * oldJ / det, T(0.6), T(20.0));
    }
  }
  T xn[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) xn[d] = xp[d] + kp.dt * v[d];
  // a non-finite v reaches x and a non-finite C reaches F (C F has a NaN in that row even where F is
  // zero), so x and F cover the whole updated state
  if (nonfinite_probe(xn, DIM) + nonfinite_probe(Fn, DD) != T(0)) raise_status(status, FFMPM_STATUS_NONFINITE);
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    Pout.x[Pout.at(q, d, DIM)] = xn[d];
    if constexpr (!kNext) Pout.v[Pout.at(q, d, DIM)] = v[d];
  }
#pragma unroll
  for (int i = 0; i < DD; ++i) {
    if constexpr (!kNext) Pout.C[Pout.at(q, i, DD)] = Cn[i];
    Pout.F[Pout.at(q, i, DD)] = Fn[i];
  }
  if (write_jp) Pout.Jp[q] = jp_new;
  if constexpr (kNext) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      next->x[d] = xn[d];
      next->v[d] = v[d];
    }
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      next->F[i] = Fn[i];
      next->C[i] = Cn[i];
    }
    next->m = Pin.mass ? Pin.mass[p] : kp.mass;
    next->mu0 = Pin.mu0 ? Pin.mu0[p] : kp.mu0;
    next->lam0 = Pin.lam0 ? Pin.lam0[p] : kp.lam0;
    next->jp = kp.model == FFMPM_MODEL_SNOW ? jp_new : T(1);
  }
  if (sorted) {
    if constexpr (kNext) {
      if (Pin.mass) Pout.mass[q] = next->m;
      if (Pin.mu0) Pout.mu0[q] = next->mu0;
      if (Pin.lam0) Pout.lam0[q] = next->lam0;
    } else {
      if (Pin.mass) Pout.mass[q] = Pin.mass[p];
      if (Pin.mu0) Pout.mu0[q] = Pin.mu0[p];
      if (Pin.lam0) Pout.lam0[q] = Pin.lam0[p];
    }
    if (ex.ids_in) ex.ids_out[q] = ex.ids_in[p];
    if (ex.keys_next) {
      // key of the updated position: the next substep's sort input (fused to avoid re-reading x)
      uint32_t key, blk;
      const bool valid = particle_key<DIM, T>(xn, kp, g, ex.cell_bits, key, blk);
      if (!valid) raise_status(status, FFMPM_STATUS_OOB);
      ex.keys_next[q] = key;
      warp_count(ex.block_count, blk, valid);
      if (ex.far_flag && valid) {
        bool far = false;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          int bn;
          T fn;
          base_of(xn[d], kp.inv_dx, kp.res, bn, fn);
          const int l = bn - org[d];
          far = far || l < -g.bs || l > 2 * g.bs - 3;
        }
        if (far) *ex.far_flag = 1u;
      }
    }
  }
  return true;
}

template <int DIM, typename T, bool kTma, bool kSorted>
__global__ void __launch_bounds__(kThreads) k_g2p(KParams<T> kp, Geom<DIM> g, PView<T> Pin, PView<T> Pout,
                                                  const uint32_t* __restrict__ perm, const int4* __restrict__ chunks,
                                                  const WsHeader* __restrict__ hdr, const __grid_constant__ CUtensorMap tmap,
                                                  const T* __restrict__ user_gv, G2PExtra ex, int32_t* status,
                                                  const uint32_t* __restrict__ sort_flag) {
  if (sort_flag && *sort_flag == 0u) perm = nullptr;  // plan kept from an earlier substep: identity order
  if (perm && wait_gave_up(status)) return;
  // Dynamic shared memory: [pad to 128 B][tile: TN Node4][mbarrier].  The TMA destination must
  // be 128-byte aligned, so the tile start is rounded up explicitly.
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int TN = tile_nodes<DIM>(g);
  const uint32_t pad = (128u - (smem_u32(smem_raw) & 127u)) & 127u;
  Node4<T>* tile = reinterpret_cast<Node4<T>*>(smem_raw + pad);
  uint64_t& bar = *reinterpret_cast<uint64_t*>(smem_raw + pad + TN * sizeof(Node4<T>));
  const uint32_t nch = hdr->n_chunks;
  const uint32_t per = (nch + gridDim.x - 1) / gridDim.x;
  const uint32_t c0 = blockIdx.x * per;
  const uint32_t c1 = min(nch, c0 + per);
  if constexpr (kTma) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      fence_barrier_init();
    }
    __syncthreads();
  }
  uint32_t phase = 0;
  int cur = -1;
  int org[DIM];
  bool timed_out = false;
  for (uint32_t c = c0; c < c1; ++c) {
    const int4 ch = chunks[c];
    if (ch.x != cur) {
      __syncthreads();  // every thread is done with the previous tile
      cur = ch.x;
      int bc[DIM];
      block_coords<DIM>(g, cur, bc);
#pragma unroll
      for (int d = 0; d < DIM; ++d) org[d] = bc[d] * g.bs;
      if constexpr (kTma) {
        if (threadIdx.x == 0) {
          const uint32_t bytes = (uint32_t)(TN * sizeof(Node4<T>));
          mbar_arrive_expect_tx(&bar, bytes);
          if constexpr (DIM == 3)
            tma_load_4d(tile, &tmap, &bar, 0, org[2], org[1], org[0]);
          else
            tma_load_3d(tile, &tmap, &bar, 0, org[1], org[0]);
        }
        if (!mbar_wait(&bar, phase)) {
          timed_out = true;
        }
        if (__syncthreads_or(timed_out)) {
          // the tile copy may still be in flight: wait for it once more (bounded) so that it does
          // not land in shared memory after this CTA has left
          if (threadIdx.x == 0) {
            raise_status(status, FFMPM_STATUS_TIMEOUT);
            mbar_wait(&bar, phase);
          }
          __syncthreads();
          return;
        }
        phase ^= 1u;
      } else {
        const int T1 = g.tile;
        for (int t = threadIdx.x; t < TN; t += blockDim.x) {
          int I[DIM];
          if constexpr (DIM == 3) {
            I[0] = org[0] + t / (T1 * T1);
            I[1] = org[1] + (t / T1) % T1;
            I[2] = org[2] + t % T1;
          } else {
            I[0] = org[0] + t / T1;
            I[1] = org[1] + t % T1;
          }
          bool in = true;
#pragma unroll
          for (int d = 0; d < DIM; ++d) in = in && I[d] < g.R;
          Node4<T> nv{T(0), T(0), T(0), T(0)};
          if (in) {
            const int64_t node = node_index<DIM>(g.R, I);
            nv.x = user_gv[node * DIM + 0];
            nv.y = user_gv[node * DIM + 1];
            if constexpr (DIM == 3) nv.z = user_gv[node * DIM + 2];
          }
          tile[t] = nv;
        }
        __syncthreads();
      }
    }
    const bool need_jp = (DIM == 2) || kSorted || kp.model == FFMPM_MODEL_SNOW;
    // two particles per thread per iteration: both particles' loads are issued before either
    // one's arithmetic
    for (int l = threadIdx.x; l < ch.z; l += 2 * blockDim.x) {
      const int l2 = l + blockDim.x;
      const bool two = l2 < ch.z;
      const uint32_t s1 = ch.y + l, s2 = ch.y + (two ? l2 : l);
      const uint32_t p1 = perm ? perm[s1] : s1, p2 = perm ? perm[s2] : s2;
      G2PIn<DIM, T> in1, in2;
      g2p_load<DIM, T>(Pin, p1, need_jp, in1);
      g2p_load<DIM, T>(Pin, p2, need_jp, in2);
      g2p_particle<DIM, T>(kp, g, Pin, Pout, p1, kSorted ? s1 : p1, org, tile, status, kSorted, ex, in1);
      if (two) g2p_particle<DIM, T>(kp, g, Pin, Pout, p2, kSorted ? s2 : p2, org, tile, status, kSorted, ex, in2);
    }
  }
}

// ----------------------------------------------------------------------------------------------
// Substep on particle arrays that live in host memory (ffmpm_substep_host).  The arrays arrive in
// chunks of particles; each chunk is scattered as soon as it has landed, in the caller's particle
// order, with one vector atomic per node (a block sort needs every particle, which would hold the
// scatter back until the last copy).  After a dense grid update each chunk is gathered, again in
// the caller's order, from the global velocity grid, and copied back while the next chunk is
// gathered.  Same arithmetic per particle as the sorted kernels (p2g_particle, grid_node,
// g2p_particle); only the order of the node sums differs.

// P2G of particles [p0, p1): three_d/p2g.py:14-80 / two_d/p2g.py:11-76, straight to the grid.
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_p2g_range(KParams<T> kp, Geom<DIM> g, PView<T> P, uint32_t p0,
                                                        uint32_t p1, InternalSink<T> sink, int32_t* status,
                                                        uint32_t* fallbacks) {
  Geom<DIM> gd = g;
  gd.tile = g.R + 2;  // origin 0 and a "tile" of the whole grid: every in-grid stencil is accepted
  DirectAdder<DIM, T, InternalSink<T>> acc;
  acc.sink = sink;
  acc.R = g.R;
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc.org[d] = 0;
  for (uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x; p < p1; p += gridDim.x * blockDim.x)
    p2g_particle<DIM, T>(kp, gd, P, p, acc.org, acc, status, fallbacks);
}

// Grid update of every node (three_d/grid_op.py:5-47 / two_d/grid_op.py:5-24): momentum of A ->
// velocity in B, A re-zeroed.  Nodes that received nothing are skipped (their B is never read).
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_grid_update_dense(KParams<T> kp, Geom<DIM> g, Node4<T>* __restrict__ A,
                                                                Node4<T>* __restrict__ B) {
  const int R = g.R;
  const int64_t nn = DIM == 3 ? (int64_t)R * R * R : (int64_t)R * R;
  for (int64_t node = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; node < nn;
       node += (int64_t)gridDim.x * blockDim.x) {
    const Node4<T> a = A[node];
    if (a.x == T(0) && a.y == T(0) && a.z == T(0) && a.w == T(0)) continue;
    int I[DIM];
    if constexpr (DIM == 3) {
      I[0] = (int)(node / ((int64_t)R * R));
      I[1] = (int)((node / R) % R);
      I[2] = (int)(node % R);
    } else {
      I[0] = (int)(node / R);
      I[1] = (int)(node % R);
    }
    T vel[3] = {a.x, a.y, a.z};
    grid_node<DIM, T>(kp, I, vel, a.w);
    B[node] = Node4<T>{vel[0], vel[1], vel[2], a.w};
    A[node] = Node4<T>{T(0), T(0), T(0), T(0)};
  }
}

// G2P of particles [p0, p1) in place (three_d/g2p.py:9-59 / two_d/g2p.py:5-47), every stencil
// gathered from the global velocity grid B.
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_g2p_range(KParams<T> kp, Geom<DIM> g, PView<T> P, uint32_t p0,
                                                        uint32_t p1, const Node4<T>* __restrict__ B, int32_t* status) {
  G2PExtra ex{};
  ex.grid_global = B;
  int org[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) org[d] = -(1 << 24);  // no staged tile: every stencil is off-tile
  const bool need_jp = (DIM == 2) || kp.model == FFMPM_MODEL_SNOW;
  for (uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x; p < p1; p += gridDim.x * blockDim.x) {
    G2PIn<DIM, T> in;
    g2p_load<DIM, T>(P, p, need_jp, in);
    g2p_particle<DIM, T>(kp, g, P, P, p, p, org, nullptr, status, false, ex, in);
  }
}

// ----------------------------------------------------------------------------------------------
// Fused G2P + P2G: substep k's G2P and substep k+1's P2G in one pass over the particles.  The
// updated particle (x, v, C, F) goes straight from the gather into the next substep's record, so
// v and C never travel through memory between the two, and x and F are read once per substep.
// Both halves use the chunk's block: the G2P tile of grid velocities (staged by TMA from the
// workspace's velocity grid) and the P2G tile of momentum/mass (flushed into the workspace's
// accumulation grid), and the cell-run phases of k_p2g_cells.  The block plan was made from the
// positions of substep k, so a particle's new stencil may leave its block's tile (it takes the
// direct global adds) or, moving fast, the blocks the plan touches: it then adds the blocks its
// stencil covers to the touched list itself, so that the grid update visits every node that
// received mass.

// Add the blocks covered by the stencil at `base` to the touched list (each block once: `tmark`
// holds 1 for every listed block).
template <int DIM>
__device__ __forceinline__ void mark_touched(const Geom<DIM>& g, const int base[DIM], uint32_t* tmark,
                                             uint32_t* touched, uint32_t* n_touched) {
  int lo[DIM], ext[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    lo[d] = base[d] >> g.bs_shift;
    ext[d] = min((base[d] + 2) >> g.bs_shift, g.nb - 1) - lo[d];  // 0 or 1
  }
  for (int o = 0; o < (1 << DIM); ++o) {
    int id = 0;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int od = (o >> (DIM - 1 - d)) & 1;
      ok = ok && od <= ext[d];
      id = id * g.nb + lo[d] + od;
    }
    if (ok && atomicCAS(&tmark[id], 0u, 1u) == 0u) touched[atomicAdd(n_touched, 1u)] = (uint32_t)id;
  }
}

// Dynamic shared memory of k_g2p2g: [pad to 128 B][G2P tile: TN Node4][mbarrier: 128 B]
// [P2G tile: 4 TN reals][cell-run arrays], every region starting on 128 bytes.
__host__ __device__ constexpr size_t align128(size_t v) { return (v + 127) & ~size_t(127); }

template <int DIM, typename T>
__host__ __device__ constexpr size_t g2p2g_smem_bytes(int TN, int bs) {
  return 128 + align128(size_t(TN) * sizeof(Node4<T>)) + 128 + align128(size_t(4) * TN * sizeof(T)) +
         cell_run_smem_bytes<DIM, T>(bs);
}

template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1) k_g2p2g(
    KParams<T> kp, Geom<DIM> g, PView<T> Pin, PView<T> Pout, const uint32_t* __restrict__ perm,
    const int4* __restrict__ chunks, WsHeader* hdr, const __grid_constant__ CUtensorMap tmap, G2PExtra ex,
    InternalSink<T> sink, uint32_t* __restrict__ tmark, uint32_t* __restrict__ touched, int32_t* status,
    uint32_t* fallbacks, const uint32_t* __restrict__ sort_flag) {
  if (sort_flag && *sort_flag == 0u) perm = nullptr;  // plan kept from an earlier substep: identity order
  if (perm && wait_gave_up(status)) return;
  constexpr int RS = RecLayout<DIM>::kStride;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int TN = tile_nodes<DIM>(g);
  unsigned char* at = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  Node4<T>* gtile = reinterpret_cast<Node4<T>*>(at);
  at += align128(size_t(TN) * sizeof(Node4<T>));
  uint64_t& bar = *reinterpret_cast<uint64_t*>(at);
  at += 128;
  T* ptile = reinterpret_cast<T*>(at);
  at += align128(size_t(4) * TN * sizeof(T));
  __shared__ int nruns_s;
  __shared__ int warp_cnt[kThreads / 32];
  __shared__ int warp_nz[kThreads / 32];
  const CellRunSmem<T> cr = cell_run_smem<DIM, T>(at, g, &nruns_s, warp_cnt, warp_nz);
  const TileAdder<DIM, T> tacc{ptile, TN, g.tile};
  const uint32_t nch = hdr->n_chunks;
  const uint32_t per = (nch + gridDim.x - 1) / gridDim.x;
  const uint32_t c0 = blockIdx.x * per;
  const uint32_t c1 = min(nch, c0 + per);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  uint32_t phase = 0;
  int cur = -1;
  int org[DIM];
  for (uint32_t c = c0; c < c1; ++c) {
    const int4 ch = chunks[c];
    if (ch.x != cur) {
      if (cur >= 0) {
        __syncthreads();  // phase 3 of the previous chunk is done with the P2G tile
        p2g_flush<DIM, T, InternalSink<T>>(ptile, TN, g, org, sink);
      }
      __syncthreads();  // every thread is done with both tiles
      cur = ch.x;
      int bc[DIM];
      block_coords<DIM>(g, cur, bc);
#pragma unroll
      for (int d = 0; d < DIM; ++d) org[d] = bc[d] * g.bs;
      if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, (uint32_t)(TN * sizeof(Node4<T>)));
        if constexpr (DIM == 3)
          tma_load_4d(gtile, &tmap, &bar, 0, org[2], org[1], org[0]);
        else
          tma_load_3d(gtile, &tmap, &bar, 0, org[1], org[0]);
      }
      for (int t = threadIdx.x; t < 4 * TN; t += blockDim.x) ptile[t] = T(0);
      const bool timed_out = !mbar_wait(&bar, phase);
      if (__syncthreads_or(timed_out)) {
        // the tile copy may still be in flight: wait for it once more (bounded) so that it does not
        // land in shared memory after this CTA has left
        if (threadIdx.x == 0) {
          raise_status(status, FFMPM_STATUS_TIMEOUT);
          mbar_wait(&bar, phase);
        }
        __syncthreads();
        return;
      }
      phase ^= 1u;
    }
    // phase 1: G2P of substep k, then the record of substep k+1, one particle per thread
    for (int l = threadIdx.x; l < ch.z; l += blockDim.x) {
      const uint32_t s = ch.y + l;
      const uint32_t p = perm ? perm[s] : s;
      G2PIn<DIM, T> in;
      g2p_load<DIM, T>(Pin, p, true, in);
      P2GIn<DIM, T> nx;
      T rec[RS];
      int cell = -1, base[DIM];
      int kind = kRecOut;
      if (g2p_particle<DIM, T, true>(kp, g, Pin, Pout, p, s, org, gtile, status, true, ex, in, &nx)) {
        kind = p2g_record<DIM, T>(kp, g, nx, org, rec, cell, status, fallbacks, base);
        if (kind == kRecStray) {
          // outside the blocks within +-1 of the chunk's block (which the plan always touches)
          bool far = false;
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            const int lb = base[d] - org[d];
            far = far || lb < -g.bs || lb > 2 * g.bs - 3;
          }
          if (far) mark_touched<DIM>(g, base, tmark, touched, &hdr->n_touched);
        }
      }
      p2g_store_record<DIM, T>(cr, l, rec, kind, cell, base);
    }
    __syncthreads();
    for (int l = threadIdx.x; l < ch.z; l += blockDim.x)
      if (cr.cells[l] == -2) p2g_scatter_record<DIM, T, InternalSink<T>>(cr.recs + (size_t)l * RS, g.R, sink);
    p2g_cell_runs<DIM, T>(cr, g, ch.z, tacc);
    __syncthreads();  // records and runs are rewritten by the next chunk
  }
  if (cur >= 0) {
    __syncthreads();
    p2g_flush<DIM, T, InternalSink<T>>(ptile, TN, g, org, sink);
  }
}

// ----------------------------------------------------------------------------------------------
// three_d/grid_op.py:50-67 check_collision_points on a caller's dense grid velocity
// [(res+1)^DIM][DIM]: every node behind one of the params' planes gets velocity zero.
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_collision_points(KParams<T> kp, T* __restrict__ gv, int64_t nnodes) {
  const int R = kp.res + 1;
  for (int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; node < nnodes;
       node += (int64_t)gridDim.x * blockDim.x) {
    int I[DIM];
    if constexpr (DIM == 3) {
      I[0] = (int)(node / ((int64_t)R * R));
      I[1] = (int)((node / R) % R);
      I[2] = (int)(node % R);
    } else {
      I[0] = (int)(node / R);
      I[1] = (int)(node % R);
    }
    bool hit = false;
    for (int q = 0; q < kp.n_planes; ++q) hit = hit || behind_plane<DIM, T>(kp, I, q);
    if (hit) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) gv[node * DIM + d] = T(0);
    }
  }
}

// ----------------------------------------------------------------------------------------------
static __global__ void k_diag_init(double* out) {
  if (threadIdx.x < 8) out[threadIdx.x] = threadIdx.x < 7 ? 0.0 : 1e300;
}

// Float64 diagnostics: [KE, elastic energy, gravitational energy, px, py, pz, mass, min det F].
template <int DIM, typename T>
__global__ void __launch_bounds__(kThreads) k_diag(KParams<T> kp, PView<T> P, uint32_t n, double* out) {
  constexpr int DD = DIM * DIM;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  double mindet = 1e300;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const double m = P.mass ? double(P.mass[p]) : double(kp.mass);
    const double mu0 = P.mu0 ? double(P.mu0[p]) : double(kp.mu0);
    const double lam0 = P.lam0 ? double(P.lam0[p]) : double(kp.lam0);
    const double h = double(kp.hardening);
    double v2 = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const double vd = double(P.v[P.at(p, d, DIM)]);
      v2 += vd * vd;
      acc[3 + d] += m * vd;
    }
    acc[0] += 0.5 * m * v2;
    acc[2] += -double(kp.gravity) * m * double(P.x[P.at(p, 1, DIM)]);
    acc[6] += m;
    double F[DD];
#pragma unroll
    for (int i = 0; i < DD; ++i) F[i] = double(P.F[P.at(p, i, DD)]);
    double J, fr = 0;
    if constexpr (DIM == 3) {
      double R[9];
      polar3_newton<double>(F, R, 60);
      J = det3(F);
#pragma unroll
      for (int i = 0; i < 9; ++i) fr += (F[i] - R[i]) * (F[i] - R[i]);
    } else {
      double R[4];
      polar2<double>(F, R);
      J = F[0] * F[3] - F[1] * F[2];
#pragma unroll
      for (int i = 0; i < 4; ++i) fr += (F[i] - R[i]) * (F[i] - R[i]);
    }
    // fixed-corotated energy density mu|F-R|^2 + lam/2 (J-1)^2, times the particle volume
    acc[1] += double(kp.volume) * (mu0 * h * fr + 0.5 * lam0 * h * (J - 1.0) * (J - 1.0));
    mindet = J < mindet ? J : mindet;
  }
  __shared__ double red[8][kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    double vsum = acc[k];
    for (int o = 16; o > 0; o >>= 1) vsum += __shfl_down_sync(0xffffffffu, vsum, o);
    if (lane == 0) red[k][warp] = vsum;
  }
  {
    double vm = mindet;
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(0xffffffffu, vm, o);
      vm = t < vm ? t : vm;
    }
    if (lane == 0) red[7][warp] = vm;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    const int k = threadIdx.x;
    double r = k < 7 ? 0.0 : 1e300;
    for (int w = 0; w < kThreads / 32; ++w) r = k < 7 ? r + red[k][w] : (red[k][w] < r ? red[k][w] : r);
    if (k < 7) {
      atomicAdd(&out[k], r);
    } else {
      // float64 atomic min via CAS on the bit pattern
      unsigned long long* addr = reinterpret_cast<unsigned long long*>(&out[7]);
      unsigned long long old = *addr, assumed;
      do {
        assumed = old;
        if (__longlong_as_double(assumed) <= r) break;
        old = atomicCAS(addr, assumed, __double_as_longlong(r));
      } while (old != assumed);
    }
  }
}

}  // namespace ffmpm
