// Reverse mode of one 3D MLS-MPM substep (the derivative of solve_mls_mpm_3d, mls_mpm.py:40-79,
// with the "neo_hookean" fixed-corotated stress of utils.py:95-135), and of the 2D substep
// (two_d/*.py with utils.py:52-92) further below.
//
// The substep is x, v, F, C -> P2G -> grid update -> G2P -> x', v', F', C'.  Its reverse, given the
// adjoints of x', v', F', C', runs five kernels on a dense (res+1)^3 grid:
//   k_adj_p2g      recompute the substep's grid (momentum, mass) from the input state
//   k_adj_gridvel  the grid update of every node once: updated velocity (and mass) for the gathers
//   k_adj_g2p      reverse G2P: per particle, scatter the node-velocity adjoints (float64 adds per
//                  stencil node) and form dL/dx, dL/dF of the gather and of F' = (I + dt C') F
//   k_adj_grid     reverse grid update per node: division by mass, gravity, clamp and walls (the
//                  clamp and the walls pass no gradient where they clip)
//   k_adj_p2g_rev  reverse P2G: per particle, gather the node adjoints and differentiate the
//                  weights, the APIC momentum and the stress, including the polar factor R of F:
//                  for F = R S, dL/dF gains R [y]_x with (tr(S) I - S) y = axial(R^T dL/dR).
//
// The adjoints carry a large, nearly uniform part (a body's bulk motion); the stress derivative
// needs only its variation across a stencil, sum W (g_i - g) (x) dpos_i.  With float node sums,
// rounding that differs from node to node (in the momentum and in the mass it is divided by) leaves
// ~1e-7 of the bulk part in that variation, which biased float E- and nu-gradients of 2000-substep
// rollouts by ~1%.  So the grids are accumulated in float64 for float particle states too, every
// node contribution formed in float64 from float factors (a product of two floats is exact in
// double).  For float states the grids the particle kernels read back (updated velocities, node
// adjoints) are then stored as float pairs hi + lo (hi = the float nearest the double, lo = the
// float nearest the rest): a stencil node's deviation from the stencil's centre node,
// (hi - hi_c) + (lo - lo_c), is formed in float with the accuracy of the double subtraction rounded
// to float (hi - hi_c is exact when the two are within a factor two), without the float64 pipe.
// Double states keep double grids throughout.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "internal.h"
#include "mpm_kernels.cuh"

namespace ffmpm {
namespace {

constexpr int kAdjThreads = 128;

template <typename T>
struct AView {
  T *x, *v, *F, *C;
  double *mu0, *lam0;
  int64_t soa;
  __device__ __forceinline__ size_t at(uint32_t p, int c, int k) const {
    return soa ? (size_t)c * (size_t)soa + p : (size_t)p * k + c;
  }
};

// Base node, fractional offset, weights w[node][axis] and their derivatives in fx.
template <typename T>
__device__ __forceinline__ bool stencil3(const KParams<T>& kp, const T x[3], int b[3], T fx[3], T w[3][3],
                                         T dw[3][3]) {
  bool ok = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) ok = ok && base_of(x[d], kp.inv_dx, kp.res, b[d], fx[d]);
  if (!ok) return false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T ww[3];
    bspline(fx[d], ww);
    w[0][d] = ww[0];
    w[1][d] = ww[1];
    w[2][d] = ww[2];
    dw[0][d] = fx[d] - T(1.5);
    dw[1][d] = T(-2) * (fx[d] - T(1));
    dw[2][d] = fx[d] - T(0.5);
  }
  return true;
}

template <typename T>
__device__ __forceinline__ void load_state(const PView<T>& P, uint32_t p, T x[3], T v[3], T F[9], T C[9]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (x) x[d] = P.x[P.at(p, d, 3)];
    if (v) v[d] = P.v[P.at(p, d, 3)];
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    if (F) F[i] = P.F[P.at(p, i, 9)];
    if (C) C[i] = P.C[P.at(p, i, 9)];
  }
}

// A float64 node {x, y, z, w} as float pairs: hi = RN(v), lo = RN(v - hi), in the 32 bytes of a
// Node4<double>.
struct HiLo4 {
  float4 hi, lo;
};
static_assert(sizeof(HiLo4) == sizeof(Node4<double>), "same slot");

// Node format of the grids read back by the particle kernels: HiLo4 for float states, double
// otherwise.
template <typename T>
using ReadNode = std::conditional_t<sizeof(T) == 4, HiLo4, Node4<double>>;

__device__ __forceinline__ void store_node(HiLo4* g, int64_t i, double x, double y, double z, double w) {
  HiLo4 o;
  o.hi = make_float4(float(x), float(y), float(z), float(w));
  o.lo = make_float4(float(x - double(o.hi.x)), float(y - double(o.hi.y)), float(z - double(o.hi.z)),
                     float(w - double(o.hi.w)));
  g[i] = o;
}
__device__ __forceinline__ void store_node(Node4<double>* g, int64_t i, double x, double y, double z, double w) {
  g[i] = Node4<double>{x, y, z, w};
}

// Node value minus the reference node value c, per component.
__device__ __forceinline__ void node_dev(const HiLo4& a, const HiLo4& c, float o[4]) {
  o[0] = (a.hi.x - c.hi.x) + (a.lo.x - c.lo.x);
  o[1] = (a.hi.y - c.hi.y) + (a.lo.y - c.lo.y);
  o[2] = (a.hi.z - c.hi.z) + (a.lo.z - c.lo.z);
  o[3] = (a.hi.w - c.hi.w) + (a.lo.w - c.lo.w);
}
__device__ __forceinline__ void node_dev(const Node4<double>& a, const Node4<double>& c, double o[4]) {
  o[0] = a.x - c.x;
  o[1] = a.y - c.y;
  o[2] = a.z - c.z;
  o[3] = a.w - c.w;
}
__device__ __forceinline__ double node_comp(const HiLo4& a, int d) {
  const float h = d == 0 ? a.hi.x : d == 1 ? a.hi.y : a.hi.z, l = d == 0 ? a.lo.x : d == 1 ? a.lo.y : a.lo.z;
  return double(h) + double(l);
}
__device__ __forceinline__ double node_comp(const Node4<double>& a, int d) { return d == 0 ? a.x : d == 1 ? a.y : a.z; }

__device__ __forceinline__ void red_add3(Node4<double>* p, double a, double b, double c) {
  atomicAdd(&p->x, a);
  atomicAdd(&p->y, b);
  atomicAdd(&p->z, c);
}

// ---------------------------------------------------------------------------------------------
// Forward P2G of the substep into a dense grid {momentum xyz, mass} (three_d/p2g.py:14-80).
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) k_adj_p2g(KParams<T> kp, PView<T> P, uint32_t n,
                                                         Node4<double>* __restrict__ grid, int32_t* status) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  T x[3], v[3], F[9], C[9];
  load_state(P, p, x, v, F, C);
  int b[3];
  T fx[3], w[3][3], dw[3][3];
  if (!stencil3(kp, x, b, fx, w, dw)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T m, mu, lam;
  lame_of(kp, P, p, m, mu, lam);
  T A[9];
  affine_of<3, T>(kp, F, C, m, mu, lam, A, nullptr);
  const int R = kp.res + 1;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double wt = double(w[i][0]) * double(w[j][1]) * double(w[k][2]);
        const T d0 = (T(i) - fx[0]) * kp.dx, d1 = (T(j) - fx[1]) * kp.dx, d2 = (T(k) - fx[2]) * kp.dx;
        const double q0 = double(m) * double(v[0]) + double(A[0] * d0 + A[1] * d1 + A[2] * d2);
        const double q1 = double(m) * double(v[1]) + double(A[3] * d0 + A[4] * d1 + A[5] * d2);
        const double q2 = double(m) * double(v[2]) + double(A[6] * d0 + A[7] * d1 + A[8] * d2);
        const int64_t node = ((int64_t)(b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
        atomic_add4(&grid[node], wt * q0, wt * q1, wt * q2, wt * double(m));
      }
}

// ---------------------------------------------------------------------------------------------
// Forward grid update (three_d/grid_op.py:5-47) of every node: {updated velocity, mass}.
template <typename G>
__global__ void __launch_bounds__(kAdjThreads) k_adj_gridvel(KParams<double> kp, const Node4<double>* __restrict__ grid,
                                                             G* __restrict__ gvel, int64_t nnodes) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nnodes) return;
  const int R = kp.res + 1;
  const int I[3] = {(int)(idx / ((int64_t)R * R)), (int)((idx / R) % R), (int)(idx % R)};
  const Node4<double> g = grid[idx];
  double vel[3] = {g.x, g.y, g.z};
  grid_node<3, double>(kp, I, vel, g.w);
  store_node(gvel, idx, vel[0], vel[1], vel[2], g.w);
}

// ---------------------------------------------------------------------------------------------
// Reverse G2P (three_d/g2p.py:9-59).  Forward: v' = sum W vg, C' = 4 inv_dx sum W vg (x) (i - fx),
// x' = x + dt v', F' = (I + dt C') F, with vg the updated node velocity.
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) k_adj_g2p(KParams<T> kp, PView<T> P, AView<T> Ab, uint32_t n,
                                                         const ReadNode<T>* __restrict__ gvel,
                                                         Node4<double>* __restrict__ gadj, int32_t* status) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  T x[3], F[9];
  load_state<T>(P, p, x, nullptr, F, nullptr);
  int b[3];
  T fx[3], w[3][3], dw[3][3];
  if (!stencil3(kp, x, b, fx, w, dw)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T xb[3], vb[3], Fb1[9], Cb[9];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xb[d] = Ab.x[Ab.at(p, d, 3)];
    vb[d] = Ab.v[Ab.at(p, d, 3)] + kp.dt * xb[d];  // x' = x + dt v'
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    Fb1[i] = Ab.F[Ab.at(p, i, 9)];
    Cb[i] = Ab.C[Ab.at(p, i, 9)];
  }
  // C' enters F' = (I + dt C') F: dL/dC' += dt dL/dF' F^T
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      Cb[a * 3 + c] += kp.dt * (Fb1[a * 3 + 0] * F[c * 3 + 0] + Fb1[a * 3 + 1] * F[c * 3 + 1] +
                                Fb1[a * 3 + 2] * F[c * 3 + 2]);
  const T c4 = T(4) * kp.inv_dx;
  // sums over node velocities relative to the centre node's u (as the forward gather): with
  // dv_i = vg_i - u, sum dW = 0 and sum dW_d (i - fx) = e_d make the u terms of dL/dx cancel, so
  //   dL/dx_d = inv_dx (sum dW_d (vb.dv_i + c4 dv_i.Cb r_i) - c4 (Cb^T sum W dv_i)_d)
  T v1[3] = {0, 0, 0}, C1[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, xacc[3] = {0, 0, 0};
  const int R = kp.res + 1;
  const ReadNode<T> u = gvel[((int64_t)(b[0] + 1) * R + (b[1] + 1)) * R + (b[2] + 1)];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T wt = w[i][0] * w[j][1] * w[k][2];
        const T g0 = dw[i][0] * w[j][1] * w[k][2], g1 = w[i][0] * dw[j][1] * w[k][2],
                g2 = w[i][0] * w[j][1] * dw[k][2];
        const T r[3] = {T(i) - fx[0], T(j) - fx[1], T(k) - fx[2]};
        const int64_t node = ((int64_t)(b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
        T vel[4];
        node_dev(gvel[node], u, vel);
        T cr[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          v1[a] += wt * vel[a];
#pragma unroll
          for (int c = 0; c < 3; ++c) C1[a * 3 + c] += wt * vel[a] * r[c];
          cr[a] = Cb[a * 3 + 0] * r[0] + Cb[a * 3 + 1] * r[1] + Cb[a * 3 + 2] * r[2];
        }
        const T term = vb[0] * vel[0] + vb[1] * vel[1] + vb[2] * vel[2] +
                       c4 * (vel[0] * cr[0] + vel[1] * cr[1] + vel[2] * cr[2]);
        xacc[0] += g0 * term;
        xacc[1] += g1 * term;
        xacc[2] += g2 * term;
        const double wd = double(wt);
        red_add3(&gadj[node], wd * (double(vb[0]) + double(c4 * cr[0])), wd * (double(vb[1]) + double(c4 * cr[1])),
                 wd * (double(vb[2]) + double(c4 * cr[2])));
      }
#pragma unroll
  for (int i = 0; i < 9; ++i) C1[i] *= c4;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    // v1 holds sum W dv_i here (the u part of v' = u + sum W dv_i cancels, see above)
    const T ct = Cb[0 * 3 + d] * v1[0] + Cb[1 * 3 + d] * v1[1] + Cb[2 * 3 + d] * v1[2];
    Ab.x[Ab.at(p, d, 3)] = xb[d] + kp.inv_dx * (xacc[d] - c4 * ct);
  }
  // dL/dF = (I + dt C')^T dL/dF'
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T s = Fb1[a * 3 + c];
#pragma unroll
      for (int e = 0; e < 3; ++e) s += kp.dt * C1[e * 3 + a] * Fb1[e * 3 + c];
      Ab.F[Ab.at(p, a * 3 + c, 9)] = s;
    }
}

// ---------------------------------------------------------------------------------------------
// Reverse grid update (three_d/grid_op.py:5-47): node adjoints {dL/dvg} -> {dL/dmomentum, dL/dmass},
// written over the node's slot in the read-back format G (a node without adjoint stays all zero,
// which reads as zero in either format).
template <typename G>
__global__ void __launch_bounds__(kAdjThreads) k_adj_grid(KParams<double> kp, const Node4<double>* __restrict__ grid,
                                                          Node4<double>* __restrict__ gadj, int64_t nnodes) {
  using T = double;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nnodes) return;
  Node4<double> a = gadj[idx];
  if (a.x == T(0) && a.y == T(0) && a.z == T(0)) return;
  const int R = kp.res + 1;
  const int I[3] = {(int)(idx / ((int64_t)R * R)), (int)((idx / R) % R), (int)(idx % R)};
  const Node4<double> g = grid[idx];
  T vb[3] = {a.x, a.y, a.z};
  const T gp[3] = {g.x, g.y, g.z};
  const T m = g.w;
  if (m > T(0)) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T vd = gp[d] / m;
      if (d == 1) vd += kp.dt * kp.gravity;
      if (vd < -kp.v_allowed || vd > kp.v_allowed) vb[d] = T(0);
    }
  }
  if (kp.wall_mode == FFMPM_WALLS_REFERENCE) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (I[d] < 1 || I[d] >= kp.res - 1) vb[d] = T(0);
  } else {
    bool near = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) near = near || I[d] < 3 || I[d] > kp.res - 3;
    if (near) vb[0] = vb[1] = vb[2] = T(0);
  }
  // planar colliders zero the node velocity: nothing passes back through them
  for (int q = 0; q < kp.n_planes; ++q)
    if (behind_plane<3, double>(kp, I, q)) vb[0] = vb[1] = vb[2] = T(0);
  Node4<double> o;
  if (m > T(0)) {
    const T im = T(1) / m;
    o.x = vb[0] * im;
    o.y = vb[1] * im;
    o.z = vb[2] * im;
    o.w = -(vb[0] * gp[0] + vb[1] * gp[1] + vb[2] * gp[2]) * im * im;
  } else {
    o.x = vb[0];
    o.y = vb[1];
    o.z = vb[2];
    o.w = T(0);
  }
  store_node(reinterpret_cast<G*>(gadj), idx, o.x, o.y, o.z, o.w);
}

// dL/dF += dL/dR through the orthogonal polar factor R of F (F = R S): R [y]_x with
// (tr(S) I - S) y = axial(R^T dL/dR), axial(M) = (M21 - M12, M02 - M20, M10 - M01).
template <typename T>
__device__ __forceinline__ void polar3_vjp(const T F[9], const T R[9], const T Rb[9], T Fb[9]) {
  T S[9], M[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      S[a * 3 + c] = R[0 * 3 + a] * F[0 * 3 + c] + R[1 * 3 + a] * F[1 * 3 + c] + R[2 * 3 + a] * F[2 * 3 + c];
      M[a * 3 + c] = R[0 * 3 + a] * Rb[0 * 3 + c] + R[1 * 3 + a] * Rb[1 * 3 + c] + R[2 * 3 + a] * Rb[2 * 3 + c];
    }
  const T s01 = T(0.5) * (S[1] + S[3]), s02 = T(0.5) * (S[2] + S[6]), s12 = T(0.5) * (S[5] + S[7]);
  const T tr = S[0] + S[4] + S[8];
  const T K[9] = {tr - S[0], -s01, -s02, -s01, tr - S[4], -s12, -s02, -s12, tr - S[8]};
  const T mv[3] = {M[7] - M[5], M[2] - M[6], M[3] - M[1]};
  T Kc[9];
  cofactor3(K, Kc);
  const T det = K[0] * Kc[0] + K[1] * Kc[1] + K[2] * Kc[2];
  if (!(ffabs(det) > T(0))) return;  // two vanishing singular values: the polar factor has no derivative
  const T id = T(1) / det;
  // K symmetric: K^{-1} = cof(K)^T / det = cof(K) / det
  const T y0 = (Kc[0] * mv[0] + Kc[1] * mv[1] + Kc[2] * mv[2]) * id;
  const T y1 = (Kc[3] * mv[0] + Kc[4] * mv[1] + Kc[5] * mv[2]) * id;
  const T y2 = (Kc[6] * mv[0] + Kc[7] * mv[1] + Kc[8] * mv[2]) * id;
  const T Y[9] = {0, -y2, y1, y2, 0, -y0, -y1, y0, 0};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      Fb[a * 3 + c] += R[a * 3 + 0] * Y[0 * 3 + c] + R[a * 3 + 1] * Y[1 * 3 + c] + R[a * 3 + 2] * Y[2 * 3 + c];
}

// ---------------------------------------------------------------------------------------------
// Reverse P2G (three_d/p2g.py:14-80, utils.py:95-135).  Forward: grid momentum += W (m v + A dpos),
// mass += W m, dpos = (i - fx) dx, A = -dt vol 4 inv_dx^2 PF + m C, PF = 2mu(F-R)F^T + lam(J-1)J
// (on all nine entries, or on the diagonal for FFMPM_MODEL_FIXED_COROTATED).
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) k_adj_p2g_rev(KParams<T> kp, PView<T> P, AView<T> Ab, uint32_t n,
                                                             const ReadNode<T>* __restrict__ gadj,
                                                             int32_t* status) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  T x[3], v[3], F[9], C[9];
  load_state(P, p, x, v, F, C);
  int b[3];
  T fx[3], w[3][3], dw[3][3];
  if (!stencil3(kp, x, b, fx, w, dw)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T m, mu, lam;
  lame_of(kp, P, p, m, mu, lam);
  // The stress derivative needs F - R at the working precision relative to its own size: its mu /
  // lam terms are sums over particles and substeps of <G, (F - R) F^T>, which cancel heavily, and
  // F - R formed as the difference of float F and float R keeps only ~1e-7 / |F - R| relative
  // accuracy.  Float states take the small-strain form of F - R (as the forward stress does; float
  // relative precision), and F - R from Newton's R where the strain is large (there |F - R| >~
  // 0.02); J and the per-particle sums over the nine entries of the mu / lam terms are float64.
  T FmR[9], Rf[9];
  bool small = false;
  if constexpr (sizeof(T) == 4) small = f_minus_r_small_strain3(F, FmR);
  if (small) {
#pragma unroll
    for (int i = 0; i < 9; ++i) Rf[i] = F[i] - FmR[i];
  } else {
    polar3<T>(F, Rf, nullptr);
#pragma unroll
    for (int i = 0; i < 9; ++i) FmR[i] = F[i] - Rf[i];
  }
  double Fd[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) Fd[i] = double(F[i]);
  const double Jd = det3(Fd);
  const T Dinv = T(4) * kp.inv_dx * kp.inv_dx;
  const T s = -(kp.dt * kp.volume);
  const bool diag = kp.model == FFMPM_MODEL_FIXED_COROTATED;
  T A[9];
  {
    const T J = T(Jd);
    const T sc = lam * (J - T(1)) * J;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        T pf = (a == c || !diag) ? sc : T(0);
#pragma unroll
        for (int e = 0; e < 3; ++e) pf += T(2) * mu * FmR[a * 3 + e] * F[c * 3 + e];
        A[a * 3 + c] = s * (Dinv * pf) + m * C[a * 3 + c];
      }
  }
  const int R = kp.res + 1;
  // pass 1: the particle's weighted node adjoints gsum = sum W g, gmsum = sum W gm, held as the
  // centre node's value c plus the weighted sums of the deviations g - c
  const ReadNode<T> c = gadj[((int64_t)(b[0] + 1) * R + (b[1] + 1)) * R + (b[2] + 1)];
  T gdev[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T wt = w[i][0] * w[j][1] * w[k][2];
        T dv[4];
        node_dev(gadj[((int64_t)(b[0] + i) * R + (b[1] + j)) * R + (b[2] + k)], c, dv);
#pragma unroll
        for (int a = 0; a < 4; ++a) gdev[a] += wt * dv[a];
      }
  // pass 2: Abar = sum W (g - gsum) (x) dpos (the same sum, since sum W dpos = 0, without the
  // cancellation of the uniform part of g) and the weight derivatives for dL/dx, also on the
  // deviations g - gsum, gm - gmsum: sum dW = 0 and sum dW_d dpos = dx e_d turn the gsum terms into
  // dx (A^T gsum)_d, which cancels the explicit -(A^T gsum)_d of dpos's own x-derivative
  T Abar[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, xacc[3] = {0, 0, 0};
#pragma unroll 1
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T wt = w[i][0] * w[j][1] * w[k][2];
        const T g0 = dw[i][0] * w[j][1] * w[k][2], g1 = w[i][0] * dw[j][1] * w[k][2],
                g2 = w[i][0] * w[j][1] * dw[k][2];
        const T dp[3] = {(T(i) - fx[0]) * kp.dx, (T(j) - fx[1]) * kp.dx, (T(k) - fx[2]) * kp.dx};
        T dv[4];
        node_dev(gadj[((int64_t)(b[0] + i) * R + (b[1] + j)) * R + (b[2] + k)], c, dv);
        const T gb[3] = {dv[0] - gdev[0], dv[1] - gdev[1], dv[2] - gdev[2]};
        T term = (dv[3] - gdev[3]) * m;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const T gc = wt * gb[a];
#pragma unroll
          for (int e = 0; e < 3; ++e) Abar[a * 3 + e] += gc * dp[e];
          term += gb[a] * (m * v[a] + A[a * 3 + 0] * dp[0] + A[a * 3 + 1] * dp[1] + A[a * 3 + 2] * dp[2]);
        }
        xacc[0] += g0 * term;
        xacc[1] += g1 * term;
        xacc[2] += g2 * term;
      }
  const double gsum[3] = {node_comp(c, 0) + double(gdev[0]), node_comp(c, 1) + double(gdev[1]),
                          node_comp(c, 2) + double(gdev[2])};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const size_t ix = Ab.at(p, d, 3);
    Ab.x[ix] = Ab.x[ix] + kp.inv_dx * xacc[d];
    Ab.v[ix] = T(double(m) * gsum[d]);
  }
  // stress: G = dL/dPF; sG = <G, dPF/d(lam(J-1)J)>, the sum of G's entries (the reference's stress)
  // or its trace (the textbook model)
  T G[9], Fb[9];
  double sG = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    G[i] = (s * Dinv) * Abar[i];
    if (!diag || i % 4 == 0) sG += double(G[i]);
    Ab.C[Ab.at(p, i, 9)] = m * Abar[i];
    Fb[i] = Ab.F[Ab.at(p, i, 9)];
  }
  T Cof[9], Rb[9];
  cofactor3(F, Cof);
  double dmu = 0;
  const T lj = T(double(lam) * (2.0 * Jd - 1.0) * sG);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T gf = 0, gtfr = 0, mfr = 0;
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        gf += G[a * 3 + e] * F[e * 3 + c];       // (G F)[a][c]
        gtfr += G[e * 3 + a] * FmR[e * 3 + c];   // (G^T (F - R))[a][c]
        mfr += FmR[a * 3 + e] * F[c * 3 + e];    // ((F - R) F^T)[a][c]
      }
      Fb[a * 3 + c] += T(2) * mu * (gf + gtfr) + lj * Cof[a * 3 + c];
      Rb[a * 3 + c] = -T(2) * mu * gf;
      dmu += double(G[a * 3 + c]) * double(mfr);
    }
  polar3_vjp<T>(F, Rf, Rb, Fb);
#pragma unroll
  for (int i = 0; i < 9; ++i) Ab.F[Ab.at(p, i, 9)] = Fb[i];
  if (Ab.mu0) Ab.mu0[p] += double(kp.hardening) * 2.0 * dmu;
  if (Ab.lam0) Ab.lam0[p] += double(kp.hardening) * (Jd - 1.0) * Jd * sG;
}


// ---------------------------------------------------------------------------------------------
// 2D (two_d/p2g.py:11-76, two_d/grid_op.py:5-24, two_d/g2p.py:5-47) for the elastic models: the
// same five kernels over a dense (res+1)^2 grid, with the 0.05 wall band (the y < 0.05 rule keeps
// v_y only where it is positive, and passes its adjoint only there), no velocity clamp, and the
// closed-form rotation R of linear_algebra.py:97-116, c = x/d, s = y/d, d = |(x, y)| + 1e-10 with
// x = F00 + F11, y = F10 - F01.  Jp does not feed back for these models.  2D grids are small, so
// every grid is float64 and read back as such; F - R comes from the float64 rotation.
template <typename T>
__device__ __forceinline__ bool stencil2(const KParams<T>& kp, const T x[2], int b[2], T fx[2], T w[3][2],
                                         T dw[3][2]) {
  bool ok = true;
#pragma unroll
  for (int d = 0; d < 2; ++d) ok = ok && base_of(x[d], kp.inv_dx, kp.res, b[d], fx[d]);
  if (!ok) return false;
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    T ww[3];
    bspline(fx[d], ww);
    w[0][d] = ww[0];
    w[1][d] = ww[1];
    w[2][d] = ww[2];
    dw[0][d] = fx[d] - T(1.5);
    dw[1][d] = T(-2) * (fx[d] - T(1));
    dw[2][d] = fx[d] - T(0.5);
  }
  return true;
}

template <typename T>
__device__ __forceinline__ void load_state2(const PView<T>& P, uint32_t p, T x[2], T v[2], T F[4], T C[4]) {
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    if (x) x[d] = P.x[P.at(p, d, 2)];
    if (v) v[d] = P.v[P.at(p, d, 2)];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (F) F[i] = P.F[P.at(p, i, 4)];
    if (C) C[i] = P.C[P.at(p, i, 4)];
  }
}

template <typename T>
__global__ void __launch_bounds__(kAdjThreads) k_adj2_p2g(KParams<T> kp, PView<T> P, uint32_t n,
                                                          Node4<double>* __restrict__ grid, int32_t* status) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  T x[2], v[2], F[4], C[4];
  load_state2(P, p, x, v, F, C);
  int b[2];
  T fx[2], w[3][2], dw[3][2];
  if (!stencil2(kp, x, b, fx, w, dw)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T m, mu, lam;
  lame_of(kp, P, p, m, mu, lam);
  T A[4];
  affine_of<2, T>(kp, F, C, m, mu, lam, A, nullptr);
  const int R = kp.res + 1;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double wt = double(w[i][0]) * double(w[j][1]);
      const T d0 = (T(i) - fx[0]) * kp.dx, d1 = (T(j) - fx[1]) * kp.dx;
      const double q0 = double(m) * double(v[0]) + double(A[0] * d0 + A[1] * d1);
      const double q1 = double(m) * double(v[1]) + double(A[2] * d0 + A[3] * d1);
      atomic_add4(&grid[(int64_t)(b[0] + i) * R + (b[1] + j)], wt * q0, wt * q1, 0.0, wt * double(m));
    }
}

__global__ void __launch_bounds__(kAdjThreads) k_adj2_gridvel(KParams<double> kp, const Node4<double>* __restrict__ grid,
                                                              Node4<double>* __restrict__ gvel, int64_t nnodes) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nnodes) return;
  const int R = kp.res + 1;
  const int I[2] = {(int)(idx / R), (int)(idx % R)};
  const Node4<double> g = grid[idx];
  double vel[3] = {g.x, g.y, 0.0};
  grid_node<2, double>(kp, I, vel, g.w);
  gvel[idx] = Node4<double>{vel[0], vel[1], 0.0, g.w};
}

template <typename T>
__global__ void __launch_bounds__(kAdjThreads) k_adj2_g2p(KParams<T> kp, PView<T> P, AView<T> Ab, uint32_t n,
                                                          const Node4<double>* __restrict__ gvel,
                                                          Node4<double>* __restrict__ gadj, int32_t* status) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  T x[2], F[4];
  load_state2<T>(P, p, x, nullptr, F, nullptr);
  int b[2];
  T fx[2], w[3][2], dw[3][2];
  if (!stencil2(kp, x, b, fx, w, dw)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T xb[2], vb[2], Fb1[4], Cb[4];
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    xb[d] = Ab.x[Ab.at(p, d, 2)];
    vb[d] = Ab.v[Ab.at(p, d, 2)] + kp.dt * xb[d];  // x' = x + dt v'
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    Fb1[i] = Ab.F[Ab.at(p, i, 4)];
    Cb[i] = Ab.C[Ab.at(p, i, 4)];
  }
  // C' enters F' = (I + dt C') F: dL/dC' += dt dL/dF' F^T
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int c = 0; c < 2; ++c) Cb[a * 2 + c] += kp.dt * (Fb1[a * 2 + 0] * F[c * 2 + 0] + Fb1[a * 2 + 1] * F[c * 2 + 1]);
  const T c4 = T(4) * kp.inv_dx;
  // node velocities relative to the centre node's u, as in 3D: the u terms of dL/dx cancel
  T v1[2] = {0, 0}, C1[4] = {0, 0, 0, 0}, xacc[2] = {0, 0};
  const int R = kp.res + 1;
  const Node4<double> u = gvel[(int64_t)(b[0] + 1) * R + (b[1] + 1)];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const T wt = w[i][0] * w[j][1];
      const T g0 = dw[i][0] * w[j][1], g1 = w[i][0] * dw[j][1];
      const T r[2] = {T(i) - fx[0], T(j) - fx[1]};
      const int64_t node = (int64_t)(b[0] + i) * R + (b[1] + j);
      const Node4<double> gn = gvel[node];
      const T vel[2] = {T(gn.x - u.x), T(gn.y - u.y)};
      T cr[2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        v1[a] += wt * vel[a];
        C1[a * 2 + 0] += wt * vel[a] * r[0];
        C1[a * 2 + 1] += wt * vel[a] * r[1];
        cr[a] = Cb[a * 2 + 0] * r[0] + Cb[a * 2 + 1] * r[1];
      }
      const T term = vb[0] * vel[0] + vb[1] * vel[1] + c4 * (vel[0] * cr[0] + vel[1] * cr[1]);
      xacc[0] += g0 * term;
      xacc[1] += g1 * term;
      const double wd = double(wt);
      atomicAdd(&gadj[node].x, wd * (double(vb[0]) + double(c4 * cr[0])));
      atomicAdd(&gadj[node].y, wd * (double(vb[1]) + double(c4 * cr[1])));
    }
#pragma unroll
  for (int i = 0; i < 4; ++i) C1[i] *= c4;
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    const T ct = Cb[0 * 2 + d] * v1[0] + Cb[1 * 2 + d] * v1[1];
    Ab.x[Ab.at(p, d, 2)] = xb[d] + kp.inv_dx * (xacc[d] - c4 * ct);
  }
  // dL/dF = (I + dt C')^T dL/dF'
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int c = 0; c < 2; ++c)
      Ab.F[Ab.at(p, a * 2 + c, 4)] =
          Fb1[a * 2 + c] + kp.dt * (C1[0 * 2 + a] * Fb1[0 * 2 + c] + C1[1 * 2 + a] * Fb1[1 * 2 + c]);
}

// Reverse 2D grid update: the band's stopped nodes and the clipped v_y pass nothing, then the
// division by mass.
__global__ void __launch_bounds__(kAdjThreads) k_adj2_grid(KParams<double> kp, const Node4<double>* __restrict__ grid,
                                                           Node4<double>* __restrict__ gadj, int64_t nnodes) {
  using T = double;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nnodes) return;
  Node4<double> a = gadj[idx];
  if (a.x == T(0) && a.y == T(0)) return;
  const int R = kp.res + 1;
  const int I[2] = {(int)(idx / R), (int)(idx % R)};
  const Node4<double> g = grid[idx];
  T vb[2] = {a.x, a.y};
  const T gp[2] = {g.x, g.y};
  const T m = g.w;
  if (m > T(0)) {
    if (kp.wall_mode == FFMPM_WALLS_REFERENCE) {
      if (I[0] < kp.wall_lo || I[0] > kp.wall_hi || I[1] > kp.wall_hi) vb[0] = vb[1] = T(0);
      if (I[1] < kp.wall_lo && !(gp[1] / m + kp.dt * kp.gravity > T(0))) vb[1] = T(0);
    } else {
      const bool near = I[0] < 3 || I[0] > kp.res - 3 || I[1] < 3 || I[1] > kp.res - 3;
      if (near) vb[0] = vb[1] = T(0);
    }
  }
  for (int q = 0; q < kp.n_planes; ++q)
    if (behind_plane<2, double>(kp, I, q)) vb[0] = vb[1] = T(0);
  Node4<double> o;
  if (m > T(0)) {
    const T im = T(1) / m;
    o = Node4<double>{vb[0] * im, vb[1] * im, T(0), -(vb[0] * gp[0] + vb[1] * gp[1]) * im * im};
  } else {
    o = Node4<double>{vb[0], vb[1], T(0), T(0)};
  }
  gadj[idx] = o;
}

template <typename T>
__global__ void __launch_bounds__(kAdjThreads) k_adj2_p2g_rev(KParams<T> kp, PView<T> P, AView<T> Ab, uint32_t n,
                                                              const Node4<double>* __restrict__ gadj,
                                                              int32_t* status) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  T x[2], v[2], F[4], C[4];
  load_state2(P, p, x, v, F, C);
  int b[2];
  T fx[2], w[3][2], dw[3][2];
  if (!stencil2(kp, x, b, fx, w, dw)) {
    raise_status(status, FFMPM_STATUS_OOB);
    return;
  }
  T m, mu, lam;
  lame_of(kp, P, p, m, mu, lam);
  // the rotation in float64 (F - R at the working precision relative to its size)
  double Fd[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) Fd[i] = double(F[i]);
  const double rx = Fd[0] + Fd[3], ry = Fd[2] - Fd[1];
  const double rr = sqrt(rx * rx + ry * ry), dd = rr + 1e-10;
  const double cth = rx / dd, sth = ry / dd;
  const double Rd[4] = {cth, -sth, sth, cth};
  T FmR[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) FmR[i] = T(Fd[i] - Rd[i]);
  const double Jd = Fd[0] * Fd[3] - Fd[1] * Fd[2];
  const T Dinv = T(4) * kp.inv_dx * kp.inv_dx;
  const T s = -(kp.dt * kp.volume);
  const bool diag = kp.model == FFMPM_MODEL_FIXED_COROTATED;
  T A[4];
  {
    const T J = T(Jd);
    const T sc = lam * (J - T(1)) * J;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        T pf = (a == c || !diag) ? sc : T(0);
        pf += T(2) * mu * FmR[a * 2 + 0] * F[c * 2 + 0];
        pf += T(2) * mu * FmR[a * 2 + 1] * F[c * 2 + 1];
        A[a * 2 + c] = s * (Dinv * pf) + m * C[a * 2 + c];
      }
  }
  const int R = kp.res + 1;
  // pass 1: gsum = sum W g, gmsum = sum W gm as the centre node's value plus deviation sums
  const Node4<double> c0 = gadj[(int64_t)(b[0] + 1) * R + (b[1] + 1)];
  T gdev[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const T wt = w[i][0] * w[j][1];
      const Node4<double> a4 = gadj[(int64_t)(b[0] + i) * R + (b[1] + j)];
      gdev[0] += wt * T(a4.x - c0.x);
      gdev[1] += wt * T(a4.y - c0.y);
      gdev[2] += wt * T(a4.w - c0.w);
    }
  // pass 2: Abar = sum W (g - gsum) (x) dpos and the weight derivatives for dL/dx (see 3D)
  T Abar[4] = {0, 0, 0, 0}, xacc[2] = {0, 0};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const T wt = w[i][0] * w[j][1];
      const T g0 = dw[i][0] * w[j][1], g1 = w[i][0] * dw[j][1];
      const T dp[2] = {(T(i) - fx[0]) * kp.dx, (T(j) - fx[1]) * kp.dx};
      const Node4<double> a4 = gadj[(int64_t)(b[0] + i) * R + (b[1] + j)];
      const T gb[2] = {T(a4.x - c0.x) - gdev[0], T(a4.y - c0.y) - gdev[1]};
      T term = (T(a4.w - c0.w) - gdev[2]) * m;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const T gc = wt * gb[a];
        Abar[a * 2 + 0] += gc * dp[0];
        Abar[a * 2 + 1] += gc * dp[1];
        term += gb[a] * (m * v[a] + A[a * 2 + 0] * dp[0] + A[a * 2 + 1] * dp[1]);
      }
      xacc[0] += g0 * term;
      xacc[1] += g1 * term;
    }
  const double gsum[2] = {c0.x + double(gdev[0]), c0.y + double(gdev[1])};
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    const size_t ix = Ab.at(p, d, 2);
    Ab.x[ix] = Ab.x[ix] + kp.inv_dx * xacc[d];
    Ab.v[ix] = T(double(m) * gsum[d]);
  }
  double G[4], Fb[4], sG = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    G[i] = double(s * Dinv) * double(Abar[i]);
    if (!diag || i % 3 == 0) sG += G[i];
    Ab.C[Ab.at(p, i, 4)] = m * Abar[i];
    Fb[i] = double(Ab.F[Ab.at(p, i, 4)]);
  }
  const double Cof[4] = {Fd[3], -Fd[2], -Fd[1], Fd[0]};
  const double mud = double(mu), lj = double(lam) * (2.0 * Jd - 1.0) * sG;
  double Rb[4], dmu = 0;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const double fmr0 = double(FmR[0 * 2 + c]), fmr1 = double(FmR[1 * 2 + c]);
      const double gf = G[a * 2 + 0] * Fd[0 * 2 + c] + G[a * 2 + 1] * Fd[1 * 2 + c];
      const double gtfr = G[0 * 2 + a] * fmr0 + G[1 * 2 + a] * fmr1;
      const double mfr = double(FmR[a * 2 + 0]) * Fd[c * 2 + 0] + double(FmR[a * 2 + 1]) * Fd[c * 2 + 1];
      Fb[a * 2 + c] += 2.0 * mud * (gf + gtfr) + lj * Cof[a * 2 + c];
      Rb[a * 2 + c] = -2.0 * mud * gf;
      dmu += G[a * 2 + c] * mfr;
    }
  // through the rotation: cb, sb of R = [[c, -s], [s, c]], then c(x, y), s(x, y)
  {
    const double cb = Rb[0] + Rb[3], sb = Rb[2] - Rb[1];
    const double k = 1.0 / (rr * dd * dd);
    const double dcx = 1.0 / dd - rx * rx * k, dcy = -rx * ry * k;
    const double dsx = -rx * ry * k, dsy = 1.0 / dd - ry * ry * k;
    const double xb = cb * dcx + sb * dsx, yb = cb * dcy + sb * dsy;
    if (rr > 0.0) {
      Fb[0] += xb;
      Fb[3] += xb;
      Fb[2] += yb;
      Fb[1] -= yb;
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) Ab.F[Ab.at(p, i, 4)] = T(Fb[i]);
  if (Ab.mu0) Ab.mu0[p] += double(kp.hardening) * 2.0 * dmu;
  if (Ab.lam0) Ab.lam0[p] += double(kp.hardening) * (Jd - 1.0) * Jd * sG;
}

struct AdjLayout {
  int64_t nnodes = 0;
  size_t off_grid = 0, off_gvel = 0, off_gadj = 0, total = 0;
};

bool adj_layout(const ffmpm_params& p, AdjLayout* L) {
  if ((p.dim != 2 && p.dim != 3) || (p.real_bytes != 4 && p.real_bytes != 8) || p.res < 3) return false;
  if (p.res > (p.dim == 3 ? 1024 : 16384)) return false;
  const int64_t R = p.res + 1;
  L->nnodes = p.dim == 3 ? R * R * R : R * R;
  const size_t nb = sizeof(Node4<double>) * L->nnodes;  // float64 node grids for either real type
  L->off_grid = sizeof(WsHeader);
  L->off_gvel = (L->off_grid + nb + 255) / 256 * 256;
  L->off_gadj = (L->off_gvel + nb + 255) / 256 * 256;
  L->total = (L->off_gadj + nb + 255) / 256 * 256;
  return true;
}

template <typename T>
int run_adjoint(const ffmpm_params& p, const AdjLayout& L, const ffmpm_particles& P, const ffmpm_adjoint& A,
                unsigned char* ws, cudaStream_t s) {
  const KParams<T> kp = kparams<T>(p);
  const PView<T> pv = pview<T>(P);
  AView<T> av{static_cast<T*>(A.x), static_cast<T*>(A.v), static_cast<T*>(A.F), static_cast<T*>(A.C), A.mu_0,
              A.lambda_0, P.stride};
  auto* hdr = reinterpret_cast<WsHeader*>(ws);
  const KParams<double> kd = kparams<double>(p);
  auto* grid = reinterpret_cast<Node4<double>*>(ws + L.off_grid);
  auto* gvel = reinterpret_cast<Node4<double>*>(ws + L.off_gvel);
  auto* gadj = reinterpret_cast<Node4<double>*>(ws + L.off_gadj);
  const size_t nb = sizeof(Node4<double>) * L.nnodes;
  cudaMemsetAsync(grid, 0, nb, s);
  cudaMemsetAsync(gadj, 0, nb, s);
  const uint32_t n = (uint32_t)P.n;
  const int pg = (int)((n + kAdjThreads - 1) / kAdjThreads);
  const int ng = (int)((L.nnodes + kAdjThreads - 1) / kAdjThreads);
  if (p.dim == 2) {
    k_adj2_p2g<T><<<pg, kAdjThreads, 0, s>>>(kp, pv, n, grid, &hdr->status);
    k_adj2_gridvel<<<ng, kAdjThreads, 0, s>>>(kd, grid, gvel, L.nnodes);
    k_adj2_g2p<T><<<pg, kAdjThreads, 0, s>>>(kp, pv, av, n, gvel, gadj, &hdr->status);
    k_adj2_grid<<<ng, kAdjThreads, 0, s>>>(kd, grid, gadj, L.nnodes);
    k_adj2_p2g_rev<T><<<pg, kAdjThreads, 0, s>>>(kp, pv, av, n, gadj, &hdr->status);
    return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
  }
  k_adj_p2g<T><<<pg, kAdjThreads, 0, s>>>(kp, pv, n, grid, &hdr->status);
  using G = ReadNode<T>;
  k_adj_gridvel<G><<<ng, kAdjThreads, 0, s>>>(kd, grid, reinterpret_cast<G*>(gvel), L.nnodes);
  k_adj_g2p<T><<<pg, kAdjThreads, 0, s>>>(kp, pv, av, n, reinterpret_cast<const G*>(gvel), gadj, &hdr->status);
  k_adj_grid<G><<<ng, kAdjThreads, 0, s>>>(kd, grid, gadj, L.nnodes);
  k_adj_p2g_rev<T><<<pg, kAdjThreads, 0, s>>>(kp, pv, av, n, reinterpret_cast<const G*>(gadj), &hdr->status);
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

}  // namespace
}  // namespace ffmpm

using namespace ffmpm;

extern "C" {

int ffmpm_adjoint_workspace_size(const ffmpm_params* p, int64_t n, size_t* bytes) {
  AdjLayout L;
  if (!p || !bytes || n < 0) return FFMPM_ERR_BADARG;
  if (p->dim != 2 && p->dim != 3) return FFMPM_ERR_UNSUPPORTED;
  if (!adj_layout(*p, &L)) return FFMPM_ERR_BADARG;
  *bytes = L.total;
  return FFMPM_OK;
}

int ffmpm_substep_adjoint(const ffmpm_params* p, const ffmpm_particles* P, ffmpm_adjoint* A, void* ws,
                          size_t ws_bytes, void* stream) {
  if (!p || !P || !A || P->n < 0 || P->n > int64_t(0x7FFFFFFF)) return FFMPM_ERR_BADARG;
  if ((p->dim != 2 && p->dim != 3) ||
      (p->model != FFMPM_MODEL_NEO_HOOKEAN && p->model != FFMPM_MODEL_FIXED_COROTATED))
    return FFMPM_ERR_UNSUPPORTED;
  if (p->wall_mode != FFMPM_WALLS_REFERENCE && p->wall_mode != FFMPM_WALLS_STICKY3) return FFMPM_ERR_BADARG;
  AdjLayout L;
  if (!adj_layout(*p, &L)) return FFMPM_ERR_BADARG;
  if (!ws || ws_bytes < L.total || (reinterpret_cast<uintptr_t>(ws) & 255)) return FFMPM_ERR_WORKSPACE;
  if (P->stride != 0 && P->stride < P->n) return FFMPM_ERR_BADARG;
  if (P->n == 0) return FFMPM_OK;
  if (!P->x || !P->v || !P->F || !P->C || !A->x || !A->v || !A->F || !A->C) return FFMPM_ERR_BADARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto* base = static_cast<unsigned char*>(ws);
  return p->real_bytes == 4 ? run_adjoint<float>(*p, L, *P, *A, base, s) : run_adjoint<double>(*p, L, *P, *A, base, s);
}

}  // extern "C"
