// Shared device code for the MLS-MPM substep kernels (sm_103a).
//
// Reference semantics (FEMFlow, femflow/solvers/mpm/...):
//   quadratic B-spline weights          three_d/p2g.py:55
//   base = int64(x*inv_dx - 0.5)        three_d/p2g.py:50 (truncation toward zero)
//   fixed-corotated stress + APIC       utils.py:95-135 (3D), utils.py:52-92 (2D)
//   polar decomposition                 numerics/linear_algebra.py:96-135
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "femflow_mpm.h"

namespace ffmpm {

constexpr int kThreads = 256;

// ----------------------------------------------------------------------------------------------
// Precision traits
template <typename T>
struct alignas(4 * sizeof(T)) Node4 {
  T x, y, z, w;
};

template <typename T>
__device__ __forceinline__ T ffabs(T a) { return a < T(0) ? -a : a; }
__device__ __forceinline__ float ffsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double ffsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float ffexp(float a) { return expf(a); }
__device__ __forceinline__ double ffexp(double a) { return exp(a); }
template <typename T>
__device__ __forceinline__ T ffclamp(T v, T lo, T hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <typename T>
struct Eps;
template <>
struct Eps<float> {
  static constexpr float value = 1.1920929e-07f;
};
template <>
struct Eps<double> {
  static constexpr double value = 2.220446049250313e-16;
};

// ----------------------------------------------------------------------------------------------
// Status word (device side).  Bits of FFMPM_STATUS_* are OR-ed in; the host reads it after sync.
__device__ __forceinline__ void raise_status(int32_t* status, int32_t bit) {
  if (status) atomicOr(status, bit);
}

// NaN when any of the n values is NaN or infinite, else 0: v * 0 is exact for finite v, so no
// finite value, however large, gives a false alarm.
template <typename T>
__device__ __forceinline__ T nonfinite_probe(const T* v, int n) {
  T acc = T(0);
#pragma unroll
  for (int i = 0; i < n; ++i) acc = fma(v[i], T(0), acc);
  return acc;
}

// True once a bounded wait has given up (since the status word was last cleared).  A permutation
// made by a sort that gave up may hold indices the sort never wrote, so kernels that read particles
// through one leave at once instead.
__device__ __forceinline__ bool wait_gave_up(const int32_t* status) {
  return status && (*reinterpret_cast<const volatile int32_t*>(status) & FFMPM_STATUS_TIMEOUT);
}

// ----------------------------------------------------------------------------------------------
// Grid geometry shared by all kernels.  Nodes per axis R = res + 1.  The grid is split into
// cubic (square in 2D) blocks of BS nodes per axis for work assignment: a particle belongs to the
// block that holds its base node, and its 3-node stencil then stays inside the block's tile of
// BS+2 nodes per axis.
template <int DIM>
struct Geom {
  int res;     // grid resolution
  int R;       // nodes per axis
  int bs;      // block side (nodes), a power of two
  int bs_shift;  // log2(bs): cell coordinates are decoded with shifts and masks, not divisions
  int nb;      // blocks per axis = ceil(R / bs)
  int nblocks; // nb^DIM
  int tile;    // bs + 2
};

// ----------------------------------------------------------------------------------------------
// Base node and fractional offset, following the reference's truncation (astype(int64)).
// Returns false for out-of-range or non-finite coordinates (the reference raises RuntimeError).
// Products and differences here are rounded separately (no FMA contraction), as numpy computes
// `pos * inv_dx - 0.5`, so the base node is reproducible bit for bit on the host.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <typename T>
__device__ __forceinline__ bool base_of(T x, T inv_dx, int res, int& b, T& fx) {
  const T xs = mul_rn(x, inv_dx);
  const T t = sub_rn(xs, T(0.5));
  if (!(t > T(-1) && t < T(res))) return false;
  b = static_cast<int>(t);  // truncation toward zero, as numpy astype(int64)
  if (b < 0 || b + 2 > res) return false;
  fx = sub_rn(xs, T(b));
  return true;
}

template <typename T>
__device__ __forceinline__ void bspline(T fx, T w[3]) {
  const T a = T(1.5) - fx, b = fx - T(1), c = fx - T(0.5);
  w[0] = T(0.5) * a * a;
  w[1] = T(0.75) - b * b;
  w[2] = T(0.5) * c * c;
}

// ----------------------------------------------------------------------------------------------
// Small dense matrix helpers (row-major).
template <typename T>
__device__ __forceinline__ T det3(const T m[9]) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

template <typename T>
__device__ __forceinline__ void cofactor3(const T m[9], T c[9]) {
  c[0] = m[4] * m[8] - m[5] * m[7];
  c[1] = m[5] * m[6] - m[3] * m[8];
  c[2] = m[3] * m[7] - m[4] * m[6];
  c[3] = m[2] * m[7] - m[1] * m[8];
  c[4] = m[0] * m[8] - m[2] * m[6];
  c[5] = m[1] * m[6] - m[0] * m[7];
  c[6] = m[1] * m[5] - m[2] * m[4];
  c[7] = m[2] * m[3] - m[0] * m[5];
  c[8] = m[0] * m[4] - m[1] * m[3];
}

// Orthogonal polar factor R of F (F = R S, S symmetric positive definite) by Newton's iteration
// X <- (g X + X^{-T}/g)/2 with Frobenius-norm scaling g (Higham 1986, "Computing the polar
// decomposition - with applications").  The iteration converges to the unique orthogonal polar
// factor of any nonsingular F, including det F < 0, where R is a reflection exactly as
// U @ Vh from an SVD (linear_algebra.py:131-132).  Returns the number of iterations, or -1 when F
// is (numerically) singular or the iteration did not settle.
__device__ __forceinline__ float ffrcp(float a) { return __frcp_rn(a); }
__device__ __forceinline__ double ffrcp(double a) { return __drcp_rn(a); }

__device__ __forceinline__ float ffrsqrt_approx(float a) { return rsqrtf(a); }
__device__ __forceinline__ double ffrsqrt_approx(double a) { return rsqrt(a); }

// Newton iteration for the orthogonal polar factor (see polar3).  `degenerate_ratio`: when > 0,
// the call returns -2 without iterating if |det F| <= degenerate_ratio * (|F|_F / sqrt 3)^3
// (F close to singular relative to its size).  Returns the number of iterations, or -1 when the
// iteration did not settle / F is singular.
template <typename T>
__device__ __forceinline__ int polar3_newton(const T F[9], T R[9], int max_iter, T degenerate_ratio = T(0)) {
  T X[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) X[i] = F[i];
  const T tol = T(8) * Eps<T>::value;
  for (int it = 0; it < max_iter; ++it) {
    T cof[9];
    cofactor3(X, cof);
    const T det = X[0] * cof[0] + X[1] * cof[1] + X[2] * cof[2];
    // Frobenius scaling g = (|X^{-1}|_F / |X|_F)^(1/2) speeds up the first iterations; close to the
    // solution g -> 1, so later iterations are unscaled.  Any positive g leaves the fixed point
    // unchanged, so g is computed with approximate square roots.
    T g = T(1);
    if (it < 2) {
      T nx = 0, nc = 0;
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        nx += X[i] * X[i];
        nc += cof[i] * cof[i];
      }
      if (it == 0 && degenerate_ratio > T(0)) {
        // (|F|/sqrt3)^3 = nx^(3/2) / 5.196
        if (!(ffabs(det) > degenerate_ratio * nx * ffsqrt(nx) * T(0.19245009))) return -2;
      }
      if (!(nx > T(0)) || !(ffabs(det) > T(0))) return -1;
      // g^4 = |cof|^2 / (det^2 |X|^2)
      const T g4 = nc * ffrcp(det * det * nx);
      g = ffrcp(ffrsqrt_approx(ffrsqrt_approx(g4)));  // g4^(1/4)
    } else if (!(ffabs(det) > T(0))) {
      return -1;
    }
    const T inv_det = ffrcp(det);
    const T ha = T(0.5) * g, hb = T(0.5) * inv_det / g;
    T diff = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const T xn = ha * X[i] + hb * cof[i];
      const T d = xn - X[i];
      diff += d * d;
      X[i] = xn;
    }
    if (diff <= tol * tol * T(3)) {
#pragma unroll
      for (int i = 0; i < 9; ++i) R[i] = X[i];
      return it + 1;
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = X[i];
  return -1;
}

// Polar factor used by the stress.  In float, F whose smallest singular value is small relative
// to its largest (|det F| / (|F|_F/sqrt 3)^3 at most 1e-3) or where the float iteration does not
// settle is redone in double; `fallbacks` counts those particles.
// The double redo of a float polar factor: a call of its own (rarely taken), so that its double
// registers do not count against the float kernels that inline polar3.
static __device__ __noinline__ void polar3_redo_fp64(const float* F, float* R, uint32_t* fallbacks) {
  double Fd[9], Rd[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) Fd[i] = double(F[i]);
  polar3_newton(Fd, Rd, 60);
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = float(Rd[i]);
  if (fallbacks) atomicAdd(fallbacks, 1u);
}

template <typename T>
__device__ __forceinline__ void polar3(const T F[9], T R[9], uint32_t* fallbacks) {
  if constexpr (sizeof(T) == 4) {
    if (polar3_newton(F, R, 12, T(1e-3)) < 0) {
      // copies made here, on the rare path, so that the call does not take the address of the
      // caller's F and R (which would keep them in local memory for every particle)
      float Fl[9], Rl[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) Fl[i] = F[i];
      polar3_redo_fp64(Fl, Rl, fallbacks);
#pragma unroll
      for (int i = 0; i < 9; ++i) R[i] = Rl[i];
    }
  } else {
    // double: a failure means F is singular to working precision; the last iterate is kept (the
    // reference's LAPACK answer is arbitrary in the null space there) and counted.
    if (polar3_newton(F, R, 60) < 0 && fallbacks) atomicAdd(fallbacks, 1u);
  }
}

// 3x3 SVD F = U diag(s) V^T, s >= 0 descending, by one-sided (Hestenes) Jacobi rotations of the
// columns of F; U and V are orthogonal (det U det V = sign det F).  Used by the snow model's
// singular-value clamp (three_d/g2p.py:48-58).
template <typename T>
__device__ __forceinline__ void svd3(const T F[9], T U[9], T s[3], T V[9]) {
  T A[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    A[i] = F[i];
    V[i] = (i % 4 == 0) ? T(1) : T(0);
  }
  const T tol = T(4) * Eps<T>::value;
  for (int sweep = 0; sweep < 12; ++sweep) {
    T off = T(0);
#pragma unroll
    for (int pi = 0; pi < 3; ++pi) {
      const int p = pi == 2 ? 1 : 0, q = pi == 0 ? 1 : 2;
      T alpha = 0, beta = 0, gamma = 0;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        alpha += A[i * 3 + p] * A[i * 3 + p];
        beta += A[i * 3 + q] * A[i * 3 + q];
        gamma += A[i * 3 + p] * A[i * 3 + q];
      }
      const T nrm = ffsqrt(alpha * beta);
      if (!(nrm > T(0)) || gamma == T(0)) continue;
      const T rel = ffabs(gamma) / nrm;
      off = rel > off ? rel : off;
      if (rel < tol) continue;
      const T zeta = (beta - alpha) / (T(2) * gamma);
      const T tt = (zeta >= T(0) ? T(1) : T(-1)) / (ffabs(zeta) + ffsqrt(T(1) + zeta * zeta));
      const T c = T(1) / ffsqrt(T(1) + tt * tt), sn = c * tt;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const T ap = A[i * 3 + p], aq = A[i * 3 + q];
        A[i * 3 + p] = c * ap - sn * aq;
        A[i * 3 + q] = sn * ap + c * aq;
        const T vp = V[i * 3 + p], vq = V[i * 3 + q];
        V[i * 3 + p] = c * vp - sn * vq;
        V[i * 3 + q] = sn * vp + c * vq;
      }
    }
    if (off < tol) break;
  }
  T n[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) n[j] = ffsqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
  // order the columns by decreasing singular value (three compare-and-swap steps)
#pragma unroll
  for (int step = 0; step < 3; ++step) {
    const int a = step == 1 ? 1 : 0, b = step == 0 ? 1 : 2;
    if (n[b] > n[a]) {
      const T tn = n[a];
      n[a] = n[b];
      n[b] = tn;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        T t1 = A[i * 3 + a];
        A[i * 3 + a] = A[i * 3 + b];
        A[i * 3 + b] = t1;
        t1 = V[i * 3 + a];
        V[i * 3 + a] = V[i * 3 + b];
        V[i * 3 + b] = t1;
      }
    }
  }
  const T smax = n[0] > T(0) ? n[0] : T(1);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    s[j] = n[j];
    const bool full = n[j] > smax * T(64) * Eps<T>::value;
#pragma unroll
    for (int i = 0; i < 3; ++i) U[i * 3 + j] = full ? A[i * 3 + j] / n[j] : T(0);
  }
  // a (numerically) null third column: complete U with the cross product of the first two
  if (!(n[2] > smax * T(64) * Eps<T>::value)) {
    U[2] = U[3] * U[7] - U[6] * U[4];
    U[5] = U[6] * U[1] - U[0] * U[7];
    U[8] = U[0] * U[4] - U[3] * U[1];
  }
}

// linear_algebra.py:96-116 (2D closed form with +1e-10 in the denominator).
template <typename T>
__device__ __forceinline__ void polar2(const T m[4], T r[4]) {
  const T x = m[0] + m[3];
  const T y = m[2] - m[1];
  const T denom = ffsqrt(x * x + y * y) + T(1e-10);
  const T scale = T(1) / denom;
  const T c = x * scale, s = y * scale;
  r[0] = c;
  r[1] = -s;
  r[2] = s;
  r[3] = c;
}

// 2x2 SVD F = U diag(s) V^T, s >= 0 descending, by the two-angle closed form.
template <typename T>
__device__ __forceinline__ void svd2(const T F[4], T U[4], T s[2], T V[4]) {
  const T a = F[0], b = F[1], c = F[2], d = F[3];
  const T E = T(0.5) * (a + d), Fh = T(0.5) * (a - d), G = T(0.5) * (c + b), H = T(0.5) * (c - b);
  const T Q = ffsqrt(E * E + H * H), Rr = ffsqrt(Fh * Fh + G * G);
  T s1 = Q + Rr, s2 = Q - Rr;
  const T a1 = atan2(G, Fh), a2 = atan2(H, E);
  const T th = T(0.5) * (a2 - a1), ph = T(0.5) * (a2 + a1);
  T su, cu, sv, cv;
  if constexpr (sizeof(T) == 4) {
    sincosf(ph, &su, &cu);
    sincosf(th, &sv, &cv);
  } else {
    sincos(ph, &su, &cu);
    sincos(th, &sv, &cv);
  }
  U[0] = cu; U[1] = -su; U[2] = su; U[3] = cu;
  V[0] = cv; V[1] = sv; V[2] = -sv; V[3] = cv;
  if (s2 < T(0)) {
    s2 = -s2;
    U[1] = -U[1];
    U[3] = -U[3];
  }
  s[0] = s1;
  s[1] = s2;
}

// ----------------------------------------------------------------------------------------------
// Warp helpers
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Add 1 to counts[key] for every lane with valid=true, one atomic per distinct key in the warp.
__device__ __forceinline__ void warp_count(unsigned* counts, unsigned key, bool valid) {
  const unsigned active = __activemask();
  const unsigned vmask = __ballot_sync(active, valid);
  if (!valid) return;
  const unsigned peers = __match_any_sync(vmask, key);
  const int leader = __ffs(peers) - 1;
  if ((threadIdx.x & 31) == leader) atomicAdd(&counts[key], (unsigned)__popc(peers));
}

// ----------------------------------------------------------------------------------------------
// Vector atomics into global memory.
__device__ __forceinline__ void atomic_add4(Node4<float>* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}
__device__ __forceinline__ void atomic_add4(Node4<double>* p, double a, double b, double c, double d) {
  atomicAdd(&p->x, a);
  atomicAdd(&p->y, b);
  atomicAdd(&p->z, c);
  atomicAdd(&p->w, d);
}

// ----------------------------------------------------------------------------------------------
// mbarrier + TMA (cp.async.bulk.tensor) wrappers.  Every wait is bounded: after kSpinLimit polls
// the caller records FFMPM_STATUS_TIMEOUT and gives up instead of hanging the GPU.
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// Returns true once the phase with the given parity has completed; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t addr = smem_u32(bar);
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_4d(void* smem_dst, const void* tmap, uint64_t* bar, int c0, int c1,
                                            int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(smem_dst)),
      "l"(tmap), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const void* tmap, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(smem_dst)),
      "l"(tmap), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

}  // namespace ffmpm
