// Scene sampling: generate_implicit_points (femflow/simulation/mpm/primitives.py:46-61) for the
// reference's three triply periodic minimal surfaces (primitives.py:9-38).
//
// The reference evaluates the implicit function at every point of a res^3 lattice in [0, 1]^3
// (femflow/numerics/geometry.py:100-116: first axis fastest, coordinate i / (res - 1)) one point
// at a time in Python, and keeps the points whose value, which already has t subtracted, is larger
// than t (`inside > t`), in lattice order.  Here one thread evaluates eight points; the kept
// points are compacted in lattice order by three launches: per-tile counts, one scan of the tile
// counts, and the write.  The arithmetic is float64 with every product, sum and difference rounded
// on its own (no fused multiply-add), in the reference's order, so that the value, and with it the
// kept set, is the reference's whenever the two sine/cosine libraries agree.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.h"

namespace ffmpm {
namespace {

constexpr int kImpThreads = 256;
constexpr int kImpItems = 8;
constexpr int kImpTile = kImpThreads * kImpItems;  // lattice points per CTA
constexpr int kImpScanThreads = 1024;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

// The implicit value minus t of lattice point p (as primitives.py writes it), compared with t.
__device__ __forceinline__ bool inside(int kind, double w, double t, int res, int64_t p, double xyz[3]) {
  const int64_t r = res;
  const int64_t idx[3] = {p % r, (p / r) % r, p / (r * r)};
#pragma unroll
  for (int d = 0; d < 3; ++d) xyz[d] = res == 1 ? 0.0 : __ddiv_rn((double)idx[d], (double)(res - 1));
  const double ax = mul(w, xyz[0]), ay = mul(w, xyz[1]), az = mul(w, xyz[2]);
  double f;
  if (kind == FFMPM_TPMS_PRIMITIVE) {
    f = add(add(cos(ax), cos(ay)), cos(az));
  } else {
    const double sx = sin(ax), sy = sin(ay), sz = sin(az);
    const double cx = cos(ax), cy = cos(ay), cz = cos(az);
    if (kind == FFMPM_TPMS_GYROID)
      f = add(add(mul(sx, cy), mul(sy, cz)), mul(sz, cx));
    else  // diamond
      f = add(add(add(mul(mul(sx, sy), sz), mul(mul(sx, cy), cz)), mul(mul(cx, sy), cz)), mul(mul(cx, cy), sz));
  }
  return __dsub_rn(f, t) > t;
}

// Kept points per tile of kImpTile lattice points.
__global__ void __launch_bounds__(kImpThreads) k_implicit_count(int kind, double w, double t, int res, int64_t n,
                                                                 uint32_t* __restrict__ tile_count) {
  __shared__ uint32_t warp_sum[kImpThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kImpTile;
  uint32_t c = 0;
  double xyz[3];
#pragma unroll
  for (int i = 0; i < kImpItems; ++i) {
    const int64_t p = base + (int64_t)i * kImpThreads + threadIdx.x;
    if (p < n && inside(kind, w, t, res, p, xyz)) ++c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w2 = 0; w2 < kImpThreads / 32; ++w2) s += warp_sum[w2];
    tile_count[blockIdx.x] = s;
  }
}

// Exclusive offsets of the tiles (one CTA, carried over chunks of kImpScanThreads) and the total.
__global__ void __launch_bounds__(kImpScanThreads) k_implicit_scan(const uint32_t* __restrict__ tile_count,
                                                                    int64_t* __restrict__ tile_off, int ntiles,
                                                                    int64_t* __restrict__ total) {
  __shared__ int64_t warp_sum[kImpScanThreads / 32];
  __shared__ int64_t carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b0 = 0; b0 < ntiles; b0 += kImpScanThreads) {
    const int i = b0 + threadIdx.x;
    const int64_t v = i < ntiles ? (int64_t)tile_count[i] : 0;
    int64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31) warp_sum[warp] = inc;
    __syncthreads();
    int64_t before = carry_s;
    for (int w2 = 0; w2 < warp; ++w2) before += warp_sum[w2];
    if (i < ntiles) tile_off[i] = before + inc - v;
    __syncthreads();
    if (threadIdx.x == kImpScanThreads - 1) carry_s = before + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry_s;
}

// The kept points of each tile at the tile's offset, in lattice order (each thread's eight points
// are consecutive lattice points, so thread order within the CTA is lattice order).
__global__ void __launch_bounds__(kImpThreads) k_implicit_write(int kind, double w, double t, int res, int64_t n,
                                                                 const int64_t* __restrict__ tile_off,
                                                                 double* __restrict__ out, int64_t capacity) {
  __shared__ uint32_t warp_sum[kImpThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kImpTile + (int64_t)threadIdx.x * kImpItems;
  uint32_t keep = 0;
#pragma unroll
  for (int i = 0; i < kImpItems; ++i) {
    const int64_t p = base + i;
    double xyz[3];
    if (p < n && inside(kind, w, t, res, p, xyz)) keep |= 1u << i;
  }
  const uint32_t c = __popc(keep);
  uint32_t inc = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) warp_sum[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
  for (int w2 = 0; w2 < warp; ++w2) before += warp_sum[w2];
  int64_t q = tile_off[blockIdx.x] + before + inc - c;
#pragma unroll
  for (int i = 0; i < kImpItems; ++i) {
    if (!(keep & (1u << i))) continue;
    if (q < capacity) {
      double xyz[3];
      inside(kind, w, t, res, base + i, xyz);
      out[q * 3 + 0] = xyz[0];
      out[q * 3 + 1] = xyz[1];
      out[q * 3 + 2] = xyz[2];
    }
    ++q;
  }
}

int64_t ntiles_of(int res) {
  const int64_t n = (int64_t)res * res * res;
  return (n + kImpTile - 1) / kImpTile;
}

}  // namespace
}  // namespace ffmpm

using namespace ffmpm;

extern "C" {

int ffmpm_implicit_points_workspace_size(int32_t res, size_t* bytes) {
  if (!bytes || res < 1 || res > FFMPM_IMPLICIT_MAX_RES) return FFMPM_ERR_BADARG;
  const int64_t nt = ntiles_of(res);
  *bytes = (size_t)nt * (sizeof(uint32_t) + sizeof(int64_t)) + 16;
  return FFMPM_OK;
}

int ffmpm_implicit_points(int32_t kind, double k, double t, int32_t res, double* points, int64_t capacity,
                          int64_t* count, void* ws, size_t ws_bytes, void* stream) {
  if (kind != FFMPM_TPMS_GYROID && kind != FFMPM_TPMS_DIAMOND && kind != FFMPM_TPMS_PRIMITIVE) return FFMPM_ERR_BADARG;
  if (res < 1 || res > FFMPM_IMPLICIT_MAX_RES || !count || capacity < 0 || (capacity > 0 && !points))
    return FFMPM_ERR_BADARG;
  if (!std::isfinite(k) || k == 0.0 || !std::isfinite(t)) return FFMPM_ERR_BADARG;
  size_t need = 0;
  ffmpm_implicit_points_workspace_size(res, &need);
  if (!ws || ws_bytes < need || (reinterpret_cast<uintptr_t>(ws) & 15)) return FFMPM_ERR_WORKSPACE;
  const int64_t nt = ntiles_of(res);
  const int64_t n = (int64_t)res * res * res;
  int64_t* off = static_cast<int64_t*>(ws);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(off + nt);
  const double w = (2.0 * M_PI) / k;  // two_pi = (2.0 * np.pi) / k, as primitives.py:10
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_implicit_count<<<(unsigned)nt, kImpThreads, 0, s>>>(kind, w, t, res, n, cnt);
  k_implicit_scan<<<1, kImpScanThreads, 0, s>>>(cnt, off, (int)nt, count);
  if (capacity > 0) k_implicit_write<<<(unsigned)nt, kImpThreads, 0, s>>>(kind, w, t, res, n, off, points, capacity);
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

}  // extern "C"
