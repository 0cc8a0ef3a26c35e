// Stable LSD radix sort of 32-bit keys with a 32-bit permutation payload (8-bit digits).
//
// Each pass: (1) per-tile digit histograms, (2) one exclusive scan over the digit-major
// [digit][tile] table, (3) a stable scatter in which every warp ranks its keys with
// __match_any_sync in index order.  Stability makes the permutation bit-exact: it equals a CPU
// stable sort of the same keys (numpy argsort kind="stable").
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace ffmpm {

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsWarps = kRsThreads / 32;
static_assert(kRsThreads * kRsItems == kRadixTile, "tile size");

__global__ void __launch_bounds__(kRsThreads) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                            int shift, uint32_t* __restrict__ hist, int ntiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * (uint32_t)kRadixTile;
#pragma unroll 4
  for (int it = 0; it < kRsItems; ++it) {
    const uint32_t i = base + it * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(__ldg(&keys[i]) >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of `total` counts in place, one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) k_radix_scan(uint32_t* __restrict__ hist, int total) {
  __shared__ uint32_t warp_sums[32];
  const int per = (total + 1023) / 1024;
  const int beg = threadIdx.x * per;
  const int end = min(total, beg + per);
  uint32_t sum = 0;
  for (int i = beg; i < end; ++i) sum += hist[i];
  // block exclusive scan of `sum`
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t ws = warp_sums[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += t;
    }
    warp_sums[lane] = ws;
  }
  __syncthreads();
  uint32_t run = inc - sum + (warp > 0 ? warp_sums[warp - 1] : 0u);
  for (int i = beg; i < end; ++i) {
    const uint32_t c = hist[i];
    hist[i] = run;
    run += c;
  }
}

__global__ void __launch_bounds__(kRsThreads) k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                                               const uint32_t* __restrict__ vals_in, uint32_t n,
                                                               int shift, const uint32_t* __restrict__ hist,
                                                               int ntiles, uint32_t* __restrict__ keys_out,
                                                               uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t wcnt[kRsWarps][256];
  for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t sub = blockIdx.x * (uint32_t)kRadixTile + warp * (kRsItems * 32);
  const unsigned lt = lanemask_lt();
  uint32_t key[kRsItems], val[kRsItems], off[kRsItems];
  uint32_t dig[kRsItems];
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const uint32_t i = sub + r * 32 + lane;
    const bool valid = i < n;
    const uint32_t k = valid ? keys_in[i] : 0u;
    const uint32_t v = valid ? (vals_in ? vals_in[i] : i) : 0u;
    const uint32_t d = valid ? ((k >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (lane == leader && d < 256u) {
      old = wcnt[warp][d];
      wcnt[warp][d] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    off[r] = old + __popc(peers & lt);
    key[r] = k;
    val[r] = v;
    dig[r] = d;
    __syncwarp();
  }
  __syncthreads();
  {
    const int d = threadIdx.x;  // 256 threads, one digit each
    uint32_t run = hist[d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
      const uint32_t t = wcnt[w][d];
      wcnt[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    if (dig[r] < 256u) {
      const uint32_t pos = wcnt[warp][dig[r]] + off[r];
      if (keys_out) keys_out[pos] = key[r];
      vals_out[pos] = val[r];
    }
  }
}

}  // namespace

void radix_sort(const uint32_t* keys_in, uint32_t n, int passes, uint32_t* keys0, uint32_t* keys1,
                uint32_t* vals0, uint32_t* vals1, uint32_t* hist, int ntiles, cudaStream_t s,
                const uint32_t** keys_sorted, const uint32_t** perm) {
  const uint32_t* kin = keys_in;
  const uint32_t* vin = nullptr;
  uint32_t* kbuf[2] = {keys0, keys1};
  uint32_t* vbuf[2] = {vals0, vals1};
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = 8 * pass;
    k_radix_hist<<<ntiles, kRsThreads, 0, s>>>(kin, n, shift, hist, ntiles);
    k_radix_scan<<<1, 1024, 0, s>>>(hist, 256 * ntiles);
    k_radix_scatter<<<ntiles, kRsThreads, 0, s>>>(kin, vin, n, shift, hist, ntiles, kbuf[pass & 1],
                                                  vbuf[pass & 1]);
    kin = kbuf[pass & 1];
    vin = vbuf[pass & 1];
  }
  *keys_sorted = kin;
  *perm = vin;
}

}  // namespace ffmpm
