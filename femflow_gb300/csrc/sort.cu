// Stable LSD radix sort of 32-bit keys with a 32-bit permutation payload (digits of up to 11
// bits; a 22-bit key sorts in two passes).
//
// Each pass: (1) per-tile digit histograms plus per-digit totals, (2) one CTA per digit turns its
// row of tile counts into global offsets, (3) a stable scatter in which every warp ranks its keys
// with __match_any_sync in index order.  Stability makes the permutation bit-exact: it equals a
// CPU stable sort of the same keys (numpy argsort kind="stable").
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace ffmpm {

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsWarps = kRsThreads / 32;
static_assert(kRsThreads * kRsItems == kRadixTile, "tile size");

// Per-tile digit histogram; also adds the tile's counts into the pass's digit totals.
__global__ void __launch_bounds__(kRsThreads) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                            int shift, uint32_t mask, uint32_t* __restrict__ hist,
                                                            int ntiles, uint32_t* __restrict__ totals) {
  extern __shared__ uint32_t h[];
  const int nbins = (int)mask + 1;
  for (int d = threadIdx.x; d < nbins; d += kRsThreads) h[d] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * (uint32_t)kRadixTile;
#pragma unroll 4
  for (int it = 0; it < kRsItems; ++it) {
    const uint32_t i = base + it * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(__ldg(&keys[i]) >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nbins; d += kRsThreads) {
    const uint32_t c = h[d];
    hist[(size_t)d * ntiles + blockIdx.x] = c;
    if (c) atomicAdd(&totals[d], c);
  }
}

__device__ __forceinline__ uint32_t block_sum_256(uint32_t v, uint32_t* buf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) buf[warp] = v;
  __syncthreads();
  uint32_t t = 0;
#pragma unroll
  for (int w = 0; w < kRsThreads / 32; ++w) t += buf[w];
  __syncthreads();
  return t;
}

// One CTA per digit d: global offset of every (d, tile) = sum of the totals of digits < d plus the
// exclusive prefix of digit d's tile counts.
__global__ void __launch_bounds__(kRsThreads) k_radix_scan(uint32_t* __restrict__ hist, int ntiles,
                                                            const uint32_t* __restrict__ totals) {
  __shared__ uint32_t buf[kRsThreads / 32];
  const int d = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t below = 0;
  for (int t = threadIdx.x; t < d; t += kRsThreads) below += totals[t];
  uint32_t run = block_sum_256(below, buf);
  uint32_t* row = hist + (size_t)d * ntiles;
  for (int seg = 0; seg < ntiles; seg += kRsThreads) {
    const int i = seg + threadIdx.x;
    const uint32_t c = i < ntiles ? row[i] : 0u;
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) buf[warp] = inc;
    __syncthreads();
    uint32_t before = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kRsThreads / 32; ++w) {
      const uint32_t bw = buf[w];
      before += w < warp ? bw : 0u;
      tot += bw;
    }
    if (i < ntiles) row[i] = run + before + inc - c;
    run += tot;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kRsThreads) k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                                               const uint32_t* __restrict__ vals_in, uint32_t n,
                                                               int shift, uint32_t mask,
                                                               const uint32_t* __restrict__ hist, int ntiles,
                                                               uint32_t* __restrict__ keys_out,
                                                               uint32_t* __restrict__ vals_out) {
  extern __shared__ uint32_t wcnt[];  // [kRsWarps][nbins]
  const int nbins = (int)mask + 1;
  for (int i = threadIdx.x; i < kRsWarps * nbins; i += kRsThreads) wcnt[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* mycnt = wcnt + warp * nbins;
  const uint32_t sub = blockIdx.x * (uint32_t)kRadixTile + warp * (kRsItems * 32);
  const unsigned lt = lanemask_lt();
  const uint32_t none = mask + 1;
  uint32_t key[kRsItems], val[kRsItems], off[kRsItems];
  uint32_t dig[kRsItems];
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const uint32_t i = sub + r * 32 + lane;
    const bool valid = i < n;
    const uint32_t k = valid ? keys_in[i] : 0u;
    const uint32_t v = valid ? (vals_in ? vals_in[i] : i) : 0u;
    const uint32_t d = valid ? ((k >> shift) & mask) : none;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (lane == leader && d < none) {
      old = mycnt[d];
      mycnt[d] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    off[r] = old + __popc(peers & lt);
    key[r] = k;
    val[r] = v;
    dig[r] = d;
    __syncwarp();
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nbins; d += kRsThreads) {
    uint32_t run = hist[(size_t)d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
      const uint32_t t = wcnt[w * nbins + d];
      wcnt[w * nbins + d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    if (dig[r] < none) {
      const uint32_t pos = mycnt[dig[r]] + off[r];
      if (keys_out) keys_out[pos] = key[r];
      vals_out[pos] = val[r];
    }
  }
}

}  // namespace

void radix_sort(const uint32_t* keys_in, uint32_t n, int passes, int digit_bits, uint32_t* keys0, uint32_t* keys1,
                uint32_t* vals0, uint32_t* vals1, uint32_t* hist, int ntiles, cudaStream_t s,
                const uint32_t** keys_sorted, const uint32_t** perm) {
  const uint32_t* kin = keys_in;
  const uint32_t* vin = nullptr;
  uint32_t* kbuf[2] = {keys0, keys1};
  uint32_t* vbuf[2] = {vals0, vals1};
  const int nbins = 1 << digit_bits;
  const uint32_t mask = (uint32_t)nbins - 1u;
  // digit totals of every pass live after the [nbins][ntiles] histogram table
  uint32_t* totals = hist + (size_t)nbins * ntiles;
  cudaMemsetAsync(totals, 0, sizeof(uint32_t) * nbins * passes, s);
  const size_t hist_smem = sizeof(uint32_t) * nbins;
  const size_t scat_smem = sizeof(uint32_t) * nbins * kRsWarps;
  if (scat_smem > 48 * 1024) {
    static bool raised = false;  // host attribute, once (before any graph capture of this path)
    if (!raised) {
      cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 * 4 * 2048);
      raised = true;
    }
  }
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = digit_bits * pass;
    uint32_t* tot = totals + nbins * pass;
    k_radix_hist<<<ntiles, kRsThreads, hist_smem, s>>>(kin, n, shift, mask, hist, ntiles, tot);
    k_radix_scan<<<nbins, kRsThreads, 0, s>>>(hist, ntiles, tot);
    k_radix_scatter<<<ntiles, kRsThreads, scat_smem, s>>>(kin, vin, n, shift, mask, hist, ntiles, kbuf[pass & 1],
                                                          vbuf[pass & 1]);
    kin = kbuf[pass & 1];
    vin = vbuf[pass & 1];
  }
  *keys_sorted = kin;
  *perm = vin;
}

}  // namespace ffmpm
