// Stable LSD radix sort of 32-bit keys with a 32-bit permutation payload, 8-bit digits.
//
// One kernel counts the digits of every pass in a single read of the keys.  Each pass is then one
// kernel ("onesweep", Adinets & Merrill 2022): a CTA takes the next 4096-key tile (tile ids come
// from an atomic counter, so a tile's predecessors have always started), ranks its keys per warp
// with __match_any_sync in index order, publishes its per-digit counts, and obtains the counts of
// all earlier tiles by decoupled look-back: it walks back over its predecessors' published words
// until it meets one that already carries an inclusive prefix.  Every wait is bounded; a tile whose
// wait runs out skips its scatter and raises FFMPM_STATUS_TIMEOUT instead of hanging.  It still
// publishes the (partial, hence too small) prefix it has, so that its successors finish: their
// positions stay below the true ones and inside [0, n).  A pass that starts with the timeout bit
// already raised does nothing: its input keys were not all written by the previous pass, so their
// digits need not match the histogram the positions are built from.
//
// Stability makes the permutation bit-exact: it equals a CPU stable sort of the same keys (numpy
// argsort kind="stable").
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace ffmpm {

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsWarps = kRsThreads / 32;
static_assert(kRsThreads * kRsItems == kRadixTile, "tile size");

// Published look-back word: 2 flag bits over a 30-bit count (n < 2^30).
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagInclusive = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kLookbackSpins = 1u << 22;  // default bound of one tile's look-back wait
constexpr int kLookbackBatch = 8;  // predecessor words read per look-back step

// Digit histograms of all passes (ghist[pass][256]), one read of the keys.  Nearly sorted keys put
// equal digits in neighbouring lanes, so each warp first merges equal digits (__match_any_sync).
__global__ void __launch_bounds__(kRsThreads) k_radix_ghist(const uint32_t* __restrict__ keys, uint32_t n,
                                                             int passes, uint32_t* __restrict__ ghist,
                                                             const uint32_t* __restrict__ sort_flag) {
  if (sort_flag && *sort_flag == 0u) return;
  __shared__ uint32_t h[kMaxRadixPasses][256];
  for (int i = threadIdx.x; i < kMaxRadixPasses * 256; i += kRsThreads) (&h[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  // each CTA takes whole 4096-key tiles; a thread's 16 keys are loaded before any is counted
  for (uint32_t tile = blockIdx.x; tile * (uint32_t)kRadixTile < n; tile += gridDim.x) {
    const uint32_t base = tile * (uint32_t)kRadixTile + threadIdx.x;
    uint32_t k[kRsItems];
#pragma unroll
    for (int r = 0; r < kRsItems; ++r) {
      const uint32_t i = base + r * kRsThreads;
      k[r] = i < n ? __ldg(&keys[i]) : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int r = 0; r < kRsItems; ++r) {
      const bool valid = base + r * kRsThreads < n;
      for (int p = 0; p < passes; ++p) {
        const uint32_t d = valid ? ((k[r] >> (8 * p)) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (d < 256u && lane == __ffs(peers) - 1) atomicAdd(&h[p][d], (uint32_t)__popc(peers));
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += kRsThreads) {
    const uint32_t c = (&h[0][0])[i];
    if (c) atomicAdd(&ghist[i], c);
  }
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
  return *reinterpret_cast<const volatile uint32_t*>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *reinterpret_cast<volatile uint32_t*>(p) = v; }

__global__ void __launch_bounds__(kRsThreads) k_radix_onesweep(const uint32_t* __restrict__ keys_in,
                                                                const uint32_t* __restrict__ vals_in, uint32_t n,
                                                                int shift, const uint32_t* __restrict__ ghist,
                                                                uint32_t* __restrict__ lookback,
                                                                uint32_t* __restrict__ tile_counter,
                                                                uint32_t* __restrict__ keys_out,
                                                                uint32_t* __restrict__ vals_out, int32_t* status,
                                                                const uint32_t* __restrict__ sort_flag,
                                                                uint32_t wait_limit, uint32_t inject) {
  if (sort_flag && *sort_flag == 0u) return;
  // an earlier pass gave up: this pass's input is incomplete
  if (status && (*reinterpret_cast<const volatile int32_t*>(status) & FFMPM_STATUS_TIMEOUT)) return;
  __shared__ uint32_t wcnt[kRsWarps][256];
  __shared__ uint32_t base[256];
  __shared__ uint32_t warp_sums[kRsWarps];
  __shared__ uint32_t s_tile;
  __shared__ int s_timeout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcnt[0][0])[i] = 0;
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(tile_counter, 1u);
    s_timeout = 0;
  }
  // global start of every digit: exclusive scan of this pass's digit histogram
  {
    const uint32_t c = ghist[threadIdx.x];
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    uint32_t before = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) before += w < warp ? warp_sums[w] : 0u;
    base[threadIdx.x] = before + inc - c;
  }
  __syncthreads();
  const uint32_t tile = s_tile;
  // rank: warp w handles keys [tile*4096 + w*512, +512) in 16 rounds of 32, in index order
  const uint32_t sub = tile * (uint32_t)kRadixTile + warp * (kRsItems * 32);
  const unsigned lt = lanemask_lt();
  uint32_t key[kRsItems], val[kRsItems], off[kRsItems], dig[kRsItems];
  // all of this thread's keys and values are loaded before the ranking starts
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const uint32_t i = sub + r * 32 + lane;
    key[r] = i < n ? __ldg(&keys_in[i]) : 0u;
    val[r] = i < n ? (vals_in ? __ldg(&vals_in[i]) : i) : 0u;
  }
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const uint32_t i = sub + r * 32 + lane;
    const bool valid = i < n;
    const uint32_t k = key[r];
    const uint32_t v = val[r];
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
    // one thread per digit: per-warp exclusive offsets, the tile's count, then look-back
    const int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
      const uint32_t t = wcnt[w][d];
      wcnt[w][d] = run;
      run += t;
    }
    uint32_t* mine = lookback + (size_t)tile * 256 + d;
    uint32_t excl = 0;
    if (tile == 0) {
      // (fault injection for tests: the first tile never publishes, so every look-back that
      // reaches it can only end by running out)
      if (!(inject & FFMPM_INJECT_LOOKBACK_STALL)) st_volatile(mine, kFlagInclusive | run);
    } else {
      st_volatile(mine, kFlagAggregate | run);
      // walk back over the predecessors kLookbackBatch words at a time (the loads of a batch are
      // in flight together): add published aggregates in order, stop at the first inclusive
      // prefix, and re-read from the first word that is not published yet
      int t = (int)tile - 1;
      uint32_t spins = 0;
      while (t >= 0) {
        uint32_t w[kLookbackBatch];
#pragma unroll
        for (int j = 0; j < kLookbackBatch; ++j) w[j] = t - j >= 0 ? ld_volatile(lookback + (size_t)(t - j) * 256 + d) : 0u;
        int used = 0;
        bool found = false;
#pragma unroll
        for (int j = 0; j < kLookbackBatch; ++j) {
          if (found || used < j || t - j < 0) continue;
          if (w[j] & kFlagInclusive) {
            excl += w[j] & kValueMask;
            found = true;
          } else if (w[j] & kFlagAggregate) {
            excl += w[j] & kValueMask;
            ++used;
          }
        }
        if (found) break;
        t -= used;
        if (used == 0) {
          if (++spins > wait_limit) {
            s_timeout = 1;
            break;
          }
          __nanosleep(32);
        }
      }
      st_volatile(mine, kFlagInclusive | (excl + run));
    }
    base[d] += excl;
  }
  __syncthreads();
  if (s_timeout) {
    if (threadIdx.x == 0) raise_status(status, FFMPM_STATUS_TIMEOUT);
    return;  // positions unknown: write nothing
  }
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const uint32_t pos = base[dig[r] & 255u] + wcnt[warp][dig[r] & 255u] + off[r];
    if (dig[r] < 256u && pos < n) {
      if (keys_out) keys_out[pos] = key[r];
      vals_out[pos] = val[r];
    }
  }
}

}  // namespace

size_t radix_scratch_words(int passes, int64_t ntiles) {
  // per pass: 256-digit histogram, tile counter (padded to 32 words), look-back words [ntiles][256]
  return size_t(passes) * (256 + 32 + 256 * size_t(ntiles));
}

void radix_sort(const uint32_t* keys_in, uint32_t n, int passes, uint32_t* keys0, uint32_t* keys1, uint32_t* vals0,
                uint32_t* vals1, uint32_t* scratch, int ntiles, int32_t* status, cudaStream_t s,
                const uint32_t** keys_sorted, const uint32_t** perm, const uint32_t* sort_flag, uint32_t wait_limit,
                uint32_t inject) {
  if (wait_limit == 0) wait_limit = kLookbackSpins;
  uint32_t* ghist = scratch;                    // [passes][256]
  uint32_t* counters = ghist + 256 * passes;    // [passes], 32-word padded
  uint32_t* lookback = counters + 32 * passes;  // [passes][ntiles][256]
  cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * radix_scratch_words(passes, ntiles), s);
  const int ghist_grid = std::max(1, std::min(ntiles, 2 * sm_count()));
  k_radix_ghist<<<ghist_grid, kRsThreads, 0, s>>>(keys_in, n, passes, ghist, sort_flag);
  const uint32_t* kin = keys_in;
  const uint32_t* vin = nullptr;
  uint32_t* kbuf[2] = {keys0, keys1};
  uint32_t* vbuf[2] = {vals0, vals1};
  for (int pass = 0; pass < passes; ++pass) {
    k_radix_onesweep<<<ntiles, kRsThreads, 0, s>>>(kin, vin, n, 8 * pass, ghist + 256 * pass,
                                                   lookback + (size_t)pass * ntiles * 256, counters + 32 * pass,
                                                   kbuf[pass & 1], vbuf[pass & 1], status, sort_flag, wait_limit,
                                                   inject);
    kin = kbuf[pass & 1];
    vin = vbuf[pass & 1];
  }
  *keys_sorted = kin;
  *perm = vin;
}

}  // namespace ffmpm
