// Host-side internals shared by the translation units of libfemflow_mpm.so.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "femflow_mpm.h"

namespace ffmpm {

constexpr uint32_t kInvalidKey = 0xFFFFFFFFu;
constexpr int kChunk = 512;       // particles per P2G/G2P work item
constexpr int kRadixTile = 4096;  // keys per radix-sort CTA (256 threads x 16)

// Workspace header: status word, counters, polar fallbacks.
struct WsHeader {
  int32_t status;
  uint32_t polar_fallbacks;
  uint32_t n_chunks;
  uint32_t n_touched;
  uint32_t n_occupied;
  uint32_t n_valid;
  uint32_t sort_now;   // sort cadence: 1 when this substep re-sorts (set by k_sort_decide)
  uint32_t far_stray;  // set by G2P when a particle left the neighbourhood its block's plan covers
  uint32_t det_next[2];  // deterministic P2G: next entry of the occupied list, per pass (zeroed per launch)
  uint32_t pad[54];
};
static_assert(sizeof(WsHeader) == 256, "header is one 256-byte line");

// Offsets (bytes) of every region of a workspace, derived from (params, n).
struct Layout {
  int dim = 3, real_bytes = 4, res = 0, R = 0, bs = 0, nb = 0, tile = 0;
  int key_bits = 0, passes = 0, cell_bits = 0;
  int64_t n = 0, nblocks = 0, nnodes = 0, max_chunks = 0, ntiles = 0;
  size_t off_block_count = 0, off_block_start = 0, off_block_cnt = 0, off_chunks = 0, off_touched = 0, off_tmark = 0,
         off_occupied = 0, off_keys_next = 0, off_keys0 = 0, off_keys1 = 0, off_vals0 = 0, off_vals1 = 0,
         off_hist = 0, off_gridA = 0, off_gridB = 0, off_stage = 0, off_plan_pref = 0, off_plan_cta = 0, total = 0;
};

bool make_layout(const ffmpm_params& p, int64_t n, Layout* L);

int sm_count();

// Radix sort (sort.cu): stable, 8-bit digits, `passes` passes over keys_in (n keys); values start
// as the identity permutation.  `scratch` holds radix_scratch_words(passes, ntiles) words (zeroed
// by the call).  Returns the buffers that hold the sorted keys / permutation.  With `sort_flag`
// (device word, nullable) the kernels do nothing when it reads 0.  `wait_limit` bounds each tile's
// look-back wait (0: the default); `inject` takes FFMPM_INJECT_LOOKBACK_STALL (tests only).
constexpr int kMaxRadixPasses = 4;
size_t radix_scratch_words(int passes, int64_t ntiles);
void radix_sort(const uint32_t* keys_in, uint32_t n, int passes, uint32_t* keys0, uint32_t* keys1, uint32_t* vals0,
                uint32_t* vals1, uint32_t* scratch, int ntiles, int32_t* status, cudaStream_t s,
                const uint32_t** keys_sorted, const uint32_t** perm, const uint32_t* sort_flag = nullptr,
                uint32_t wait_limit = 0, uint32_t inject = 0);

}  // namespace ffmpm
