// ffmpm_sort_by_block_static: the block sort for callers that cannot allocate device memory.
//
// The scratch of the sort lives in one file-scope __device__ array of fixed size.  Host code
// never passes the array's name to a kernel (on the host it is only a stand-in symbol): on the
// first call in each CUDA context, with that context's device current, cudaGetSymbolAddress gives
// the array's device address, which is cached against the context's unique id and passed to the
// kernels.  A new context on the device (after cudaDeviceReset, or after the primary context was
// released and created again) loads the module again, so the address is looked up again.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"
#include "mpm_kernels.cuh"

namespace ffmpm {
namespace {

constexpr int64_t kStaticMaxN = FFMPM_STATIC_SORT_MAX_N;
constexpr int64_t kStaticTiles = (kStaticMaxN + kRadixTile - 1) / kRadixTile;
// [status word + pad: 64 words][keys_next][keys0][keys1][vals0][vals1][radix scratch of 4 passes:
// digit histograms, tile counters, look-back words 256 x tiles]
constexpr size_t kHeaderWords = 64;
constexpr size_t kRadixWords = size_t(kMaxRadixPasses) * (256 + 32 + 256 * size_t(kStaticTiles));
constexpr size_t kStaticWords = kHeaderWords + 5 * size_t(kStaticMaxN) + kRadixWords;

__device__ __align__(256) uint32_t g_sort_scratch[kStaticWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct CachedScratch {
  unsigned long long ctx_id;
  uint32_t* ptr;
};
CachedScratch g_scratch[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the current CUDA context (0 when there is none or the driver cannot tell).
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &ptr, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(ptr);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &ptr, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(ptr);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_sort_scratch in the current context (looked up once per context).
int scratch_on_current_device(uint32_t** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FFMPM_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  const unsigned long long id = current_context_id();
  CachedScratch& c = g_scratch[dev];
  if (!c.ptr || id == 0 || c.ctx_id != id) {
    void* p = nullptr;
    // also creates the device's primary context when the caller has not used the device yet
    if (cudaGetSymbolAddress(&p, g_sort_scratch) != cudaSuccess || !p) return FFMPM_ERR_CUDA;
    c.ptr = static_cast<uint32_t*>(p);
    c.ctx_id = current_context_id();
  }
  *out = c.ptr;
  return FFMPM_OK;
}

template <int DIM, typename T>
void sort_static(const ffmpm_params& p, const Layout& L, uint32_t* base, const void* x, uint32_t* keys_out,
                 uint32_t* perm_out, int32_t* status_out, cudaStream_t s) {
  KParams<T> kp{};
  kp.inv_dx = T(p.inv_dx);
  kp.res = p.res;
  Geom<DIM> g;
  g.res = L.res;
  g.R = L.R;
  g.bs = L.bs;
  g.bs_shift = __builtin_ctz((unsigned)L.bs);
  g.nb = L.nb;
  g.nblocks = (int)L.nblocks;
  g.tile = L.tile;
  const uint32_t n = (uint32_t)L.n;
  int32_t* status = reinterpret_cast<int32_t*>(base);
  uint32_t* keys_next = base + kHeaderWords;
  uint32_t* keys0 = keys_next + kStaticMaxN;
  uint32_t* keys1 = keys0 + kStaticMaxN;
  uint32_t* vals0 = keys1 + kStaticMaxN;
  uint32_t* vals1 = vals0 + kStaticMaxN;
  uint32_t* hist = vals1 + kStaticMaxN;
  // the array keeps the previous call's status word: start from zero
  cudaMemsetAsync(status, 0, sizeof(int32_t), s);
  PView<T> xv{};
  xv.x = static_cast<T*>(const_cast<void*>(x));
  k_keys<DIM, T><<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(kp, g, xv, n, L.cell_bits, keys_next, nullptr,
                                                                     status);
  const uint32_t *ks = nullptr, *perm = nullptr;
  radix_sort(keys_next, n, L.passes, keys0, keys1, vals0, vals1, hist, (int)L.ntiles, status, s, &ks, &perm, nullptr,
             p.wait_limit, p.inject);
  if (keys_out) cudaMemcpyAsync(keys_out, ks, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  if (perm_out) cudaMemcpyAsync(perm_out, perm, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  // the status word is only valid until the next call overwrites the array: hand it over now
  if (status_out) cudaMemcpyAsync(status_out, status, sizeof(int32_t), cudaMemcpyDefault, s);
}

}  // namespace
}  // namespace ffmpm

extern "C" int ffmpm_sort_by_block_static(const ffmpm_params* p, const void* x, int64_t n, uint32_t* keys_out,
                                          uint32_t* perm_out, int32_t* status_out, void* stream) {
  using namespace ffmpm;
  if (n > kStaticMaxN) return FFMPM_ERR_CAPACITY;
  Layout L;
  if (!p || !make_layout(*p, n, &L)) return FFMPM_ERR_BADARG;
  if (L.ntiles > kStaticTiles) return FFMPM_ERR_CAPACITY;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n == 0) {
    if (status_out) return cudaMemsetAsync(status_out, 0, sizeof(int32_t), s) == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
    return FFMPM_OK;
  }
  if (!x) return FFMPM_ERR_BADARG;
  uint32_t* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc != FFMPM_OK) return rc;
  if (p->dim == 3) {
    if (p->real_bytes == 4)
      sort_static<3, float>(*p, L, base, x, keys_out, perm_out, status_out, s);
    else
      sort_static<3, double>(*p, L, base, x, keys_out, perm_out, status_out, s);
  } else {
    if (p->real_bytes == 4)
      sort_static<2, float>(*p, L, base, x, keys_out, perm_out, status_out, s);
    else
      sort_static<2, double>(*p, L, base, x, keys_out, perm_out, status_out, s);
  }
  return cudaGetLastError() == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}
