// extern "C" entry points of libfemflow_mpm.so (declared in include/femflow_mpm.h) and the host
// code that sequences the kernels of a substep on the caller's stream.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "mpm_kernels.cuh"

namespace ffmpm {

namespace {

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// The Python mirror (_native.Params / Particles, ctypes) relies on these layouts; its test checks
// the same sizes.
static_assert(sizeof(ffmpm_params) == 504, "ffmpm_params layout");
static_assert(sizeof(ffmpm_particles) == 80, "ffmpm_particles layout");

int ilog2_ceil(int64_t v) {
  int b = 0;
  while ((int64_t(1) << b) < v) ++b;
  return b;
}

int default_block_size(int dim, bool det) {
  if (dim == 3) return det ? 4 : 8;
  return det ? 8 : 16;
}

bool valid_params(const ffmpm_params* p) {
  if (!p) return false;
  if (p->dim != 2 && p->dim != 3) return false;
  if (p->real_bytes != 4 && p->real_bytes != 8) return false;
  if (p->res < 3 || p->res > 4096) return false;
  if (p->model != FFMPM_MODEL_NEO_HOOKEAN && p->model != FFMPM_MODEL_SNOW && p->model != FFMPM_MODEL_FIXED_COROTATED)
    return false;
  if (p->wall_mode != FFMPM_WALLS_REFERENCE && p->wall_mode != FFMPM_WALLS_STICKY3) return false;
  if (p->block_size != 0 && (p->block_size < 2 || p->block_size > 16 || (p->block_size & (p->block_size - 1))))
    return false;
  if (p->n_planes < 0 || p->n_planes > FFMPM_MAX_PLANES) return false;
  if (p->plane_rule != FFMPM_PLANES_STICKY && p->plane_rule != FFMPM_PLANES_REFERENCE_LITERAL) return false;
  for (int q = 0; q < p->n_planes; ++q) {
    double ss = 0.0;
    for (int d = 0; d < 6; ++d)
      if (!std::isfinite(p->planes[q][d])) return false;
    for (int d = 0; d < p->dim; ++d) ss += p->planes[q][3 + d] * p->planes[q][3 + d];
    if (!(ss > 0.0)) return false;
  }
  return true;
}

}  // namespace

bool make_layout(const ffmpm_params& p, int64_t n, Layout* L) {
  // below 2^30 particles: the radix sort's look-back words carry 30-bit counts
  if (!valid_params(&p) || n < 0 || n >= (int64_t(1) << 30)) return false;
  L->dim = p.dim;
  L->real_bytes = p.real_bytes;
  L->res = p.res;
  L->R = p.res + 1;
  L->bs = p.block_size ? p.block_size : default_block_size(p.dim, p.deterministic != 0);
  L->nb = (L->R + L->bs - 1) / L->bs;
  L->tile = L->bs + 2;
  L->nblocks = p.dim == 3 ? int64_t(L->nb) * L->nb * L->nb : int64_t(L->nb) * L->nb;
  L->nnodes = p.dim == 3 ? int64_t(L->R) * L->R * L->R : int64_t(L->R) * L->R;
  // keys order particles by block, then by cell inside the block, so that each P2G chunk spans few
  // cells (between re-sorts the P2G regroups each chunk by cell itself)
  L->cell_bits = p.dim * ilog2_ceil(L->bs);
  L->key_bits = ilog2_ceil(L->nblocks) + L->cell_bits;
  if (L->key_bits > 31) return false;
  L->passes = std::max(1, (L->key_bits + 7) / 8);
  if (L->passes > kMaxRadixPasses) return false;
  L->n = n;
  L->ntiles = std::max<int64_t>(1, (n + kRadixTile - 1) / kRadixTile);
  L->max_chunks = (n + kChunk - 1) / kChunk + L->nblocks;
  const size_t node_bytes = size_t(4) * p.real_bytes;
  const int64_t tile_nodes = p.dim == 3 ? int64_t(L->tile) * L->tile * L->tile : int64_t(L->tile) * L->tile;
  size_t off = sizeof(WsHeader);
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  L->off_block_count = take(sizeof(uint32_t) * L->nblocks);
  L->off_block_start = take(sizeof(uint32_t) * L->nblocks);
  L->off_block_cnt = take(sizeof(uint32_t) * L->nblocks);
  L->off_chunks = take(sizeof(int4) * L->max_chunks);
  L->off_touched = take(sizeof(uint32_t) * L->nblocks);
  L->off_tmark = take(sizeof(uint32_t) * L->nblocks);
  L->off_occupied = take(sizeof(int4) * L->nblocks);
  L->off_keys_next = take(sizeof(uint32_t) * std::max<int64_t>(n, 1));
  L->off_keys0 = take(sizeof(uint32_t) * std::max<int64_t>(n, 1));
  L->off_keys1 = take(sizeof(uint32_t) * std::max<int64_t>(n, 1));
  L->off_vals0 = take(sizeof(uint32_t) * std::max<int64_t>(n, 1));
  L->off_vals1 = take(sizeof(uint32_t) * std::max<int64_t>(n, 1));
  L->off_hist = take(sizeof(uint32_t) * radix_scratch_words(L->passes, L->ntiles));
  L->off_gridA = take(node_bytes * L->nnodes);
  L->off_gridB = take(node_bytes * L->nnodes);
  L->off_stage = take(p.deterministic ? node_bytes * tile_nodes * L->nblocks : 0);
  // the plan kernels' per-block prefixes (3 x nblocks) and per-CTA totals and offsets
  L->off_plan_pref = take(sizeof(uint32_t) * 3 * L->nblocks);
  L->off_plan_cta = take(2 * 16 * ((L->nblocks + kPlanCta - 1) / kPlanCta));
  L->total = off;
  return true;
}

int sm_count() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached = v > 0 ? v : 148;
  }
  return cached;
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

// Tensor map of a dense grid of Node4 records: dims (4 components, R, R[, R]) innermost first.
bool encode_grid_map(CUtensorMap* map, void* base, const Layout& L) {
  auto fn = encode_fn();
  if (!fn) return false;
  const CUtensorMapDataType dt = L.real_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const cuuint64_t eb = L.real_bytes;
  cuuint64_t dims[4] = {4, (cuuint64_t)L.R, (cuuint64_t)L.R, (cuuint64_t)L.R};
  cuuint64_t strides[3] = {4 * eb, 4 * eb * L.R, 4 * eb * L.R * L.R};  // bytes, dims 1..rank-1
  cuuint32_t box[4] = {4, (cuuint32_t)L.tile, (cuuint32_t)L.tile, (cuuint32_t)L.tile};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  const cuuint32_t rank = L.dim == 3 ? 4 : 3;
  CUresult r = fn(map, dt, rank, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int DIM>
Geom<DIM> geom(const Layout& L) {
  Geom<DIM> g;
  g.res = L.res;
  g.R = L.R;
  g.bs = L.bs;
  g.bs_shift = __builtin_ctz((unsigned)L.bs);
  g.nb = L.nb;
  g.nblocks = (int)L.nblocks;
  g.tile = L.tile;
  return g;
}

struct Ws {
  unsigned char* base;
  WsHeader* hdr;
  uint32_t *block_count, *block_start, *block_cnt, *touched, *tmark, *keys_next, *keys0, *keys1, *vals0, *vals1, *hist;
  int4 *chunks, *occupied;
  void *gridA, *gridB, *stage;
  uint32_t* plan_pref;
  Scan4 *cta_tot, *cta_off;
};

Ws bind(void* ws, const Layout& L) {
  Ws w;
  w.base = static_cast<unsigned char*>(ws);
  w.hdr = reinterpret_cast<WsHeader*>(w.base);
  w.block_count = reinterpret_cast<uint32_t*>(w.base + L.off_block_count);
  w.block_start = reinterpret_cast<uint32_t*>(w.base + L.off_block_start);
  w.block_cnt = reinterpret_cast<uint32_t*>(w.base + L.off_block_cnt);
  w.chunks = reinterpret_cast<int4*>(w.base + L.off_chunks);
  w.touched = reinterpret_cast<uint32_t*>(w.base + L.off_touched);
  w.tmark = reinterpret_cast<uint32_t*>(w.base + L.off_tmark);
  w.occupied = reinterpret_cast<int4*>(w.base + L.off_occupied);
  w.keys_next = reinterpret_cast<uint32_t*>(w.base + L.off_keys_next);
  w.keys0 = reinterpret_cast<uint32_t*>(w.base + L.off_keys0);
  w.keys1 = reinterpret_cast<uint32_t*>(w.base + L.off_keys1);
  w.vals0 = reinterpret_cast<uint32_t*>(w.base + L.off_vals0);
  w.vals1 = reinterpret_cast<uint32_t*>(w.base + L.off_vals1);
  w.hist = reinterpret_cast<uint32_t*>(w.base + L.off_hist);
  w.gridA = w.base + L.off_gridA;
  w.gridB = w.base + L.off_gridB;
  w.stage = w.base + L.off_stage;
  w.plan_pref = reinterpret_cast<uint32_t*>(w.base + L.off_plan_pref);
  w.cta_tot = reinterpret_cast<Scan4*>(w.base + L.off_plan_cta);
  w.cta_off = w.cta_tot + (L.nblocks + kPlanCta - 1) / kPlanCta;
  return w;
}

int check_launch() {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FFMPM_OK : FFMPM_ERR_CUDA;
}

int work_grid(int64_t max_items, int per_sm) {
  const int64_t cap = int64_t(sm_count()) * per_sm;
  return (int)std::max<int64_t>(1, std::min<int64_t>(max_items, cap));
}

// Resident CTAs per SM of `kernel` at kThreads threads and `smem` dynamic bytes (cached), so the
// chunk-loop kernels launch exactly one wave.
template <typename F>
int resident_per_sm(F* kernel, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<const void*, size_t>, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(reinterpret_cast<const void*>(kernel), smem);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kThreads, smem) != cudaSuccess || nb < 1) nb = 1;
  cache[key] = nb;
  return nb;
}

// Optional per-phase CUDA-event timer of the profiling entry point.
struct PhaseTimer {
  std::vector<cudaEvent_t> ev;     // pairs (start, stop)
  std::vector<int> phase;
  std::vector<int> launches;
  cudaStream_t s = nullptr;
  void begin(int ph) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    ev.push_back(e0);
    ev.push_back(e1);
    phase.push_back(ph);
  }
  void end(int nlaunch) {
    cudaEventRecord(ev.back(), s);
    launches.push_back(nlaunch);
  }
  void collect(double* ms, int64_t* cnt) {
    cudaStreamSynchronize(s);
    for (size_t i = 0; i < phase.size(); ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]);
      ms[phase[i]] += t;
      cnt[phase[i]] += launches[i];
    }
    for (auto e : ev) cudaEventDestroy(e);
    ev.clear();
  }
};

// Substeps between re-sorts (ffmpm_params.variant bits 8..15; 0 or 1: every substep).  The
// deterministic mode always re-sorts (the CTA that sums a block needs every particle in that block).
int sort_every(const ffmpm_params& p) {
  const int k = (p.variant >> kVariantSortShift) & 0xFF;
  return (p.deterministic || k < 1) ? 1 : k;
}

// Start of a substep of a cadenced run: re-sort when the cadence says so or when the previous
// G2P saw a particle leave the neighbourhood its block's plan covers.
__global__ void k_sort_decide(WsHeader* h, int periodic) {
  h->sort_now = (periodic || h->far_stray) ? 1u : 0u;
  h->far_stray = 0u;
}

// keys -> sort -> plan.  Leaves the permutation pointer in *perm.  With `flag` (cadenced runs) the
// sort and the plan do their work only when the device word reads 1.  With `sym` (default: with a
// flag) the plan dilates the occupied blocks by +-1 so that it stays valid until the next re-sort.
template <int DIM, typename T>
void sort_and_plan(const ffmpm_params& p, const Layout& L, const Ws& w, const PView<T>& x, bool keys_ready,
                   const uint32_t** perm, cudaStream_t s, PhaseTimer* tm = nullptr, const uint32_t* flag = nullptr,
                   int sym = -1) {
  const KParams<T> kp = kparams<T>(p);
  const Geom<DIM> g = geom<DIM>(L);
  const uint32_t n = (uint32_t)L.n;
  if (!keys_ready) {
    if (tm) tm->begin(0);
    k_keys<DIM, T><<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(kp, g, x, n, L.cell_bits, w.keys_next,
                                                                       w.block_count, &w.hdr->status);
    if (tm) tm->end(1);
  }
  const uint32_t* ks = nullptr;
  if (tm) tm->begin(1);
  radix_sort(w.keys_next, n, L.passes, w.keys0, w.keys1, w.vals0, w.vals1, w.hist, (int)L.ntiles, &w.hdr->status, s,
             &ks, perm, flag, p.wait_limit, p.inject);
  if (tm) tm->end(1 + L.passes);
  if (tm) tm->begin(2);
  const int ncta = (int)((L.nblocks + kPlanCta - 1) / kPlanCta);
  k_plan_local<DIM><<<ncta, kPlanCta, 0, s>>>(g, w.block_count, w.block_start, w.block_cnt, w.tmark, w.plan_pref,
                                              w.cta_tot, flag, sym >= 0 ? sym : (flag ? 1 : 0));
  k_plan_offsets<<<1, kPlanCta, 0, s>>>(w.cta_tot, w.cta_off, ncta, w.hdr, flag);
  k_plan_write<DIM><<<ncta, kPlanCta, 0, s>>>(g, w.block_count, w.block_start, w.block_cnt, w.tmark, w.plan_pref,
                                              w.cta_off, w.chunks, w.touched, w.occupied, flag);
  if (tm) tm->end(3);
}

template <int DIM, typename T>
size_t tile_smem(const Layout& L) {
  const int64_t tn = DIM == 3 ? int64_t(L.tile) * L.tile * L.tile : int64_t(L.tile) * L.tile;
  return size_t(tn) * 4 * sizeof(T);
}

// Dynamic shared memory every kernel may use (set_smem raises each kernel's limit to it).
constexpr size_t kMaxDynSmem = 200 * 1024;

// Dynamic shared memory of the cell-run P2G and of the fused G2P + P2G for this layout.
size_t cells_smem_bytes(const Layout& L) {
  if (L.real_bytes == 4)
    return L.dim == 3 ? tile_smem<3, float>(L) + cell_run_smem_bytes<3, float>(L.bs)
                      : tile_smem<2, float>(L) + cell_run_smem_bytes<2, float>(L.bs);
  return L.dim == 3 ? tile_smem<3, double>(L) + cell_run_smem_bytes<3, double>(L.bs)
                    : tile_smem<2, double>(L) + cell_run_smem_bytes<2, double>(L.bs);
}

size_t fused_smem_bytes(const Layout& L) {
  const int tn = L.dim == 3 ? L.tile * L.tile * L.tile : L.tile * L.tile;
  if (L.real_bytes == 4)
    return L.dim == 3 ? g2p2g_smem_bytes<3, float>(tn, L.bs) : g2p2g_smem_bytes<2, float>(tn, L.bs);
  return L.dim == 3 ? g2p2g_smem_bytes<3, double>(tn, L.bs) : g2p2g_smem_bytes<2, double>(tn, L.bs);
}

// Raise a kernel's dynamic shared-memory limit once per kernel (a host-side attribute call,
// kept out of CUDA-graph captures, which run after the first direct call).
template <typename F>
void set_smem(F* kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return;
  static std::mutex mu;
  static std::set<const void*> done;
  std::lock_guard<std::mutex> lock(mu);
  if (done.insert(reinterpret_cast<const void*>(kernel)).second)
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDynSmem);
}

template <int DIM, typename T, typename Sink>
void launch_p2g(const ffmpm_params& p, const Layout& L, const Ws& w, const PView<T>& P, const uint32_t* perm,
                const Sink& sink, cudaStream_t s, const uint32_t* flag = nullptr) {
  // plans kept over several substeps need the stray path of the cell-run kernel
  const bool direct = !flag && (p.variant & kVariantP2GDirect) != 0;
  const bool lanes = !flag && (p.variant & kVariantP2GLanes) != 0;
  if (!direct && !lanes) {
    // default: cell-run P2G (tile + per-particle records + cell ids + run starts)
    const size_t smem = tile_smem<DIM, T>(L) + cell_run_smem_bytes<DIM, T>(L.bs);
    auto kern = k_p2g_cells<DIM, T, Sink>;
    set_smem(kern, smem);
    kern<<<work_grid(L.max_chunks, resident_per_sm(kern, smem)), kThreads, smem, s>>>(
        kparams<T>(p), geom<DIM>(L), P, perm, w.chunks, w.hdr, sink, &w.hdr->status, &w.hdr->polar_fallbacks, flag);
    return;
  }
  const size_t smem = direct ? 0 : tile_smem<DIM, T>(L);
  auto kern = direct ? k_p2g<DIM, T, Sink, true> : k_p2g<DIM, T, Sink, false>;
  set_smem(kern, smem);
  kern<<<work_grid(L.max_chunks, resident_per_sm(kern, smem)), kThreads, smem, s>>>(
      kparams<T>(p), geom<DIM>(L), P, perm, w.chunks, w.hdr, sink, &w.hdr->status, &w.hdr->polar_fallbacks);
}

template <int DIM, typename T>
void launch_p2g_det(const ffmpm_params& p, const Layout& L, const Ws& w, const PView<T>& P, const uint32_t* perm,
                    cudaStream_t s) {
  const int tn = DIM == 3 ? L.tile * L.tile * L.tile : L.tile * L.tile;
  const size_t smem = p2g_det_smem_bytes<DIM, T>(tn);
  auto kern = k_p2g_det<DIM, T>;
  set_smem(kern, smem);
  cudaMemsetAsync(w.hdr->det_next, 0, sizeof(w.hdr->det_next), s);  // the CTAs' shared work counters
  kern<<<work_grid(L.nblocks, resident_per_sm(kern, smem)), kThreads, smem, s>>>(
      kparams<T>(p), geom<DIM>(L), P, perm, w.occupied, w.hdr, static_cast<Node4<T>*>(w.stage), &w.hdr->status,
      &w.hdr->polar_fallbacks, w.hdr->det_next);
}

template <int DIM, typename T>
void launch_grid_update_det(const ffmpm_params& p, const Layout& L, const Ws& w, cudaStream_t s, T* user_gv = nullptr,
                            T* user_gm = nullptr) {
  k_grid_update_det<DIM, T><<<work_grid(L.nblocks, 8), kThreads, 0, s>>>(
      kparams<T>(p), geom<DIM>(L), w.touched, w.block_cnt, w.hdr, static_cast<const Node4<T>*>(w.stage),
      static_cast<Node4<T>*>(w.gridB), user_gv, user_gm);
}

template <int DIM, typename T>
void launch_grid_update(const ffmpm_params& p, const Layout& L, const Ws& w, cudaStream_t s) {
  k_grid_update<DIM, T><<<work_grid(L.nblocks, 8), kThreads, 0, s>>>(
      kparams<T>(p), geom<DIM>(L), w.touched, w.hdr, static_cast<Node4<T>*>(w.gridA), static_cast<Node4<T>*>(w.gridB));
}

template <int DIM, typename T, bool kTma, bool kSorted>
int launch_g2p(const ffmpm_params& p, const Layout& L, const Ws& w, const PView<T>& Pin, const PView<T>& Pout,
               const uint32_t* perm, const T* user_gv, const G2PExtra& ex, cudaStream_t s,
               const uint32_t* flag = nullptr) {
  alignas(64) CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  if (kTma && !encode_grid_map(&map, w.gridB, L)) return FFMPM_ERR_CUDA;
  const size_t smem = tile_smem<DIM, T>(L) + 128 + 16;  // + alignment pad + mbarrier
  auto kern = k_g2p<DIM, T, kTma, kSorted>;
  set_smem(kern, smem);
  kern<<<work_grid(L.max_chunks, resident_per_sm(kern, smem)), kThreads, smem, s>>>(
      kparams<T>(p), geom<DIM>(L), Pin, Pout, perm, w.chunks, w.hdr, map, user_gv, ex, &w.hdr->status, flag);
  return FFMPM_OK;
}

template <int DIM, typename T>
int launch_g2p2g(const ffmpm_params& p, const Layout& L, const Ws& w, const PView<T>& Pin, const PView<T>& Pout,
                 const uint32_t* perm, const G2PExtra& ex, cudaStream_t s, const uint32_t* flag) {
  alignas(64) CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  if (!encode_grid_map(&map, w.gridB, L)) return FFMPM_ERR_CUDA;
  const int tn = DIM == 3 ? L.tile * L.tile * L.tile : L.tile * L.tile;
  const size_t smem = g2p2g_smem_bytes<DIM, T>(tn, L.bs);
  auto kern = k_g2p2g<DIM, T>;
  set_smem(kern, smem);
  kern<<<work_grid(L.max_chunks, resident_per_sm(kern, smem)), kThreads, smem, s>>>(
      kparams<T>(p), geom<DIM>(L), Pin, Pout, perm, w.chunks, w.hdr, map, ex,
      InternalSink<T>{static_cast<Node4<T>*>(w.gridA)}, w.tmark, w.touched, &w.hdr->status, &w.hdr->polar_fallbacks,
      flag);
  return FFMPM_OK;
}

// Fused G2P + P2G in the sorted solver: the default outside the deterministic mode and the P2G
// variants, for runs of two or more substeps whose two tiles and records fit in shared memory.
bool fused(const ffmpm_params& p, const Layout& L, int nsteps) {
  return !p.deterministic && nsteps >= 2 &&
         (p.variant & (kVariantNoFuse | kVariantP2GDirect | kVariantP2GLanes)) == 0 &&
         fused_smem_bytes(L) <= kMaxDynSmem;
}

// ------------------------------------------------------------------------------------ operations
template <int DIM, typename T>
int op_substep(const ffmpm_params& p, const Layout& L, const Ws& w, ffmpm_particles* P, cudaStream_t s) {
  const PView<T> pv = pview<T>(*P);
  const uint32_t* perm = nullptr;
  sort_and_plan<DIM, T>(p, L, w, pv, false, &perm, s);
  if (p.deterministic) {
    launch_p2g_det<DIM, T>(p, L, w, pv, perm, s);
    launch_grid_update_det<DIM, T>(p, L, w, s);
  } else {
    launch_p2g<DIM, T>(p, L, w, pv, perm, InternalSink<T>{static_cast<Node4<T>*>(w.gridA)}, s);
    launch_grid_update<DIM, T>(p, L, w, s);
  }
  G2PExtra ex{};
  int rc = launch_g2p<DIM, T, true, false>(p, L, w, pv, pv, perm, nullptr, ex, s);
  return rc != FFMPM_OK ? rc : check_launch();
}

// ----------------------------------------------------------------------------- host-array substep
// Copy streams and events of ffmpm_substep_host, one set per device, created by the first call on
// that device (with it current) and kept until the process exits.
constexpr int kHostChunks = 4;
struct HostPipe {
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t start = nullptr, gathered_all = nullptr, down_done = nullptr;
  cudaEvent_t landed[kHostChunks] = {}, gathered[kHostChunks] = {};
};

int host_pipe(HostPipe** out) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static HostPipe pipes[kMaxDevices];
  static bool made[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FFMPM_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  HostPipe& h = pipes[dev];
  if (!made[dev]) {
    bool ok = cudaStreamCreateWithFlags(&h.up, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&h.down, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&h.start, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&h.gathered_all, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&h.down_done, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; ok && k < kHostChunks; ++k)
      ok = cudaEventCreateWithFlags(&h.landed[k], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&h.gathered[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) return FFMPM_ERR_CUDA;
    made[dev] = true;
  }
  *out = &h;
  return FFMPM_OK;
}

// One substep on host arrays H through the device arrays D (same shapes, row-major).  Chunk k of
// every input array goes up on the upload stream and is scattered on `s` once it has landed; after
// the dense grid update, chunk k is gathered on `s` and its outputs go down on the download stream
// while chunk k + 1 is gathered.  `s` finally waits for the last download, so that the call is
// complete, host arrays included, once `s` has run.  (Kernels reading and writing mapped pinned
// host memory in place measured about 4x slower than this on a GB300: the copy engines, not SM
// loads and stores, reach the host link's rate here.)
template <int DIM, typename T>
int op_substep_host(const ffmpm_params& p, const Layout& L, const Ws& w, const ffmpm_particles* H,
                    ffmpm_particles* D, cudaStream_t s) {
  const int64_t n = H->n;
  HostPipe* hp = nullptr;
  int rc = host_pipe(&hp);
  if (rc != FFMPM_OK) return rc;
  const size_t rb = sizeof(T);
  struct Arr {
    void* h;
    void* d;
    size_t per;   // bytes per particle
    bool in;      // read by the substep
    bool out;     // written by the substep
    bool whole;   // one real per particle: sent up whole before the first chunk (fewer, larger copies)
  };
  // Jp is read and changed only in 2D and for snow (two_d/g2p.py:44-46, three_d/p2g.py:57-61,
  // three_d/g2p.py:48-58): elsewhere it is neither sent up nor sent back
  const bool jp_used = DIM == 2 || p.model == FFMPM_MODEL_SNOW;
  const Arr arrs[8] = {{H->x, D->x, DIM * rb, true, true, false},
                       {H->v, D->v, DIM * rb, true, true, false},
                       {H->F, D->F, DIM * DIM * rb, true, true, false},
                       {H->C, D->C, DIM * DIM * rb, true, true, false},
                       {H->Jp, D->Jp, rb, jp_used, jp_used, true},
                       {const_cast<void*>(H->mass), const_cast<void*>(D->mass), rb, true, false, true},
                       {const_cast<void*>(H->mu_0), const_cast<void*>(D->mu_0), rb, true, false, true},
                       {const_cast<void*>(H->lambda_0), const_cast<void*>(D->lambda_0), rb, true, false, true}};
  // copies of [a, b) of the chunked arrays (whole = false: the per-particle scalars over [0, n))
  auto copy = [&](bool down, int64_t a, int64_t b, cudaStream_t cs, bool whole = false) {
    for (const Arr& r : arrs) {
      if (!r.h || (down && !r.out) || (!down && (!r.in || r.whole != whole))) continue;
      unsigned char* hb = static_cast<unsigned char*>(r.h) + a * r.per;
      unsigned char* db = static_cast<unsigned char*>(r.d) + a * r.per;
      if (down)
        cudaMemcpyAsync(hb, db, (b - a) * r.per, cudaMemcpyDeviceToHost, cs);
      else
        cudaMemcpyAsync(db, hb, (b - a) * r.per, cudaMemcpyHostToDevice, cs);
    }
  };
  // the uploads start after the work already queued on the caller's stream
  cudaEventRecord(hp->start, s);
  cudaStreamWaitEvent(hp->up, hp->start, 0);
  if (p.deterministic) {
    // the fixed summation order needs the block-sorted path: whole arrays up, ffmpm_substep, down
    copy(false, 0, n, hp->up, true);
    copy(false, 0, n, hp->up);
    cudaEventRecord(hp->landed[0], hp->up);
    cudaStreamWaitEvent(s, hp->landed[0], 0);
    rc = op_substep<DIM, T>(p, L, w, D, s);
    if (rc != FFMPM_OK) return rc;
    copy(true, 0, n, s);
    return check_launch();
  }
  // Upload chunks shrink (sizes K, K-1, ..., 1) so that little scatter is left once the last one
  // has landed; gather/download chunks grow (1, 2, ..., K) so that the first download starts soon
  // after the grid update.
  const int K = (int)std::max<int64_t>(1, std::min<int64_t>(kHostChunks, (n + 65535) / 65536));
  const int64_t parts = int64_t(K) * (K + 1) / 2;
  auto up_lo = [&](int k) { return n * (int64_t(k) * (2 * K - k + 1) / 2) / parts; };
  auto lo = [&](int k) { return n * (int64_t(k) * (k + 1) / 2) / parts; };
  const KParams<T> kp = kparams<T>(p);
  const Geom<DIM> g = geom<DIM>(L);
  const PView<T> pv = pview<T>(*D);
  const InternalSink<T> sink{static_cast<Node4<T>*>(w.gridA)};
  copy(false, 0, n, hp->up, true);
  for (int k = 0; k < K; ++k) {
    const int64_t a = up_lo(k), b = up_lo(k + 1);
    copy(false, a, b, hp->up);
    cudaEventRecord(hp->landed[k], hp->up);
    cudaStreamWaitEvent(s, hp->landed[k], 0);
    k_p2g_range<DIM, T><<<work_grid((b - a + kThreads - 1) / kThreads, 8), kThreads, 0, s>>>(
        kp, g, pv, (uint32_t)a, (uint32_t)b, sink, &w.hdr->status, &w.hdr->polar_fallbacks);
  }
  k_grid_update_dense<DIM, T><<<work_grid((L.nnodes + kThreads - 1) / kThreads, 8), kThreads, 0, s>>>(
      kp, g, static_cast<Node4<T>*>(w.gridA), static_cast<Node4<T>*>(w.gridB));
  for (int k = 0; k < K; ++k) {
    const int64_t a = lo(k), b = lo(k + 1);
    k_g2p_range<DIM, T><<<work_grid((b - a + kThreads - 1) / kThreads, 8), kThreads, 0, s>>>(
        kp, g, pv, (uint32_t)a, (uint32_t)b, static_cast<const Node4<T>*>(w.gridB), &w.hdr->status);
    cudaEventRecord(hp->gathered[k], s);
    cudaStreamWaitEvent(hp->down, hp->gathered[k], 0);
    copy(true, a, b, hp->down);
  }
  cudaEventRecord(hp->down_done, hp->down);
  cudaStreamWaitEvent(s, hp->down_done, 0);
  return check_launch();
}

// Per-substep copies of the positions and ids (ffmpm_substeps_sorted_snapshots): after substep k
// the output buffer's x (dim components of n reals, in its sorted order) goes to x + k dim n and
// its ids to ids + k n, on the run's stream.
struct SnapOut {
  void* x;
  int32_t* ids;
};

template <int DIM, typename T>
void snapshot(const SnapOut* snap, int k, const PView<T>& out, const int32_t* ids_out, int64_t n, cudaStream_t s) {
  if (!snap) return;
  T* dst = static_cast<T*>(snap->x) + (size_t)k * DIM * n;
  if (out.soa == n) {
    cudaMemcpyAsync(dst, out.x, sizeof(T) * DIM * n, cudaMemcpyDeviceToDevice, s);
  } else {
    for (int d = 0; d < DIM; ++d)
      cudaMemcpyAsync(dst + (size_t)d * n, out.x + (size_t)d * out.soa, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
  }
  cudaMemcpyAsync(snap->ids + (size_t)k * n, ids_out, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s);
}

// Substeps 0..n-1 with the fused kernel: P2G(0), then for k = 0..n-2: grid update(k), re-sort if
// due (k a multiple of the cadence), G2P(k) + P2G(k+1); then grid update(n-1) and G2P(n-1).  The
// state after every substep is in buffer a or b as in the unfused loop (x, F, Jp, ids, per-particle
// material), with v and C written by the last G2P only.  The grid update of substep k runs before
// the re-sort, on the touched blocks of the plan its P2G scattered under.  The re-sorts are
// scheduled on the host: the fused kernel adds the blocks a fast particle reaches to the touched
// list itself, so correctness does not wait for a re-sort, and substeps without one launch no
// sort or plan kernel at all.  Keys and the block histogram are written only by the fused launch
// that precedes a re-sort.
template <int DIM, typename T>
int op_substeps_fused(const ffmpm_params& p, const Layout& L, const Ws& w, PView<T> va, PView<T> vb, int32_t* ids_a,
                      int32_t* ids_b, int nsteps, cudaStream_t s, PhaseTimer* tm, const SnapOut* snap) {
  const int K = sort_every(p);
  const auto resorts = [&](int k) { return k >= 1 && k <= nsteps - 2 && k % K == 0; };
  const uint32_t* sorted_perm = nullptr;
  sort_and_plan<DIM, T>(p, L, w, va, false, &sorted_perm, s, tm, nullptr, 1);
  const uint32_t* perm = sorted_perm;  // the permutation the next P2G / G2P applies (null: none)
  if (tm) tm->begin(3);
  launch_p2g<DIM, T>(p, L, w, va, perm, InternalSink<T>{static_cast<Node4<T>*>(w.gridA)}, s);
  if (tm) tm->end(1);
  for (int k = 0; k < nsteps; ++k) {
    const PView<T>& in = (k & 1) ? vb : va;
    const PView<T>& out = (k & 1) ? va : vb;
    const int32_t* ids_in = (k & 1) ? ids_b : ids_a;
    int32_t* ids_out = (k & 1) ? ids_a : ids_b;
    if (tm) tm->begin(4);
    launch_grid_update<DIM, T>(p, L, w, s);
    if (tm) tm->end(1);
    if (k == nsteps - 1) {
      // k >= 1: the buffer is already in the order of the current plan
      G2PExtra ex{ids_in, ids_out, nullptr, nullptr, L.cell_bits, w.gridB, nullptr};
      if (tm) tm->begin(5);
      const int rc = launch_g2p<DIM, T, true, true>(p, L, w, in, out, nullptr, nullptr, ex, s);
      if (tm) tm->end(1);
      if (rc != FFMPM_OK) return rc;
      snapshot<DIM, T>(snap, k, out, ids_out, L.n, s);
      break;
    }
    if (k > 0) perm = nullptr;
    if (resorts(k)) sort_and_plan<DIM, T>(p, L, w, in, true, &perm, s, tm, nullptr, 1);
    const bool keys = resorts(k + 1);
    G2PExtra ex{ids_in, ids_out, keys ? w.keys_next : nullptr, keys ? w.block_count : nullptr, L.cell_bits, w.gridB,
                nullptr};
    if (tm) tm->begin(6);
    const int rc = launch_g2p2g<DIM, T>(p, L, w, in, out, perm, ex, s, nullptr);
    if (tm) tm->end(1);
    if (rc != FFMPM_OK) return rc;
    snapshot<DIM, T>(snap, k, out, ids_out, L.n, s);
  }
  return check_launch();
}

template <int DIM, typename T>
int op_substeps_sorted(const ffmpm_params& p, const Layout& L, const Ws& w, ffmpm_particles* a, ffmpm_particles* b,
                       int32_t* ids_a, int32_t* ids_b, int nsteps, cudaStream_t s, PhaseTimer* tm = nullptr,
                       const SnapOut* snap = nullptr) {
  PView<T> va = pview<T>(*a), vb = pview<T>(*b);
  if (fused(p, L, nsteps)) return op_substeps_fused<DIM, T>(p, L, w, va, vb, ids_a, ids_b, nsteps, s, tm, snap);
  const int K = sort_every(p);
  const uint32_t* flag = K > 1 ? &w.hdr->sort_now : nullptr;
  for (int k = 0; k < nsteps; ++k) {
    const PView<T>& in = (k & 1) ? vb : va;
    const PView<T>& out = (k & 1) ? va : vb;
    const int32_t* ids_in = (k & 1) ? ids_b : ids_a;
    int32_t* ids_out = (k & 1) ? ids_a : ids_b;
    const uint32_t* perm = nullptr;
    if (flag) k_sort_decide<<<1, 1, 0, s>>>(w.hdr, k % K == 0 ? 1 : 0);
    sort_and_plan<DIM, T>(p, L, w, in, k > 0, &perm, s, tm, flag);
    if (tm) tm->begin(3);
    if (p.deterministic)
      launch_p2g_det<DIM, T>(p, L, w, in, perm, s);
    else
      launch_p2g<DIM, T>(p, L, w, in, perm, InternalSink<T>{static_cast<Node4<T>*>(w.gridA)}, s, flag);
    if (tm) tm->end(1);
    if (tm) tm->begin(4);
    if (p.deterministic)
      launch_grid_update_det<DIM, T>(p, L, w, s);
    else
      launch_grid_update<DIM, T>(p, L, w, s);
    if (tm) tm->end(1);
    G2PExtra ex{ids_in, ids_out, w.keys_next, w.block_count, L.cell_bits, flag ? w.gridB : nullptr,
                flag ? &w.hdr->far_stray : nullptr};
    if (tm) tm->begin(5);
    int rc = launch_g2p<DIM, T, true, true>(p, L, w, in, out, perm, nullptr, ex, s, flag);
    if (tm) tm->end(1);
    if (rc != FFMPM_OK) return rc;
    snapshot<DIM, T>(snap, k, out, ids_out, L.n, s);
  }
  // The last G2P counted the blocks of the final state for a substep that will not run here:
  // clear the histogram so the workspace invariant (zero between calls) holds.
  cudaMemsetAsync(w.block_count, 0, sizeof(uint32_t) * L.nblocks, s);
  return check_launch();
}

template <int DIM, typename T>
int op_p2g(const ffmpm_params& p, const Layout& L, const Ws& w, const ffmpm_particles* P, ffmpm_grid* grid,
           cudaStream_t s) {
  const PView<T> pv = pview<T>(*P);
  const uint32_t* perm = nullptr;
  sort_and_plan<DIM, T>(p, L, w, pv, false, &perm, s);
  if (p.deterministic) {
    launch_p2g_det<DIM, T>(p, L, w, pv, perm, s);
    launch_grid_update_det<DIM, T>(p, L, w, s, static_cast<T*>(grid->velocity), static_cast<T*>(grid->mass));
  } else {
    launch_p2g<DIM, T>(p, L, w, pv, perm,
                       UserSink<T, DIM>{static_cast<T*>(grid->velocity), static_cast<T*>(grid->mass)}, s);
  }
  return check_launch();
}

template <int DIM, typename T>
int op_g2p(const ffmpm_params& p, const Layout& L, const Ws& w, const ffmpm_grid* grid, ffmpm_particles* P,
           cudaStream_t s) {
  const PView<T> pv = pview<T>(*P);
  const uint32_t* perm = nullptr;
  sort_and_plan<DIM, T>(p, L, w, pv, false, &perm, s);
  G2PExtra ex{};
  int rc = launch_g2p<DIM, T, false, false>(p, L, w, pv, pv, perm, static_cast<const T*>(grid->velocity), ex, s);
  return rc != FFMPM_OK ? rc : check_launch();
}

template <int DIM, typename T>
int op_grid_op(const ffmpm_params& p, ffmpm_grid* grid, cudaStream_t s) {
  const int R = p.res + 1;
  const int64_t nn = DIM == 3 ? int64_t(R) * R * R : int64_t(R) * R;
  const int blocks = (int)std::min<int64_t>((nn + kThreads - 1) / kThreads, int64_t(sm_count()) * 16);
  k_grid_op_dense<DIM, T><<<std::max(blocks, 1), kThreads, 0, s>>>(kparams<T>(p), R, static_cast<T*>(grid->velocity),
                                                                   static_cast<const T*>(grid->mass));
  return check_launch();
}

template <int DIM, typename T>
int op_sort(const ffmpm_params& p, const Layout& L, const Ws& w, const void* x, uint32_t* keys_out,
            uint32_t* perm_out, cudaStream_t s) {
  const KParams<T> kp = kparams<T>(p);
  const Geom<DIM> g = geom<DIM>(L);
  const uint32_t n = (uint32_t)L.n;
  PView<T> xv{};
  xv.x = static_cast<T*>(const_cast<void*>(x));
  k_keys<DIM, T><<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(kp, g, xv, n, L.cell_bits, w.keys_next, nullptr,
                                                                     &w.hdr->status);
  const uint32_t *ks = nullptr, *perm = nullptr;
  radix_sort(w.keys_next, n, L.passes, w.keys0, w.keys1, w.vals0, w.vals1, w.hist, (int)L.ntiles, &w.hdr->status, s, &ks,
             &perm, nullptr, p.wait_limit, p.inject);
  if (keys_out) cudaMemcpyAsync(keys_out, ks, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  if (perm_out) cudaMemcpyAsync(perm_out, perm, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  return check_launch();
}

template <int DIM, typename T>
int op_diag(const ffmpm_params& p, const ffmpm_particles* P, double* out, cudaStream_t s) {
  k_diag_init<<<1, 32, 0, s>>>(out);
  const uint32_t n = (uint32_t)P->n;
  const int blocks = std::max(1, (int)std::min<int64_t>((n + kThreads - 1) / kThreads, int64_t(sm_count()) * 8));
  if (n > 0) k_diag<DIM, T><<<blocks, kThreads, 0, s>>>(kparams<T>(p), pview<T>(*P), n, out);
  return check_launch();
}

// Dispatch on (dim, precision).
template <template <int, typename> class Op, typename... Args>
int dispatch(const ffmpm_params& p, Args&&... args) {
  if (p.dim == 3) {
    if (p.real_bytes == 4) return Op<3, float>::run(p, args...);
    return Op<3, double>::run(p, args...);
  }
  if (p.real_bytes == 4) return Op<2, float>::run(p, args...);
  return Op<2, double>::run(p, args...);
}

#define FFMPM_OP(NAME, FN)                                          \
  template <int DIM, typename T>                                    \
  struct NAME {                                                     \
    template <typename... A>                                        \
    static int run(const ffmpm_params& p, A&&... a) {               \
      return FN<DIM, T>(p, a...);                                   \
    }                                                               \
  };
FFMPM_OP(SubstepOp, op_substep)
FFMPM_OP(SubstepHostOp, op_substep_host)
FFMPM_OP(SortedOp, op_substeps_sorted)
FFMPM_OP(ProfileOp, op_substeps_sorted)
FFMPM_OP(SnapshotOp, op_substeps_sorted)
FFMPM_OP(P2GOp, op_p2g)
FFMPM_OP(G2POp, op_g2p)
FFMPM_OP(GridOp, op_grid_op)
FFMPM_OP(SortOp, op_sort)
FFMPM_OP(DiagOp, op_diag)
#undef FFMPM_OP

bool particles_ok(const ffmpm_params& p, const ffmpm_particles* P, bool need_jp) {
  if (!P || P->n < 0) return false;
  if (P->stride != 0 && P->stride < P->n) return false;
  if (P->n == 0) return true;
  if (!P->x || !P->v || !P->F || !P->C) return false;
  if (need_jp && !P->Jp) return false;
  return true;
}

bool supported(const ffmpm_params& p) { return true; }

int prologue(const ffmpm_params* p, int64_t n, void* ws, size_t ws_bytes, Layout* L) {
  if (!p || !make_layout(*p, n, L)) return FFMPM_ERR_BADARG;
  if (!supported(*p)) return FFMPM_ERR_UNSUPPORTED;
  if (p->deterministic) {
    const int tn = p->dim == 3 ? L->tile * L->tile * L->tile : L->tile * L->tile;
    const size_t smem = p->real_bytes == 4 ? (p->dim == 3 ? p2g_det_smem_bytes<3, float>(tn) : p2g_det_smem_bytes<2, float>(tn))
                                           : (p->dim == 3 ? p2g_det_smem_bytes<3, double>(tn)
                                                          : p2g_det_smem_bytes<2, double>(tn));
    if (smem > kMaxDynSmem) return FFMPM_ERR_UNSUPPORTED;  // warp tiles + records must fit in shared memory
  } else if (cells_smem_bytes(*L) > kMaxDynSmem) {
    return FFMPM_ERR_UNSUPPORTED;  // the cell-run P2G's tile and records must fit in shared memory
  }
  if (!ws || ws_bytes < L->total || (reinterpret_cast<uintptr_t>(ws) & 255)) return FFMPM_ERR_WORKSPACE;
  return FFMPM_OK;
}

}  // namespace
}  // namespace ffmpm

using namespace ffmpm;

extern "C" {

const char* ffmpm_version(void) { return "femflow_gb300 mpm 0.1 (sm_103a)"; }

int ffmpm_workspace_size(const ffmpm_params* p, int64_t n, size_t* bytes) {
  Layout L;
  if (!p || !bytes || !make_layout(*p, n, &L)) return FFMPM_ERR_BADARG;
  *bytes = L.total;
  return FFMPM_OK;
}

int ffmpm_workspace_init(const ffmpm_params* p, int64_t n, void* ws, size_t ws_bytes, void* stream) {
  Layout L;
  if (!p || !make_layout(*p, n, &L)) return FFMPM_ERR_BADARG;
  if (!ws || ws_bytes < L.total) return FFMPM_ERR_WORKSPACE;
  cudaMemsetAsync(ws, 0, L.total, static_cast<cudaStream_t>(stream));
  return check_launch();
}

int ffmpm_status_read(void* ws, int32_t* status, uint32_t* polar_fallbacks, void* stream) {
  if (!ws) return FFMPM_ERR_WORKSPACE;
  WsHeader h;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&h, ws, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FFMPM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return FFMPM_ERR_CUDA;
  if (status) *status = h.status;
  if (polar_fallbacks) *polar_fallbacks = h.polar_fallbacks;
  return FFMPM_OK;
}

int ffmpm_status_clear(void* ws, void* stream) {
  if (!ws) return FFMPM_ERR_WORKSPACE;
  cudaMemsetAsync(ws, 0, 8, static_cast<cudaStream_t>(stream));  // status + polar_fallbacks
  return check_launch();
}

int ffmpm_substep(const ffmpm_params* p, ffmpm_particles* P, void* ws, size_t ws_bytes, void* stream) {
  Layout L;
  if (!P) return FFMPM_ERR_BADARG;
  int rc = prologue(p, P->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, P, true)) return FFMPM_ERR_BADARG;
  if (P->n == 0) return FFMPM_OK;
  Ws w = bind(ws, L);
  return dispatch<SubstepOp>(*p, L, w, P, static_cast<cudaStream_t>(stream));
}

int ffmpm_substep_host(const ffmpm_params* p, const ffmpm_particles* host, ffmpm_particles* dev, void* ws,
                       size_t ws_bytes, void* stream) {
  Layout L;
  if (!host || !dev || host->n != dev->n || host->stride != 0 || dev->stride != 0) return FFMPM_ERR_BADARG;
  int rc = prologue(p, host->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, host, true) || !particles_ok(*p, dev, true)) return FFMPM_ERR_BADARG;
  if ((host->mass && !dev->mass) || (host->mu_0 && !dev->mu_0) || (host->lambda_0 && !dev->lambda_0))
    return FFMPM_ERR_BADARG;
  if (host->n == 0) return FFMPM_OK;
  // the device arrays stand in for the host ones: material pointers the host leaves NULL stay NULL
  ffmpm_particles d = *dev;
  if (!host->mass) d.mass = nullptr;
  if (!host->mu_0) d.mu_0 = nullptr;
  if (!host->lambda_0) d.lambda_0 = nullptr;
  Ws w = bind(ws, L);
  return dispatch<SubstepHostOp>(*p, L, w, host, &d, static_cast<cudaStream_t>(stream));
}

int ffmpm_substeps_sorted(const ffmpm_params* p, ffmpm_particles* a, ffmpm_particles* b, int32_t* ids_a,
                          int32_t* ids_b, int32_t nsteps, void* ws, size_t ws_bytes, void* stream) {
  Layout L;
  if (!a || !b || nsteps < 0 || a->n != b->n) return FFMPM_ERR_BADARG;
  int rc = prologue(p, a->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, a, true) || !particles_ok(*p, b, true)) return FFMPM_ERR_BADARG;
  if ((a->mass != nullptr) != (b->mass != nullptr) || (a->mu_0 != nullptr) != (b->mu_0 != nullptr) ||
      (a->lambda_0 != nullptr) != (b->lambda_0 != nullptr) || ((ids_a != nullptr) != (ids_b != nullptr)))
    return FFMPM_ERR_BADARG;
  if (a->n == 0 || nsteps == 0) return FFMPM_OK;
  Ws w = bind(ws, L);
  return dispatch<SortedOp>(*p, L, w, a, b, ids_a, ids_b, (int)nsteps, static_cast<cudaStream_t>(stream));
}

int ffmpm_substeps_sorted_snapshots(const ffmpm_params* p, ffmpm_particles* a, ffmpm_particles* b, int32_t* ids_a,
                                    int32_t* ids_b, int32_t nsteps, void* snap_x, int32_t* snap_ids, void* ws,
                                    size_t ws_bytes, void* stream) {
  Layout L;
  if (!a || !b || nsteps < 0 || a->n != b->n || !ids_a || !ids_b || !snap_x || !snap_ids) return FFMPM_ERR_BADARG;
  if (a->stride < a->n || b->stride < b->n) return FFMPM_ERR_BADARG;  // component-major buffers only
  int rc = prologue(p, a->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, a, true) || !particles_ok(*p, b, true)) return FFMPM_ERR_BADARG;
  if ((a->mass != nullptr) != (b->mass != nullptr) || (a->mu_0 != nullptr) != (b->mu_0 != nullptr) ||
      (a->lambda_0 != nullptr) != (b->lambda_0 != nullptr))
    return FFMPM_ERR_BADARG;
  if (a->n == 0 || nsteps == 0) return FFMPM_OK;
  Ws w = bind(ws, L);
  const SnapOut snap{snap_x, snap_ids};
  return dispatch<SnapshotOp>(*p, L, w, a, b, ids_a, ids_b, (int)nsteps, static_cast<cudaStream_t>(stream),
                              static_cast<PhaseTimer*>(nullptr), &snap);
}

int ffmpm_profile_substeps(const ffmpm_params* p, ffmpm_particles* a, ffmpm_particles* b, int32_t* ids_a,
                           int32_t* ids_b, int32_t nsteps, void* ws, size_t ws_bytes, void* stream, double* phase_ms,
                           int64_t* phase_launches) {
  Layout L;
  if (!a || !b || nsteps < 0 || a->n != b->n || !phase_ms || !phase_launches) return FFMPM_ERR_BADARG;
  int rc = prologue(p, a->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, a, true) || !particles_ok(*p, b, true)) return FFMPM_ERR_BADARG;
  if (a->n == 0 || nsteps == 0) return FFMPM_OK;
  Ws w = bind(ws, L);
  PhaseTimer tm;
  tm.s = static_cast<cudaStream_t>(stream);
  rc = dispatch<ProfileOp>(*p, L, w, a, b, ids_a, ids_b, (int)nsteps, tm.s, &tm);
  tm.collect(phase_ms, phase_launches);
  return rc;
}

int ffmpm_plan_info(const ffmpm_params* p, int64_t n, int64_t* info) {
  Layout L;
  if (!p || !info || !make_layout(*p, n, &L)) return FFMPM_ERR_BADARG;
  info[0] = L.bs;
  info[1] = L.nb;
  info[2] = L.nblocks;
  info[3] = L.key_bits;
  info[4] = L.passes;
  // digit histogram + one kernel per radix pass + 3 plan kernels + P2G + grid + G2P (+ the re-sort
  // decision of cadenced runs)
  info[5] = L.passes + 7 + (sort_every(*p) > 1 ? 1 : 0);
  info[6] = L.tile;
  info[7] = L.max_chunks;
  return FFMPM_OK;
}

int ffmpm_check_collision_points(const ffmpm_params* p, const double* points, const double* normals, int32_t n,
                                 void* grid_velocity, void* stream) {
  if (!p || n < 0 || (n > 0 && (!points || !normals || !grid_velocity))) return FFMPM_ERR_BADARG;
  if (!valid_params(p)) return FFMPM_ERR_BADARG;
  if (p->plane_rule != FFMPM_PLANES_STICKY && p->plane_rule != FFMPM_PLANES_REFERENCE_LITERAL) return FFMPM_ERR_BADARG;
  const int dim = p->dim;
  for (int i = 0; i < n * dim; ++i)
    if (!std::isfinite(points[i]) || !std::isfinite(normals[i])) return FFMPM_ERR_BADARG;
  for (int i = 0; i < n; ++i) {
    double ss = 0.0;
    for (int d = 0; d < dim; ++d) ss += normals[i * dim + d] * normals[i * dim + d];
    if (!(ss > 0.0)) return FFMPM_ERR_BADARG;  // the reference divides by |normal|
  }
  const int64_t R = p->res + 1;
  const int64_t nnodes = dim == 3 ? R * R * R : R * R;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the planes go to the kernel in batches of FFMPM_MAX_PLANES (zeroing is idempotent, so the
  // batches compose like the reference's loop over planes)
  for (int b = 0; b < n; b += FFMPM_MAX_PLANES) {
    ffmpm_params q = *p;
    q.n_planes = std::min(n - b, FFMPM_MAX_PLANES);
    for (int i = 0; i < q.n_planes; ++i)
      for (int d = 0; d < 3; ++d) {
        q.planes[i][d] = d < dim ? points[(b + i) * dim + d] : 0.0;
        q.planes[i][3 + d] = d < dim ? normals[(b + i) * dim + d] : 0.0;
      }
    const int blocks = work_grid((nnodes + kThreads - 1) / kThreads, 8);
    if (p->real_bytes == 4) {
      if (dim == 3)
        k_collision_points<3, float><<<blocks, kThreads, 0, s>>>(kparams<float>(q), static_cast<float*>(grid_velocity), nnodes);
      else
        k_collision_points<2, float><<<blocks, kThreads, 0, s>>>(kparams<float>(q), static_cast<float*>(grid_velocity), nnodes);
    } else {
      if (dim == 3)
        k_collision_points<3, double><<<blocks, kThreads, 0, s>>>(kparams<double>(q), static_cast<double*>(grid_velocity), nnodes);
      else
        k_collision_points<2, double><<<blocks, kThreads, 0, s>>>(kparams<double>(q), static_cast<double*>(grid_velocity), nnodes);
    }
  }
  return check_launch();
}

int ffmpm_kernels_per_call(const ffmpm_params* p, int64_t n, int32_t nsteps, int64_t* count) {
  Layout L;
  if (!p || !count || nsteps < 0 || !make_layout(*p, n, &L)) return FFMPM_ERR_BADARG;
  const int64_t sort = 1 + L.passes + 3;  // digit histogram, one kernel per pass, three plan kernels
  if (n == 0 || nsteps == 0) {
    *count = 0;
  } else if (fused(*p, L, nsteps)) {
    // keys + sort + P2G; per substep k < n-1: grid update + fused kernel (+ sort when 1 <= k <= n-2
    // is a multiple of the cadence); the last substep: grid update + G2P
    *count = (1 + sort + 1) + int64_t(nsteps - 1) * 2 + int64_t((nsteps - 2) / sort_every(*p)) * sort + 2;
  } else {
    // per substep: (decide) + sort + P2G + grid update + G2P; keys once
    *count = int64_t(nsteps) * ((sort_every(*p) > 1 ? 1 : 0) + sort + 3) + 1;
  }
  return FFMPM_OK;
}

int ffmpm_p2g(const ffmpm_params* p, const ffmpm_particles* P, ffmpm_grid* grid, void* ws, size_t ws_bytes,
              void* stream) {
  Layout L;
  if (!P || !grid || !grid->velocity || !grid->mass) return FFMPM_ERR_BADARG;
  int rc = prologue(p, P->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, P, p->model == FFMPM_MODEL_SNOW)) return FFMPM_ERR_BADARG;
  if (P->n == 0) return FFMPM_OK;
  Ws w = bind(ws, L);
  return dispatch<P2GOp>(*p, L, w, P, grid, static_cast<cudaStream_t>(stream));
}

int ffmpm_grid_op(const ffmpm_params* p, ffmpm_grid* grid, void* stream) {
  Layout L;
  if (!p || !make_layout(*p, 0, &L)) return FFMPM_ERR_BADARG;
  if (!grid || !grid->velocity || !grid->mass) return FFMPM_ERR_BADARG;
  return dispatch<GridOp>(*p, grid, static_cast<cudaStream_t>(stream));
}

int ffmpm_g2p(const ffmpm_params* p, const ffmpm_grid* grid, ffmpm_particles* P, void* ws, size_t ws_bytes,
              void* stream) {
  Layout L;
  if (!P || !grid || !grid->velocity) return FFMPM_ERR_BADARG;
  int rc = prologue(p, P->n, ws, ws_bytes, &L);
  if (rc != FFMPM_OK) return rc;
  if (!particles_ok(*p, P, p->dim == 2 || p->model == FFMPM_MODEL_SNOW)) return FFMPM_ERR_BADARG;
  if (P->n == 0) return FFMPM_OK;
  Ws w = bind(ws, L);
  return dispatch<G2POp>(*p, L, w, grid, P, static_cast<cudaStream_t>(stream));
}

int ffmpm_sort_by_block(const ffmpm_params* p, const void* x, int64_t n, uint32_t* keys_out, uint32_t* perm_out,
                        void* ws, size_t ws_bytes, void* stream) {
  Layout L;
  if (!p || !make_layout(*p, n, &L)) return FFMPM_ERR_BADARG;
  if (!ws || ws_bytes < L.total || (reinterpret_cast<uintptr_t>(ws) & 255)) return FFMPM_ERR_WORKSPACE;
  if (n == 0) return FFMPM_OK;
  if (!x) return FFMPM_ERR_BADARG;
  Ws w = bind(ws, L);
  return dispatch<SortOp>(*p, L, w, x, keys_out, perm_out, static_cast<cudaStream_t>(stream));
}

int ffmpm_diagnostics_fp64(const ffmpm_params* p, const ffmpm_particles* P, double* out, void* stream) {
  Layout L;
  if (!p || !make_layout(*p, 0, &L) || !P || !out) return FFMPM_ERR_BADARG;
  if (P->n > 0 && (!P->x || !P->v || !P->F)) return FFMPM_ERR_BADARG;
  return dispatch<DiagOp>(*p, P, out, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
