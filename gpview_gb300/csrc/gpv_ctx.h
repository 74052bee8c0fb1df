// gpv_ctx.h -- the library context (one per host thread) and helpers shared by the host files.
#pragma once
#include <chrono>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "gpv_hostio.h"
#include "gpv_internal.h"

namespace gpv {

constexpr int kMaxSlabs = kSlabsMax;  // z slabs of gpv_voxelize_to_host's Level2 launch, at most
constexpr int kCopySlabs = 8;         // ... when its slabs are copied (pageable or slab outputs)

// Result arrays of one batch; every result of the batch holds a reference.
struct ResultSet {
  void *l1 = nullptr, *prefix = nullptr, *bindex = nullptr, *l2 = nullptr;
  void *l1n = nullptr, *l2n = nullptr;  // normals (optional)
  void *hier = nullptr;                 // voxel box hierarchy (optional)
  bool l2_external = false;             // l2 is the caller's pinned host buffer (not freed)
  cudaStream_t stream = 0;
  int refs = 0;
};

}  // namespace gpv

struct gpv_ctx {
  static constexpr int kStages = 9;
  int device = 0;
  int num_sms = 148;
  bool timing = false;                 // record per-stage CUDA events on the launching stream
  cudaEvent_t ev[kStages + 1] = {};
  double stage_ms[kStages] = {};       // accumulated stage durations
  uint64_t stage_calls = 0;
  // host-side time per call segment (timing on): 0 setup up to the first recorded launch,
  // 1 first launch to the first synchronisation returning, 2 planning between the
  // synchronisations, 3 second launch to the last synchronisation returning, 4 result assembly
  double host_ms[5] = {};
  std::string err;
  int tile = 0;                        // Level1 triangles per tile (autotuned; 0: by mesh size)
  // Level2 boundary voxels per chunk, upper bound (autotuned by gpv_autotune; the mask space caps
  // it at 4 for 16^3 sub-grids).  torus262k at 8^3, Level2 kernel ms: 8 -> 0.626, 16 -> 0.596,
  // 32 -> 0.712 (fewer chunks per column repeat the fill's u/v work for the triangles above them)
  int l2_chunk_cap = 16;
  int l2_mode = GPV_LEVEL2_AUTO;       // Level2 SAT organisation (GPV_LEVEL2_*)
  // failure-detection hooks (gpv_set_debug) and what they caused (gpv_get_debug)
  uint32_t wait_limit = 0;             // Level1 tile wait polls (0: built-in)
  int fail_wait = 0;                   // Level1's tile wait gives up at once
  int64_t debug_pair_cap = 0;          // next call's first pair capacity (one-shot)
  int64_t fail_allocs = 0;             // refuse this many of the next device allocations
  int64_t replans = 0;                 // calls re-run after a pair-buffer overflow
  // gpv_voxelize_to_host's packed Level2 output (gpv_set_host_expand): host threads expanding
  // 2-bit codes from page-locked staging, and which of the 8 z slabs send codes
  int host_threads = -1;               // -1: by the machine (up to 16); 0 or 1: off
  // slab k sends codes for the first packed_share percent of its boundary voxels when bit k is
  // set, and bytes for the rest.  Sharing every slab keeps the link and the host threads busy
  // together from the first slab to the last (star1310k host to host, ms: all bytes 7.30; the
  // first four slabs as codes 6.70; every slab 20% codes 6.78, 40% 6.48, 45% 6.41, 50% 6.56,
  // 60% 6.79, 100% 8.28)
  uint32_t packed_slabs = 0xff;
  int packed_share = 45;
  int64_t packed_min_bytes = 64ll << 20;  // smaller Level2 outputs go as bytes
  std::unique_ptr<gpv::ExpandPool> pool;
  uint32_t *h_codes = nullptr;         // page-locked staging of the codes (device-mapped)
  size_t h_codes_cap = 0;              // words
  bool graphs = true;                  // record the launch sequences as CUDA graphs
  // One-graph calls (gpv_set_graphs): a call whose meshes (triangle counts) and grids repeat the
  // previous call on this path (og_key) is recorded as one graph whose result arrays and
  // second-half launches are sized by that call's counts (og_caps).
  bool one_graph = true;
  uint64_t og_key = 0;
  gpv::PlanCaps og_caps = {};
  int64_t og_calls = 0, og_replans = 0;
  int64_t debug_og_cap = 0;            // the next one-graph call's boundary capacity (one-shot)
  bool og_skip = false;                // the next call runs as two graphs (a re-run, one-shot)
  int normals = 0;                     // GPV_NORMALS_* for the next voxelizations
  bool hierarchy = false;              // build the voxel box hierarchy
  int fill = GPV_FILL_RAY;             // inside fill of both levels
  cudaGraphExec_t gexec[3] = {};       // cached executable graphs: the two phases, one-graph calls
  // Launch signature of each cached graph (every value its kernels and copies take as
  // arguments: workspace pointers, sizes, flags) and its kernel count: a call whose signature
  // matches replays the graph without recording it again.
  std::vector<uint64_t> gsig[3];
  uint64_t glaunch[3] = {};
  uint64_t graph_launches = 0, graph_instantiations = 0;
  gpv::MeshStats *h_stats = nullptr;   // pinned, h_cap entries
  gpv::MeshDesc *h_md = nullptr;       // pinned, h_cap entries
  size_t h_cap = 0;
  gpv::SortTile *h_tiles = nullptr;    // pinned
  int64_t *h_tb = nullptr;             // pinned
  size_t h_tiles_cap = 0, h_tb_cap = 0;
  uint32_t *h_u32 = nullptr;           // pinned scratch (small)
  float *h_tables = nullptr;           // pinned staging for coordinate tables
  size_t h_tables_cap = 0;
  // Device workspace kept across calls (grow-only): every intermediate of a voxelization is carved
  // from this slab; requests beyond it fall back to stream-ordered allocations and the slab is
  // grown to the recorded need at the next call.  Calls on one context run one at a time (each
  // ends with a stream synchronisation), so the slab is idle between calls.
  void *slab = nullptr;
  size_t slab_cap = 0, slab_want = 0;
  int64_t pair_hint = 0;               // pair-buffer capacity for the next call (grow-only)
  cudaStream_t cstream = nullptr;      // copy stream of gpv_voxelize_to_host (lazily created)
  cudaEvent_t cev[gpv::kMaxSlabs + 2] = {};  // its ordering events
  gpv::SlabStreams slab_aux = {};      // two streams for overlapping Level2 slab launches
  gpv_grid_spec last_spec = {};        // grid of the previous single-mesh call, derived
  std::shared_ptr<gpv::GridHost> last_gh;
  uint64_t next_handle = 1;
  std::mutex owned_mu;                 // results may be released from another host thread
  std::unordered_map<uint64_t, std::shared_ptr<gpv::ResultSet>> owned;
};

namespace gpv {

inline int ctx_fail(gpv_ctx *ctx, int code, const char *what) {
  if (ctx) ctx->err = what;
  return code;
}

inline int ctx_cuda_fail(gpv_ctx *ctx, cudaError_t e, const char *where) {
  if (ctx) ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? GPV_ERR_OOM : GPV_ERR_CUDA;
}

// Stream-ordered device allocation of the context; refused while the failure-detection hook
// GPV_DEBUG_FAIL_ALLOCS has refusals left.
inline cudaError_t ctx_malloc_async(gpv_ctx *ctx, void **p, size_t bytes, cudaStream_t s) {
  if (ctx->fail_allocs > 0) {
    ctx->fail_allocs--;
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocAsync(p, bytes, s);
}

inline cudaError_t ctx_ensure_tables(gpv_ctx *ctx, size_t n) {
  if (ctx->h_tables_cap >= n) return cudaSuccess;
  if (ctx->h_tables) cudaFreeHost(ctx->h_tables);
  ctx->h_tables = nullptr;
  ctx->h_tables_cap = 0;
  cudaError_t e = cudaMallocHost(&ctx->h_tables, std::max<size_t>(n, 1024) * sizeof(float));
  if (e == cudaSuccess) ctx->h_tables_cap = std::max<size_t>(n, 1024);
  return e;
}

inline cudaError_t ctx_ensure_host(gpv_ctx *ctx, size_t nmesh) {
  if (ctx->h_cap >= nmesh) return cudaSuccess;
  if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
  if (ctx->h_md) cudaFreeHost(ctx->h_md);
  ctx->h_stats = nullptr;
  ctx->h_md = nullptr;
  ctx->h_cap = 0;
  const size_t cap = std::max<size_t>(nmesh, 16);
  cudaError_t e = cudaMallocHost(&ctx->h_stats, cap * sizeof(MeshStats));
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_md, cap * sizeof(MeshDesc));
  if (e == cudaSuccess) ctx->h_cap = cap;
  return e;
}

inline cudaError_t ctx_ensure_host_tiles(gpv_ctx *ctx, size_t ntiles, size_t ntb) {
  cudaError_t e = cudaSuccess;
  if (ctx->h_tiles_cap < ntiles) {
    if (ctx->h_tiles) cudaFreeHost(ctx->h_tiles);
    ctx->h_tiles = nullptr;
    ctx->h_tiles_cap = 0;
    e = cudaMallocHost(&ctx->h_tiles, ntiles * sizeof(SortTile));
    if (e != cudaSuccess) return e;
    ctx->h_tiles_cap = ntiles;
  }
  if (ctx->h_tb_cap < ntb) {
    if (ctx->h_tb) cudaFreeHost(ctx->h_tb);
    ctx->h_tb = nullptr;
    ctx->h_tb_cap = 0;
    e = cudaMallocHost(&ctx->h_tb, ntb * sizeof(int64_t));
    if (e != cudaSuccess) return e;
    ctx->h_tb_cap = ntb;
  }
  return e;
}

// Host destinations of gpv_voxelize_to_host (one mesh): the Level1 outputs are copied on the
// context's copy stream as soon as they exist, the Level2 outputs slab by slab while later slabs
// compute.
struct HostSink {
  uint8_t *l1;
  int32_t *prefix, *bindex;
  uint8_t *l2;
  int64_t l2_cap;  // bytes available at l2
  int nslab;       // z slabs of the Level2 launch (0: by the Level2 output size)
  uint8_t *l2_dev; // device address of l2 when it is pinned host memory the Level2 kernel may
                   // write directly (no copy), else null
  bool l1_pinned;  // the Level1 destinations are page-locked (their copies can be recorded)
};
int run_batch(gpv_ctx *ctx, int n, const float *const *d_tris, const int64_t *T,
              const gpv_grid_spec *specs, gpv_result *out, cudaStream_t s,
              const HostSink *sink = nullptr);
int autotune(gpv_ctx *ctx, int n, const float *const *d_tris, const int64_t *T,
             const gpv_grid_spec *specs, cudaStream_t s, int reps, int *best_tile,
             int *best_chunk, float *best_ms);

}  // namespace gpv
