// gpv_api.cu -- host orchestration of the plain (one mesh per launch sequence) path and the
// native C ABI.  Grid and coordinate tables are derived on the host in double and rounded to
// float exactly as the reference's CPU code does; the kernels only ever see float.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>

#include "gpv_ctx.h"

namespace gpv {

float eps_threshold() {
  float a = 1e-6f;
  while ((double)a >= 1e-6) a = std::nextafter(a, 0.0f);
  while ((double)std::nextafter(a, 1.0f) < 1e-6) a = std::nextafter(a, 1.0f);
  return a;
}

int grid_derive(const gpv_grid_spec &spec, GridHost &gh, const float *ext1_override) {
  gh.spec = spec;
  int64_t N1 = 1;
  for (int a = 0; a < 3; ++a) {
    if (spec.ndiv[a] < 1 || spec.ndiv[a] > 65535) return GPV_ERR_INVALID;
    if (!std::isfinite(spec.bbox_min[a]) || !std::isfinite(spec.bbox_max[a]) ||
        !(spec.bbox_max[a] > spec.bbox_min[a]))
      return GPV_ERR_INVALID;
    if (spec.ndiv2[a] < 0 || spec.ndiv2[a] > 32) return GPV_ERR_INVALID;
    N1 *= spec.ndiv[a];
  }
  if (N1 >= (int64_t)1 << 31) return GPV_ERR_INVALID;
  const bool any2 = spec.ndiv2[0] || spec.ndiv2[1] || spec.ndiv2[2];
  const bool all2 = spec.ndiv2[0] && spec.ndiv2[1] && spec.ndiv2[2];
  if (any2 && !all2) return GPV_ERR_INVALID;
  gh.level2 = all2;
  gh.N1 = N1;
  gh.cells = all2 ? (int64_t)spec.ndiv2[0] * spec.ndiv2[1] * spec.ndiv2[2] : 0;
  for (int a = 0; a < 3; ++a) {
    const int n = spec.ndiv[a], n2 = all2 ? spec.ndiv2[a] : 1;
    gh.n[a] = n;
    gh.n2[a] = all2 ? n2 : 0;
    const float span = spec.bbox_max[a] - spec.bbox_min[a];
    // gridSize = (bBoxMax - bBoxMin) / (numDiv*1.0)  (src/Object.cpp:3108-3110)
    gh.g[a] = (float)(span / (n * 1.0));
    // boxExtents = gridSize / 2.0  (src/Object.cpp:3167, :2266)
    gh.e1[a] = ext1_override ? ext1_override[a] : (float)(gh.g[a] / 2.0);
    // gridSize2 = gridSize / (numDiv2*1.0), extents2 = gridSize2 / 2.0  (:3128-3130, :2359)
    gh.g2[a] = (float)(gh.g[a] / (n2 * 1.0));
    gh.e2[a] = (float)(gh.g2[a] / 2.0);
    gh.c1[a].resize(n);
    gh.c2s[a].resize((size_t)n * n2);
    gh.o2[a].resize((size_t)n * n2);
    const double bmin = spec.bbox_min[a];
    for (int i = 0; i < n; ++i) {
      // (p + 0.5)*boxExtents*2 + bBoxMin in double (src/Object.cpp:2329-2331); equal to the
      // midpoint/ray-origin form (i + 0.5)*gridSize + bBoxMin (:743-745, :3176) since
      // gridSize == 2*boxExtents and both products are exact in double.
      const float mid = (float)((i + 0.5) * gh.e1[a] * 2 + bmin);
      gh.c1[a][i] = mid;
      // Level2 ray origins: minPoint = i*gridSize + bBoxMin in float (:1132-1134), then
      // minPoint + (p + 0.5)*gridSize2 in double (:1158-1160).
      const float mn = (float)i * gh.g[a] + spec.bbox_min[a];
      for (int p = 0; p < n2; ++p) {
        // (p + 0.5)*gridSize2 + midPoint - boxExtentsLevel1 in double (:2389-2391)
        gh.c2s[a][(size_t)i * n2 + p] = (float)((p + 0.5) * gh.g2[a] + (double)mid - gh.e1[a]);
        gh.o2[a][(size_t)i * n2 + p] = (float)((double)mn + (p + 0.5) * gh.g2[a]);
      }
    }
  }
  // stencil fill clip heights (slice + 0.5)*gridSizeZ + bBoxMin[2] in double, float in GL
  // (src/Object.cpp:1534)
  gh.sp1.resize(gh.n[2]);
  for (int k = 0; k < gh.n[2]; ++k)
    gh.sp1[k] = (float)((k + 0.5) * (double)gh.g[2] + (double)spec.bbox_min[2]);
  gh.nxw = (gh.n[0] + 31) / 32;
  gh.nzw = (gh.n[2] + 31) / 32;
  int kb = 1;
  while (kb < 32 && ((int64_t)1 << kb) < N1) ++kb;
  gh.key_bits = kb;
  gh.thr = eps_threshold();
  gh.oz_monotone = true;
  for (size_t q = 1; q < gh.o2[2].size(); ++q)
    if (!(gh.o2[2][q] > gh.o2[2][q - 1])) gh.oz_monotone = false;
  return GPV_OK;
}

int64_t table_floats(const GridHost &gh) {
  int64_t n = 0;
  for (int a = 0; a < 3; ++a) n += (int64_t)gh.c1[a].size() + 2 * (int64_t)gh.c2s[a].size();
  return n + (int64_t)gh.sp1.size();
}

void pack_tables(const GridHost &gh, float *host) {
  size_t o = 0;
  for (int a = 0; a < 3; ++a) { std::memcpy(host + o, gh.c1[a].data(), 4 * gh.c1[a].size()); o += gh.c1[a].size(); }
  for (int a = 0; a < 3; ++a) { std::memcpy(host + o, gh.c2s[a].data(), 4 * gh.c2s[a].size()); o += gh.c2s[a].size(); }
  for (int a = 0; a < 3; ++a) { std::memcpy(host + o, gh.o2[a].data(), 4 * gh.o2[a].size()); o += gh.o2[a].size(); }
  std::memcpy(host + o, gh.sp1.data(), 4 * gh.sp1.size());
}

GridDev make_griddev(const GridHost &gh, const float *dt) {
  GridDev g;
  size_t o = 0;
  for (int a = 0; a < 3; ++a) {
    g.bmin[a] = gh.spec.bbox_min[a];
    g.bmax[a] = gh.spec.bbox_max[a];
    g.n[a] = gh.n[a];
    g.n2[a] = gh.n2[a];
    g.e1[a] = gh.e1[a];
    g.e2[a] = gh.e2[a];
    g.g[a] = gh.g[a];
    g.g2[a] = gh.g2[a];
  }
  for (int a = 0; a < 3; ++a) { g.c1[a] = dt + o; o += gh.c1[a].size(); }
  for (int a = 0; a < 3; ++a) { g.c2s[a] = dt + o; o += gh.c2s[a].size(); }
  for (int a = 0; a < 3; ++a) { g.o2[a] = dt + o; o += gh.o2[a].size(); }
  g.sp1 = dt + o;
  g.nxw = gh.nxw;
  g.nzw = gh.nzw;
  g.key_bits = gh.key_bits;
  g.thr = gh.thr;
  g.oz_monotone = gh.oz_monotone ? 1 : 0;
  for (int a = 0; a < 3; ++a) g.inv_g2[a] = gh.g2[a] > 0.f ? 1.0f / gh.g2[a] : 0.f;
  return g;
}

}  // namespace gpv

using namespace gpv;

namespace {
// Device address of a page-locked, 16-byte aligned host buffer (which kernels may read and write
// in place), or null for any other pointer.
template <typename T>
T *pinned_alias(T *h) {
  if (!h || (reinterpret_cast<uintptr_t>(h) & 15u)) return nullptr;
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, h) != cudaSuccess) {
    cudaGetLastError();  // an unknown pointer only means: not pinned
    return nullptr;
  }
  return pa.type == cudaMemoryTypeHost && pa.devicePointer ? static_cast<T *>(pa.devicePointer)
                                                           : nullptr;
}
}  // namespace

#define GPV_CUDA(call)                                        \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ctx_cuda_fail(ctx, e_, #call); \
  } while (0)

extern "C" {

int gpv_init(int device, gpv_ctx **out) {
  if (!out) return GPV_ERR_INVALID;
  *out = nullptr;
  gpv_ctx *ctx = new gpv_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete ctx; return GPV_ERR_CUDA; }
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (ctx_ensure_host(ctx, 16) != cudaSuccess || cudaMallocHost(&ctx->h_u32, 256) != cudaSuccess) {
    delete ctx;
    return GPV_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  *out = ctx;
  return GPV_OK;
}

void gpv_destroy(gpv_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  std::vector<ResultSet *> sets;
  for (auto &kv : ctx->owned) sets.push_back(kv.second.get());
  std::sort(sets.begin(), sets.end());
  sets.erase(std::unique(sets.begin(), sets.end()), sets.end());
  for (ResultSet *r : sets) {
    cudaFree(r->l1);
    cudaFree(r->prefix);
    cudaFree(r->bindex);
    if (!r->l2_external) cudaFree(r->l2);
    if (r->l1n) cudaFree(r->l1n);
    if (r->l2n) cudaFree(r->l2n);
    if (r->hier) cudaFree(r->hier);
  }
  ctx->owned.clear();
  for (cudaGraphExec_t &ge : ctx->gexec)
    if (ge) cudaGraphExecDestroy(ge);
  if (ctx->cstream) {
    cudaStreamSynchronize(ctx->cstream);
    cudaStreamDestroy(ctx->cstream);
  }
  for (cudaEvent_t &e : ctx->cev)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t &x : ctx->slab_aux.st)
    if (x) { cudaStreamSynchronize(x); cudaStreamDestroy(x); }
  if (ctx->slab_aux.fork) cudaEventDestroy(ctx->slab_aux.fork);
  for (cudaEvent_t &e : ctx->slab_aux.join)
    if (e) cudaEventDestroy(e);
  ctx->pool.reset();
  if (ctx->h_codes) cudaFreeHost(ctx->h_codes);
  if (ctx->slab) cudaFree(ctx->slab);
  if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
  if (ctx->h_md) cudaFreeHost(ctx->h_md);
  if (ctx->h_tiles) cudaFreeHost(ctx->h_tiles);
  if (ctx->h_tb) cudaFreeHost(ctx->h_tb);
  if (ctx->h_u32) cudaFreeHost(ctx->h_u32);
  if (ctx->h_tables) cudaFreeHost(ctx->h_tables);
  delete ctx;
}

const char *gpv_last_error(gpv_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int gpv_set_timing(gpv_ctx *ctx, int on) {
  if (!ctx) return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (on && !ctx->ev[0])
    for (int i = 0; i <= gpv_ctx::kStages; ++i)
      if (cudaEventCreate(&ctx->ev[i]) != cudaSuccess) return GPV_ERR_CUDA;
  ctx->timing = on != 0;
  for (double &v : ctx->stage_ms) v = 0.0;
  for (double &v : ctx->host_ms) v = 0.0;
  ctx->stage_calls = 0;
  return GPV_OK;
}

int gpv_stage_times(gpv_ctx *ctx, double *ms, int n) {
  if (!ctx || !ms) return GPV_ERR_INVALID;
  for (int i = 0; i < n && i < gpv_ctx::kStages; ++i) ms[i] = ctx->stage_ms[i];
  return (int)ctx->stage_calls;
}

int gpv_host_times(gpv_ctx *ctx, double *ms, int n) {
  if (!ctx || !ms) return GPV_ERR_INVALID;
  for (int i = 0; i < n && i < 5; ++i) ms[i] = ctx->host_ms[i];
  return (int)ctx->stage_calls;
}

uint64_t gpv_kernel_launches(void) { return gpv::launch_count(); }

int gpv_set_graphs(gpv_ctx *ctx, int mode) {
  if (!ctx) return GPV_ERR_INVALID;
  ctx->graphs = mode != 0;
  ctx->one_graph = mode != 0 && mode != GPV_GRAPHS_TWO;
  return GPV_OK;
}

int gpv_set_hierarchy(gpv_ctx *ctx, int on) {
  if (!ctx) return GPV_ERR_INVALID;
  ctx->hierarchy = on != 0;
  return GPV_OK;
}

int gpv_set_fill(gpv_ctx *ctx, int mode) {
  if (!ctx || (mode != GPV_FILL_RAY && mode != GPV_FILL_STENCIL))
    return ctx_fail(ctx, GPV_ERR_INVALID, "fill mode must be GPV_FILL_RAY or GPV_FILL_STENCIL");
  ctx->fill = mode;
  return GPV_OK;
}

int gpv_result_copy_hierarchy_to_host(gpv_ctx *ctx, const gpv_result *res, gpv_box *out,
                                      cudaStream_t s) {
  if (!ctx || !res || !out) return GPV_ERR_INVALID;
  if (!res->hierarchy || res->num_level1 < 2)
    return ctx_fail(ctx, GPV_ERR_INVALID, "the result has no hierarchy (gpv_set_hierarchy, power-of-two grid)");
  cudaSetDevice(ctx->device);
  GPV_CUDA(cudaMemcpyAsync(out, res->hierarchy, sizeof(gpv_box) * (res->num_level1 - 1),
                           cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaStreamSynchronize(s));
  return GPV_OK;
}

int gpv_set_normals(gpv_ctx *ctx, int mode) {
  if (!ctx || mode < GPV_NORMALS_OFF || mode > GPV_NORMALS_FLOAT) return GPV_ERR_INVALID;
  ctx->normals = mode;
  return GPV_OK;
}

int gpv_set_level2_chunk(gpv_ctx *ctx, int cap) {
  if (!ctx || cap < 1 || cap > 32) return GPV_ERR_INVALID;
  ctx->l2_chunk_cap = cap;
  return GPV_OK;
}

int gpv_set_host_expand(gpv_ctx *ctx, int threads, uint32_t slab_mask, int32_t share_percent,
                        int64_t min_level2_bytes) {
  if (!ctx || threads < -1 || threads > 256 || min_level2_bytes < 0 || share_percent < 0 ||
      share_percent > 100)
    return GPV_ERR_INVALID;
  if (threads != ctx->host_threads) ctx->pool.reset();  // made again with the new count
  ctx->host_threads = threads;
  ctx->packed_slabs = slab_mask;
  ctx->packed_share = share_percent;
  ctx->packed_min_bytes = min_level2_bytes;
  return GPV_OK;
}

int gpv_set_debug(gpv_ctx *ctx, int what, int64_t value) {
  if (!ctx || value < 0) return GPV_ERR_INVALID;
  switch (what) {
    case GPV_DEBUG_WAIT_LIMIT:
      if (value > 0xffffffffll) return GPV_ERR_INVALID;
      ctx->wait_limit = (uint32_t)value;
      return GPV_OK;
    case GPV_DEBUG_FAIL_WAIT: ctx->fail_wait = value != 0; return GPV_OK;
    case GPV_DEBUG_PAIR_CAPACITY: ctx->debug_pair_cap = value; return GPV_OK;
    case GPV_DEBUG_FAIL_ALLOCS: ctx->fail_allocs = value; return GPV_OK;
    case GPV_DEBUG_ONE_GRAPH_CAPACITY: ctx->debug_og_cap = value; return GPV_OK;
    default: return GPV_ERR_INVALID;
  }
}

int64_t gpv_get_debug(gpv_ctx *ctx, int what) {
  if (!ctx) return GPV_ERR_INVALID;
  switch (what) {
    case GPV_DEBUG_WAIT_LIMIT: return ctx->wait_limit;
    case GPV_DEBUG_FAIL_WAIT: return ctx->fail_wait;
    case GPV_DEBUG_PAIR_CAPACITY: return ctx->debug_pair_cap;
    case GPV_DEBUG_FAIL_ALLOCS: return ctx->fail_allocs;
    case GPV_DEBUG_REPLANS: return ctx->replans;
    case GPV_DEBUG_ONE_GRAPH_CAPACITY: return ctx->debug_og_cap;
    case GPV_DEBUG_ONE_GRAPH_CALLS: return ctx->og_calls;
    case GPV_DEBUG_ONE_GRAPH_REPLANS: return ctx->og_replans;
    default: return GPV_ERR_INVALID;
  }
}

int gpv_set_level2_mode(gpv_ctx *ctx, int mode) {
  if (!ctx || mode < GPV_LEVEL2_AUTO || mode > GPV_LEVEL2_INLINE) return GPV_ERR_INVALID;
  ctx->l2_mode = mode;
  return GPV_OK;
}

int gpv_autotune(gpv_ctx *ctx, int32_t n, const float *const *d_tris, const int64_t *num_triangles,
                 const gpv_grid_spec *specs, cudaStream_t stream, int32_t *tile,
                 int32_t *level2_chunk, float *ms_per_batch) {
  if (!ctx || n <= 0 || !d_tris || !num_triangles || !specs) return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  int t = 0, c = 0;
  const int rc = autotune(ctx, n, d_tris, num_triangles, specs, stream, 2, &t, &c, ms_per_batch);
  if (tile) *tile = t;
  if (level2_chunk) *level2_chunk = c;
  return rc;
}

int gpv_set_tile(gpv_ctx *ctx, int t) {
  if (!ctx || (t != 0 && t != 32 && t != 64 && t != 128 && t != 256)) return GPV_ERR_INVALID;
  ctx->tile = t;
  return GPV_OK;
}

int gpv_grid_padded(const float mesh_min[3], const float mesh_max[3], const int32_t ndiv[3],
                    const int32_t ndiv2[3], gpv_grid_spec *out) {
  if (!mesh_min || !mesh_max || !ndiv || !out) return GPV_ERR_INVALID;
  for (int a = 0; a < 3; ++a) {
    if (ndiv[a] < 3 || !std::isfinite(mesh_min[a]) || !std::isfinite(mesh_max[a]) ||
        mesh_max[a] < mesh_min[a])
      return GPV_ERR_INVALID;
    float ext = mesh_max[a] - mesh_min[a];
    if (!(ext > 0.f)) ext = 1e-3f;
    // one cell of padding on each side: n cells of size ext/(n-2)
    const float cell = ext / (float)(ndiv[a] - 2);
    out->bbox_min[a] = mesh_min[a] - cell;
    out->bbox_max[a] = mesh_max[a] + cell;
    out->ndiv[a] = ndiv[a];
    out->ndiv2[a] = ndiv2 ? ndiv2[a] : 0;
  }
  return GPV_OK;
}

int gpv_grid_reference(const float bbox_min[3], const float bbox_max[3], float max_model_size,
                       int32_t voxel_count, int32_t voxel_count2, gpv_grid_spec *out) {
  if (!bbox_min || !bbox_max || !out || voxel_count < 1 || voxel_count2 < 0) return GPV_ERR_INVALID;
  // src/Object.cpp:3094-3107: nominal = maxModelSize/(1.0*voxelCount) rounded to float;
  // numDiv = GetNextDiv4(max(1, int(extent / nominal))) with the extent divided in float.
  const float nominal = (float)(max_model_size / (1.0 * voxel_count));
  for (int a = 0; a < 3; ++a) {
    int n = (int)((bbox_max[a] - bbox_min[a]) / nominal);
    if (n == 0) n++;
    n = (n % 4 == 0) ? n : n + (4 - n % 4);
    out->ndiv[a] = n;
    out->ndiv2[a] = voxel_count2;
    out->bbox_min[a] = bbox_min[a];
    out->bbox_max[a] = bbox_max[a];
  }
  return GPV_OK;
}

int gpv_voxelize(gpv_ctx *ctx, const float *d_tris, int64_t num_triangles,
                 const gpv_grid_spec *spec, gpv_result *out, cudaStream_t stream) {
  if (!ctx || !spec || !out || (num_triangles > 0 && !d_tris)) return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return run_batch(ctx, 1, &d_tris, &num_triangles, spec, out, stream);
}

int gpv_voxelize_host(gpv_ctx *ctx, const float *h_tris, int64_t num_triangles,
                      const gpv_grid_spec *spec, gpv_result *out, cudaStream_t stream) {
  if (!ctx || !spec || !out || num_triangles < 0 || (num_triangles > 0 && !h_tris))
    return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (const float *dp = pinned_alias(h_tris))
    return run_batch(ctx, 1, &dp, &num_triangles, spec, out, stream);
  float *d = nullptr;
  const size_t bytes = (size_t)std::max<int64_t>(num_triangles, 1) * 9 * sizeof(float);
  cudaError_t e = cudaMallocAsync((void **)&d, bytes, stream);
  if (e != cudaSuccess) return ctx_cuda_fail(ctx, e, "cudaMallocAsync");
  if (num_triangles > 0) {
    e = cudaMemcpyAsync(d, h_tris, (size_t)num_triangles * 9 * sizeof(float),
                        cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) { cudaFreeAsync(d, stream); return ctx_cuda_fail(ctx, e, "cudaMemcpyAsync"); }
  }
  const float *dp = d;
  int rc = run_batch(ctx, 1, &dp, &num_triangles, spec, out, stream);
  cudaFreeAsync(d, stream);
  return rc;
}

int gpv_voxelize_to_host(gpv_ctx *ctx, const float *h_tris, int64_t num_triangles,
                         const gpv_grid_spec *spec, uint8_t *h_l1, int32_t *h_prefix,
                         int32_t *h_bindex, uint8_t *h_l2, int64_t h_l2_bytes, int32_t slabs,
                         gpv_result *out, cudaStream_t stream) {
  if (!ctx || !spec || !out || num_triangles < 0 || (num_triangles > 0 && !h_tris) ||
      h_l2_bytes < 0)
    return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  // page-locked triangles are read by the prep kernel in place (it packs them into device
  // memory for every later stage), so no device copy is made
  const float *pin = pinned_alias(h_tris);
  float *d = nullptr;
  if (!pin) {
    const size_t bytes = (size_t)std::max<int64_t>(num_triangles, 1) * 9 * sizeof(float);
    cudaError_t e = cudaMallocAsync((void **)&d, bytes, stream);
    if (e != cudaSuccess) return ctx_cuda_fail(ctx, e, "cudaMallocAsync");
    if (num_triangles > 0) {
      e = cudaMemcpyAsync(d, h_tris, (size_t)num_triangles * 9 * sizeof(float),
                          cudaMemcpyHostToDevice, stream);
      if (e != cudaSuccess) { cudaFreeAsync(d, stream); return ctx_cuda_fail(ctx, e, "cudaMemcpyAsync"); }
    }
  }
  // slabs == 0 with a pinned Level2 buffer: the Level2 kernel writes it directly
  uint8_t *l2_dev = slabs == 0 ? pinned_alias(h_l2) : nullptr;
  const bool l1_pinned = (!h_l1 || pinned_alias(h_l1)) && (!h_prefix || pinned_alias(h_prefix)) &&
                         (!h_bindex || pinned_alias(h_bindex));
  HostSink sink{h_l1, h_prefix, h_bindex, h_l2, h_l2_bytes, std::max(slabs, 0), l2_dev, l1_pinned};
  const float *dp = pin ? pin : d;
  int rc = run_batch(ctx, 1, &dp, &num_triangles, spec, out, stream, &sink);
  if (d) cudaFreeAsync(d, stream);
  return rc;
}

int gpv_result_copy_to_host(gpv_ctx *ctx, const gpv_result *res, uint8_t *l1, int32_t *prefix,
                            int32_t *bindex, uint8_t *l2, cudaStream_t s) {
  if (!ctx || !res) return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  const int64_t cells = (int64_t)res->spec.ndiv2[0] * res->spec.ndiv2[1] * res->spec.ndiv2[2];
  if (l1 && res->num_level1)
    GPV_CUDA(cudaMemcpyAsync(l1, res->level1_inout, res->num_level1, cudaMemcpyDeviceToHost, s));
  if (prefix && res->num_level1)
    GPV_CUDA(cudaMemcpyAsync(prefix, res->level1_prefix, 4 * res->num_level1,
                             cudaMemcpyDeviceToHost, s));
  if (bindex && res->num_boundary)
    GPV_CUDA(cudaMemcpyAsync(bindex, res->boundary_index, 4 * res->num_boundary,
                             cudaMemcpyDeviceToHost, s));
  // cudaMemcpyDefault: a result of gpv_voxelize_to_host may hold its Level2 bytes in host memory
  if (l2 && res->num_boundary && cells)
    GPV_CUDA(cudaMemcpyAsync(l2, res->level2_inout, res->num_boundary * cells, cudaMemcpyDefault,
                             s));
  GPV_CUDA(cudaStreamSynchronize(s));
  return GPV_OK;
}

int gpv_result_copy_normals_to_host(gpv_ctx *ctx, const gpv_result *res, void *l1n, void *l2n,
                                    cudaStream_t s) {
  if (!ctx || !res) return GPV_ERR_INVALID;
  if (res->normal_mode == GPV_NORMALS_OFF || !res->level1_normal)
    return ctx_fail(ctx, GPV_ERR_INVALID, "the result has no normals (gpv_set_normals)");
  cudaSetDevice(ctx->device);
  const int64_t cells = (int64_t)res->spec.ndiv2[0] * res->spec.ndiv2[1] * res->spec.ndiv2[2];
  const int64_t vb = res->normal_mode == GPV_NORMALS_FLOAT ? 12 : 3;  // bytes per voxel / cell
  if (l1n && res->num_level1)
    GPV_CUDA(cudaMemcpyAsync(l1n, res->level1_normal, vb * res->num_level1, cudaMemcpyDeviceToHost, s));
  if (l2n && res->num_boundary && cells)
    GPV_CUDA(cudaMemcpyAsync(l2n, res->level2_normal, vb * res->num_boundary * cells,
                             cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaStreamSynchronize(s));
  return GPV_OK;
}

int gpv_result_release(gpv_ctx *ctx, gpv_result *res) {
  if (!ctx || !res) return GPV_ERR_INVALID;
  std::shared_ptr<ResultSet> set;
  {
    std::lock_guard<std::mutex> lk(ctx->owned_mu);
    auto it = ctx->owned.find(res->handle);
    if (it == ctx->owned.end()) return GPV_ERR_INVALID;
    set = it->second;
    if (--set->refs <= 0) ctx->owned.erase(it);
    else set.reset();
  }
  cudaSetDevice(ctx->device);
  if (set) {
    // freed on the stream that made them, so the next call on that stream reuses the memory
    // directly (a free on another stream would make the pool map fresh memory for the next
    // large result)
    cudaStream_t fs = set->stream;
    cudaFreeAsync(set->l1, fs);
    cudaFreeAsync(set->prefix, fs);
    cudaFreeAsync(set->bindex, fs);
    if (!set->l2_external) cudaFreeAsync(set->l2, fs);
    if (set->l1n) cudaFreeAsync(set->l1n, fs);
    if (set->l2n) cudaFreeAsync(set->l2n, fs);
    if (set->hier) cudaFreeAsync(set->hier, fs);
  }
  res->level1_inout = nullptr;
  res->level1_prefix = nullptr;
  res->boundary_index = nullptr;
  res->level2_inout = nullptr;
  res->level1_normal = nullptr;
  res->level2_normal = nullptr;
  res->hierarchy = nullptr;
  res->handle = 0;
  return GPV_OK;
}

int gpv_voxelize_batch(gpv_ctx *ctx, int32_t n, const float *const *d_tris,
                       const int64_t *num_triangles, const gpv_grid_spec *specs,
                       gpv_result *results, cudaStream_t stream) {
  if (!ctx || n <= 0 || !d_tris || !num_triangles || !specs || !results) return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return run_batch(ctx, n, d_tris, num_triangles, specs, results, stream);
}

}  // extern "C"
