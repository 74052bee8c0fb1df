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

#include "gpv_internal.h"

struct gpv_ctx {
  static constexpr int kStages = 8;
  int device = 0;
  bool timing = false;                 // record per-stage CUDA events on the launching stream
  cudaEvent_t ev[kStages + 1] = {};
  double stage_ms[kStages] = {};      // accumulated stage durations
  uint64_t stage_calls = 0;
  std::string err;
  int tile = 128;
  gpv::MeshStats *h_stats = nullptr;  // pinned
  uint32_t *h_u32 = nullptr;          // pinned scratch (small)
  float *h_tables = nullptr;          // pinned staging for coordinate tables
  size_t h_tables_cap = 0;
  uint64_t next_handle = 1;
  struct Owned {
    void *l1, *prefix, *bindex, *l2;
  };
  std::unordered_map<uint64_t, Owned> owned;
};

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
  return n;
}

void pack_tables(const GridHost &gh, float *host) {
  size_t o = 0;
  for (int a = 0; a < 3; ++a) { std::memcpy(host + o, gh.c1[a].data(), 4 * gh.c1[a].size()); o += gh.c1[a].size(); }
  for (int a = 0; a < 3; ++a) { std::memcpy(host + o, gh.c2s[a].data(), 4 * gh.c2s[a].size()); o += gh.c2s[a].size(); }
  for (int a = 0; a < 3; ++a) { std::memcpy(host + o, gh.o2[a].data(), 4 * gh.o2[a].size()); o += gh.o2[a].size(); }
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
  g.nxw = gh.nxw;
  g.nzw = gh.nzw;
  g.key_bits = gh.key_bits;
  g.thr = gh.thr;
  g.oz_monotone = gh.oz_monotone ? 1 : 0;
  return g;
}

}  // namespace gpv

using namespace gpv;

namespace {

int fail(gpv_ctx *ctx, int code, const char *what) {
  if (ctx) ctx->err = what;
  return code;
}

int cuda_fail(gpv_ctx *ctx, cudaError_t e, const char *where) {
  if (ctx) ctx->err = std::string(where) + ": " + cudaGetErrorString(e);
  return GPV_ERR_CUDA;
}

#define GPV_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

// Stream-ordered allocation list freed together.
struct Arena {
  std::vector<void *> ptrs;
  cudaStream_t s;
  explicit Arena(cudaStream_t st) : s(st) {}
  template <typename T>
  cudaError_t get(T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(count * sizeof(T), 16), s);
    if (e == cudaSuccess) ptrs.push_back(q);
    *p = (T *)q;
    return e;
  }
  ~Arena() {
    for (void *p : ptrs) cudaFreeAsync(p, s);
  }
};

int ensure_tables(gpv_ctx *ctx, size_t n) {
  if (ctx->h_tables_cap >= n) return GPV_OK;
  if (ctx->h_tables) cudaFreeHost(ctx->h_tables);
  ctx->h_tables = nullptr;
  GPV_CUDA(cudaMallocHost(&ctx->h_tables, n * sizeof(float)));
  ctx->h_tables_cap = n;
  return GPV_OK;
}

}  // namespace

// ---- plain pipeline -----------------------------------------------------------------------------
static int voxelize_impl(gpv_ctx *ctx, const float *d_tris, int64_t T, const gpv_grid_spec *spec,
                         gpv_result *out, cudaStream_t s) {
  GridHost gh;
  int rc = grid_derive(*spec, gh);
  if (rc) return fail(ctx, rc, "invalid grid specification");
  if (T < 0 || T >= ((int64_t)1 << 31)) return fail(ctx, GPV_ERR_INVALID, "bad triangle count");
  if (T > 0 && (reinterpret_cast<uintptr_t>(d_tris) & 15u))
    return fail(ctx, GPV_ERR_INVALID, "triangle buffer must be 16-byte aligned");

  Arena ws(s);
  const int64_t nt = table_floats(gh);
  rc = ensure_tables(ctx, (size_t)nt);
  if (rc) return rc;
  float *d_tab;
  GPV_CUDA(ws.get(&d_tab, nt));
  pack_tables(gh, ctx->h_tables);
  GPV_CUDA(cudaMemcpyAsync(d_tab, ctx->h_tables, nt * sizeof(float), cudaMemcpyHostToDevice, s));
  const GridDev g = make_griddev(gh, d_tab);

  const int64_t N1 = gh.N1;
  const int64_t N1w = (int64_t)gh.n[2] * gh.n[1] * gh.nxw;
  const int64_t ncol = (int64_t)gh.n[0] * gh.n[1];
  Level1Bufs b{};
  b.tris = d_tris;
  b.T = T;
  GPV_CUDA(ws.get(&b.ptri, 3 * (size_t)std::max<int64_t>(T, 1)));
  GPV_CUDA(ws.get(&b.rng, (size_t)std::max<int64_t>(T, 1)));
  GPV_CUDA(ws.get(&b.fbox, (size_t)std::max<int64_t>(T, 1)));
  GPV_CUDA(ws.get(&b.bplane, (size_t)N1w));
  GPV_CUDA(ws.get(&b.iplane, (size_t)N1w));
  GPV_CUDA(ws.get(&b.toggles, (size_t)(ncol * gh.nzw)));
  GPV_CUDA(ws.get(&b.stats, 1));
  uint32_t *wcnt, *wpre, *d_tot, *scan_tmp;
  GPV_CUDA(ws.get(&wcnt, (size_t)N1w));
  GPV_CUDA(ws.get(&wpre, (size_t)N1w));
  GPV_CUDA(ws.get(&d_tot, 4));
  GPV_CUDA(ws.get(&scan_tmp, (size_t)scan_temp_words(N1w)));
  GPV_CUDA(cudaMemsetAsync(b.stats, 0, sizeof(MeshStats), s));
  GPV_CUDA(cudaMemsetAsync(b.bplane, 0, N1w * 4, s));
  GPV_CUDA(cudaMemsetAsync(b.toggles, 0, ncol * gh.nzw * 4, s));

  // results with sizes known up front
  uint8_t *l1 = nullptr;
  int32_t *prefix = nullptr;
  GPV_CUDA(cudaMallocAsync((void **)&l1, std::max<int64_t>(N1, 16), s));
  GPV_CUDA(cudaMallocAsync((void **)&prefix, 4 * std::max<int64_t>(N1, 4), s));
  int32_t *bindex = nullptr;
  uint8_t *l2 = nullptr;
  auto drop_results = [&]() {
    cudaFreeAsync(l1, s);
    cudaFreeAsync(prefix, s);
    if (bindex) cudaFreeAsync(bindex, s);
    if (l2) cudaFreeAsync(l2, s);
  };

  auto mark = [&](int i) {
    if (ctx->timing) cudaEventRecord(ctx->ev[i], s);
  };
  // 1. per-triangle preparation and work counts
  mark(0);
  launch_prep(g, b, s);
  mark(1);
  GPV_CUDA(cudaMemcpyAsync(ctx->h_stats, b.stats, sizeof(MeshStats), cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaStreamSynchronize(s));
  const uint64_t cap = std::max<uint64_t>(ctx->h_stats->sat1, 1);
  GPV_CUDA(ws.get(&b.keys, cap));
  GPV_CUDA(ws.get(&b.vals, cap));
  ctx->h_stats->pair_cap = cap;
  GPV_CUDA(cudaMemcpyAsync(&b.stats->pair_cap, &ctx->h_stats->pair_cap, sizeof(uint64_t),
                           cudaMemcpyHostToDevice, s));

  // 2. Level1 SAT + fill, boundary counts
  mark(2);
  launch_level1(g, b, ctx->tile, s);
  mark(3);
  launch_fill_finish(g, b, s);
  launch_popc(g, b.bplane, wcnt, s);
  scan_u32(wcnt, wpre, N1w, d_tot, scan_tmp, s);
  mark(4);
  GPV_CUDA(cudaGetLastError());
  GPV_CUDA(cudaMemcpyAsync(ctx->h_stats, b.stats, sizeof(MeshStats), cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaMemcpyAsync(ctx->h_u32, d_tot, 4, cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaStreamSynchronize(s));
  if (ctx->h_stats->status) {
    drop_results();
    return fail(ctx, (ctx->h_stats->status & ST_BAD_INPUT) ? GPV_ERR_INVALID : GPV_ERR_DEVICE,
                (ctx->h_stats->status & ST_BAD_INPUT) ? "non-finite vertex" : "device status raised");
  }
  const int64_t P = (int64_t)ctx->h_stats->pairs;
  const int64_t B = (int64_t)ctx->h_u32[0];

  // 3. outputs of Level1, sorted pair lists, Level2
  GPV_CUDA(cudaMallocAsync((void **)&bindex, 4 * std::max<int64_t>(B, 4), s));
  const int64_t l2bytes = gh.level2 ? B * gh.cells : 0;
  GPV_CUDA(cudaMallocAsync((void **)&l2, std::max<int64_t>(l2bytes, 16), s));
  mark(5);
  launch_expand(g, b.bplane, b.iplane, wpre, l1, prefix, bindex, b.stats, s);
  mark(6);
  if (gh.level2 && B > 0) {
    uint32_t *kalt, *valt, *flags, *uidx, *useg, *stmp, *l2tmp;
    GPV_CUDA(ws.get(&kalt, (size_t)P));
    GPV_CUDA(ws.get(&valt, (size_t)P));
    GPV_CUDA(ws.get(&flags, (size_t)P));
    GPV_CUDA(ws.get(&uidx, (size_t)P));
    GPV_CUDA(ws.get(&useg, (size_t)B + 1));
    GPV_CUDA(ws.get(&stmp, (size_t)std::max(sort_temp_words(P), scan_temp_words(P))));
    GPV_CUDA(ws.get(&l2tmp, (size_t)level2_temp_words(B)));
    const bool in_alt = sort_pairs(b.keys, b.vals, kalt, valt, P, gh.key_bits, stmp, s);
    const uint32_t *sk = in_alt ? kalt : b.keys;
    const uint32_t *sv = in_alt ? valt : b.vals;
    launch_heads(sk, P, flags, s);
    scan_u32(flags, uidx, P, d_tot + 1, stmp, s);
    launch_useg(flags, uidx, P, useg, s);
    mark(7);
    launch_level2c(g, b.ptri, b.fbox, sk, sv, useg, prefix, B, l2tmp, l2, b.stats, s);
  } else {
    mark(7);
  }
  mark(8);
  GPV_CUDA(cudaGetLastError());
  GPV_CUDA(cudaMemcpyAsync(ctx->h_stats, b.stats, sizeof(MeshStats), cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaMemcpyAsync(ctx->h_u32 + 1, d_tot + 1, 4, cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaStreamSynchronize(s));
  if (ctx->timing) {
    // stages: 0 prep, 1 level1, 2 fill finish + boundary scan, 3 expand, 4 sort + lists,
    // 5 level2 (event pairs (0,1) (2,3) (3,4) (5,6) (6,7) (7,8))
    const int pr[6][2] = {{0, 1}, {2, 3}, {3, 4}, {5, 6}, {6, 7}, {7, 8}};
    for (int k = 0; k < 6; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ctx->ev[pr[k][0]], ctx->ev[pr[k][1]]) == cudaSuccess)
        ctx->stage_ms[k] += ms;
    }
    ctx->stage_calls++;
  }
  const MeshStats &st = *ctx->h_stats;
  if (st.status) {
    drop_results();
    return fail(ctx, GPV_ERR_DEVICE, "device status raised");
  }
  if (gh.level2 && B > 0 && (int64_t)ctx->h_u32[1] != B) {
    drop_results();
    return fail(ctx, GPV_ERR_DEVICE, "boundary plane and pair lists disagree");
  }

  std::memset(out, 0, sizeof(*out));
  out->spec = *spec;
  for (int a = 0; a < 3; ++a) {
    out->grid_size[a] = gh.g[a];
    out->grid_size2[a] = gh.level2 ? gh.g2[a] : 0.f;
  }
  out->num_level1 = N1;
  out->num_boundary = B;
  out->num_level1_inside = (int64_t)st.l1_inside;
  out->num_level2_inside = (int64_t)st.l2_inside;
  out->num_level2_boundary = (int64_t)st.l2_boundary;
  out->num_pairs = P;
  out->work.sat1 = (int64_t)st.sat1;
  out->work.sat2 = gh.level2 ? P * gh.cells : 0;
  out->work.ray1 = (int64_t)st.ray1;
  out->work.ray2 = (int64_t)st.ray2;
  out->level1_inout = l1;
  out->level1_prefix = prefix;
  out->boundary_index = bindex;
  out->level2_inout = l2;
  out->handle = ctx->next_handle++;
  ctx->owned[out->handle] = {l1, prefix, bindex, l2};
  return GPV_OK;
}

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
  if (cudaMallocHost(&ctx->h_stats, sizeof(MeshStats)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_u32, 64) != cudaSuccess) {
    delete ctx;
    return GPV_ERR_CUDA;
  }
  *out = ctx;
  return GPV_OK;
}

void gpv_destroy(gpv_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  for (auto &kv : ctx->owned) {
    cudaFree(kv.second.l1);
    cudaFree(kv.second.prefix);
    cudaFree(kv.second.bindex);
    cudaFree(kv.second.l2);
  }
  if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
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
  ctx->stage_calls = 0;
  return GPV_OK;
}

int gpv_stage_times(gpv_ctx *ctx, double *ms, int n) {
  if (!ctx || !ms) return GPV_ERR_INVALID;
  for (int i = 0; i < n && i < gpv_ctx::kStages; ++i) ms[i] = ctx->stage_ms[i];
  return (int)ctx->stage_calls;
}

uint64_t gpv_kernel_launches(void) { return gpv::launch_count(); }

int gpv_set_tile(gpv_ctx *ctx, int t) {
  if (!ctx || (t != 32 && t != 64 && t != 128 && t != 256)) return GPV_ERR_INVALID;
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
  return voxelize_impl(ctx, d_tris, num_triangles, spec, out, stream);
}

int gpv_voxelize_host(gpv_ctx *ctx, const float *h_tris, int64_t num_triangles,
                      const gpv_grid_spec *spec, gpv_result *out, cudaStream_t stream) {
  if (!ctx || !spec || !out || num_triangles < 0 || (num_triangles > 0 && !h_tris))
    return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  float *d = nullptr;
  const size_t bytes = (size_t)std::max<int64_t>(num_triangles, 1) * 9 * sizeof(float);
  cudaError_t e = cudaMallocAsync((void **)&d, bytes, stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMallocAsync");
  if (num_triangles > 0) {
    e = cudaMemcpyAsync(d, h_tris, (size_t)num_triangles * 9 * sizeof(float),
                        cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) { cudaFreeAsync(d, stream); return cuda_fail(ctx, e, "cudaMemcpyAsync"); }
  }
  int rc = voxelize_impl(ctx, d, num_triangles, spec, out, stream);
  cudaFreeAsync(d, stream);
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
  if (l2 && res->num_boundary && cells)
    GPV_CUDA(cudaMemcpyAsync(l2, res->level2_inout, res->num_boundary * cells,
                             cudaMemcpyDeviceToHost, s));
  GPV_CUDA(cudaStreamSynchronize(s));
  return GPV_OK;
}

int gpv_result_release(gpv_ctx *ctx, gpv_result *res) {
  if (!ctx || !res) return GPV_ERR_INVALID;
  auto it = ctx->owned.find(res->handle);
  if (it == ctx->owned.end()) return GPV_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaFreeAsync(it->second.l1, 0);
  cudaFreeAsync(it->second.prefix, 0);
  cudaFreeAsync(it->second.bindex, 0);
  cudaFreeAsync(it->second.l2, 0);
  ctx->owned.erase(it);
  res->level1_inout = nullptr;
  res->level1_prefix = nullptr;
  res->boundary_index = nullptr;
  res->level2_inout = nullptr;
  res->handle = 0;
  return GPV_OK;
}

}  // extern "C"
