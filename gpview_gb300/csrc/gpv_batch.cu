// gpv_batch.cu -- host orchestration of a batch of meshes (the plain path is a batch of one).
//
// Two phases, one host synchronisation after each, independent of the number of meshes:
//   1  prep over every triangle of every mesh, the per-mesh pair segments from its candidate
//      counts (on the device), persistent Level1 (tiles of all meshes), fill finish, boundary
//      scan                                              -> per-mesh pair and boundary counts
//   2  Level1 expansion, the per-voxel pair lists (a counting sort by voxel rank; a segmented
//      radix sort when normals need triangle order), persistent Level2 over the column chunks of
//      all meshes                                        -> per-mesh statistics
// Each phase is recorded into a CUDA graph when graphs are enabled (gpv_set_graphs) and replayed
// while its launch arguments repeat; its launch shapes are fixed by the counts read at the phase
// boundary.  A staging kernel at each end of a phase moves the small per-call data between
// page-locked host staging and the device.
// One graph: a call whose meshes and grids repeat the previous call's (device triangles, no
// normals, ray fill, no hierarchy) records both phases as one graph.  The result arrays and the
// second phase's launches take that call's sizes as capacities, a planning kernel (k_plan) puts
// the per-mesh bases and sizes in device memory between the phases, and the second phase's
// kernels read them; a size above its capacity re-runs the call as two phases.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "gpv_ctx.h"

namespace gpv {

// Runs f(i) for i in [0, n) on up to the machine's hardware threads when n is large enough to
// repay the thread start (the per-mesh host work of a batch); inline otherwise.
template <typename F>
void host_parallel_for(int n, F &&f) {
  if (n < 128) {  // below two threads' worth: inline (and no query of the machine)
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  static const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::min(std::min(hw, 16), n / 64);
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      for (int i = t; i < n; i += nt) f(i);
    });
  for (std::thread &x : th) x.join();
}

namespace {

// Per-call workspace carved from the context's slab (256-byte aligned pieces).  Pieces that do
// not fit fall back to stream-ordered allocations, freed at the end of the call; the total need
// is recorded so that the next call grows the slab first.
struct Arena {
  gpv_ctx *ctx;
  cudaStream_t s;
  size_t off = 0;
  std::vector<void *> extra;
  Arena(gpv_ctx *c, cudaStream_t st) : ctx(c), s(st) {}
  template <typename T>
  cudaError_t get(T **p, size_t count) {
    const size_t bytes = (std::max<size_t>(count * sizeof(T), 16) + 255) & ~size_t(255);
    if (ctx->slab && off + bytes <= ctx->slab_cap) {
      *p = reinterpret_cast<T *>(static_cast<char *>(ctx->slab) + off);
      off += bytes;
      return cudaSuccess;
    }
    off += bytes;
    void *q = nullptr;
    cudaError_t e = ctx_malloc_async(ctx, &q, bytes, s);
    if (e == cudaSuccess) extra.push_back(q);
    *p = (T *)q;
    return e;
  }
  ~Arena() {
    for (void *p : extra) cudaFreeAsync(p, s);
    ctx->slab_want = std::max(ctx->slab_want, off);
  }
};

// Grows the slab to the need recorded by earlier calls (the slab is idle between calls).
cudaError_t grow_slab(gpv_ctx *ctx, cudaStream_t s) {
  if (ctx->slab_want <= ctx->slab_cap) return cudaSuccess;
  if (ctx->slab) {
    cudaError_t e = cudaFreeAsync(ctx->slab, s);
    if (e != cudaSuccess) return e;
    ctx->slab = nullptr;
    ctx->slab_cap = 0;
  }
  const size_t want = ctx->slab_want + ctx->slab_want / 8;
  cudaError_t e = cudaMallocAsync(&ctx->slab, want, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ctx->slab = nullptr;
    return cudaSuccess;  // keep going on per-call allocations
  }
  ctx->slab_cap = want;
  return cudaSuccess;
}

size_t al16(size_t v) { return (v + 15) & ~size_t(15); }

// Identity of a call's meshes for the one-graph form: the triangle counts and grids (FNV-1a over
// their bytes).  Equal keys give equal result sizes unless the triangles themselves moved.
uint64_t call_key(int n, const int64_t *T, const gpv_grid_spec *specs) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void *p, size_t bytes) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < bytes; ++i) h = (h ^ c[i]) * 1099511628211ull;
  };
  mix(&n, sizeof(n));
  mix(T, sizeof(int64_t) * (size_t)n);
  mix(specs, sizeof(gpv_grid_spec) * (size_t)n);
  return h;
}

// Word of the page-locked scratch (gpv_ctx::h_u32) where a one-graph call's DevPlan lands.
constexpr int kPlanWord = 32;

// Runs `launches` on stream s, recorded as a CUDA graph when the context asks for graphs.  The
// executable graph of each phase is cached in the context and updated in place when the new
// recording has the same topology; otherwise it is re-instantiated.  If recording fails the
// launches run directly.
template <typename F>
cudaError_t run_phase(gpv_ctx *ctx, int phase, cudaStream_t s, bool &capturing, F &&launches,
                      bool allow_graph = true, const std::vector<uint64_t> *sig = nullptr) {
  if (!ctx->graphs || !allow_graph) {
    launches();
    return cudaGetLastError();
  }
  cudaGraphExec_t &ge = ctx->gexec[phase];
  if (sig && ge && ctx->gsig[phase] == *sig) {
    // same arguments as the cached graph: replay it (recording and updating it again would
    // only reproduce it, while the GPU waits)
    count_launch(ctx->glaunch[phase]);
    ctx->graph_launches++;
    return cudaGraphLaunch(ge, s);
  }
  ctx->gsig[phase].clear();
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    launches();
    return cudaGetLastError();
  }
  capturing = true;
  const uint64_t l0 = launch_count();
  launches();
  const uint64_t nl = launch_count() - l0;
  capturing = false;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (e != cudaSuccess || !graph) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    launches();
    return cudaGetLastError();
  }
  bool ok = false;
  if (ge) {
    cudaGraphExecUpdateResultInfo info;
    ok = cudaGraphExecUpdate(ge, graph, &info) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      cudaGraphExecDestroy(ge);
      ge = nullptr;
    }
  }
  if (!ok) {
    e = cudaGraphInstantiate(&ge, graph, 0);
    ctx->graph_instantiations++;
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      ge = nullptr;
      return e;
    }
  }
  e = cudaGraphLaunch(ge, s);
  ctx->graph_launches++;
  cudaGraphDestroy(graph);
  if (e == cudaSuccess && sig) {
    ctx->gsig[phase] = *sig;
    ctx->glaunch[phase] = nl;
  }
  return e;
}

}  // namespace

int run_batch(gpv_ctx *ctx, int n, const float *const *d_tris, const int64_t *T,
              const gpv_grid_spec *specs, gpv_result *out, cudaStream_t s, const HostSink *sink) {
#define CK(call)                                                    \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) return ctx_cuda_fail(ctx, e_, #call);    \
  } while (0)
  if (n <= 0) return ctx_fail(ctx, GPV_ERR_INVALID, "empty batch");
  if (sink && n != 1) return ctx_fail(ctx, GPV_ERR_INVALID, "host outputs take one mesh");
  using HClock = std::chrono::steady_clock;
  HClock::time_point ht[6];
  ht[0] = HClock::now();
  std::vector<GridHost> gh(n);
  std::vector<int> grc(n, GPV_OK);
  if (n == 1 && ctx->last_gh && std::memcmp(&ctx->last_spec, &specs[0], sizeof(gpv_grid_spec)) == 0) {
    gh[0] = *ctx->last_gh;  // the same grid as the previous single-mesh call
  } else {
    host_parallel_for(n, [&](int m) { grc[m] = grid_derive(specs[m], gh[m]); });
    if (n == 1 && grc[0] == GPV_OK) {
      ctx->last_spec = specs[0];
      ctx->last_gh = std::make_shared<GridHost>(gh[0]);
    }
  }
  for (int m = 0; m < n; ++m) {
    if (grc[m] != GPV_OK)
      return ctx_fail(ctx, GPV_ERR_INVALID, ("invalid grid specification for mesh " + std::to_string(m)).c_str());
    if (T[m] < 0 || T[m] >= ((int64_t)1 << 31) || (T[m] > 0 && !d_tris[m]))
      return ctx_fail(ctx, GPV_ERR_INVALID, "bad triangle count or pointer");
    if (T[m] > 0 && (reinterpret_cast<uintptr_t>(d_tris[m]) & 15u))
      return ctx_fail(ctx, GPV_ERR_INVALID, "triangle buffers must be 16-byte aligned");
  }
  // Level1 tile: the caller's (or the autotuner's), else the largest that still gives every SM
  // three tiles -- larger tiles amortise the per-tile staging and barriers, but a small mesh
  // needs small ones to occupy the GPU (torus262k: 256; a 16k-triangle sphere: 32)
  int tile = ctx->tile;
  if (tile <= 0) {
    int64_t total = 0;
    for (int m = 0; m < n; ++m) total += T[m];
    tile = 256;
    while (tile > 32 && total < (int64_t)tile * 3 * ctx->num_sms) tile >>= 1;
  }
  const int nmode = ctx->normals;
  const bool stencil = ctx->fill == GPV_FILL_STENCIL;
  const size_t nsz = nmode == GPV_NORMALS_FLOAT ? sizeof(float) : 1;  // bytes per normal value

  // ---- sizes and per-mesh bases
  std::vector<int64_t> tab_off(n + 1, 0), res_l1(n + 1, 0), res_pre(n + 1, 0), res_l1n(n + 1, 0),
      res_hier(n + 1, 0);
  std::vector<MeshDesc> md(n);
  int64_t tris = 0, tiles = 0, fwarps = 0, rows = 0, xchunks = 0, words = 0, togg = 0, stgw = 0;
  int max_keybits = 1, warp_words = 0;
  int64_t max_T = 1;
  bool any_l2 = false;
  for (int m = 0; m < n; ++m) {
    const GridHost &g = gh[m];
    MeshDesc &d = md[m];
    std::memset(&d, 0, sizeof(d));
    d.T = T[m];
    d.tri_base = tris;
    d.tile_base = tiles;
    d.fwarp_base = fwarps;
    d.row_base = rows;
    d.xc_base = xchunks;
    d.word_base = words;
    tris += T[m];
    tiles += (T[m] + tile - 1) / tile;
    fwarps += (int64_t)g.n[1] * g.nxw * g.nzw;
    rows += (int64_t)g.n[2] * g.n[1];
    xchunks += ((int64_t)g.n[0] * g.n[1] * g.n[2] + 127) / 128;
    words += (int64_t)g.n[2] * g.n[1] * g.nxw;
    togg += (int64_t)g.n[0] * g.n[1] * g.nzw;
    if (stencil) stgw += 4 * (int64_t)g.n[0] * g.n[1] * g.nzw;
    tab_off[m + 1] = tab_off[m] + table_floats(g);
    res_l1[m + 1] = res_l1[m] + (int64_t)al16(g.N1);
    res_pre[m + 1] = res_pre[m] + (int64_t)al16(g.N1);  // int32 elements, 64-byte aligned
    res_l1n[m + 1] = res_l1n[m] + (int64_t)al16(3 * g.N1 * nsz);  // bytes
    res_hier[m + 1] = res_hier[m] + ((ctx->hierarchy && hierarchy_levels(g.N1)) ? g.N1 - 1 : 0);
    max_keybits = std::max(max_keybits, g.key_bits);
    max_T = std::max(max_T, T[m]);
    any_l2 = any_l2 || g.level2;
  }

  int val_bits = 1;  // bits of the largest triangle id (normals: the sort's value digits)
  while (val_bits < 31 && ((int64_t)1 << val_bits) < max_T) ++val_bits;

  CK(grow_slab(ctx, s));
  Arena ws(ctx, s);
  // coordinate tables: one pinned staging copy
  CK(ctx_ensure_tables(ctx, (size_t)tab_off[n]));
  host_parallel_for(n, [&](int m) { pack_tables(gh[m], ctx->h_tables + tab_off[m]); });
  float *d_tab;
  CK(ws.get(&d_tab, (size_t)tab_off[n]));

  float4 *ptri, *fbox;
  int4 *rng;
  uint32_t *bplane, *iplane, *toggles, *wcnt, *wpre, *wtot, *stmp, *queue;
  MeshStats *stats;
  MeshDesc *d_md;
  CK(ws.get(&ptri, 3 * (size_t)std::max<int64_t>(tris, 1)));
  CK(ws.get(&rng, (size_t)std::max<int64_t>(tris, 1)));
  CK(ws.get(&fbox, (size_t)std::max<int64_t>(tris, 1)));
  // without normals the pair lists are built by a counting sort, which ranks the voxels of the
  // pairs through a second, column-major bit plane after the boundary plane; one popcount and one
  // scan cover both planes
  const bool kmark = nmode == 0 && words > 0;
  const int64_t swords = kmark ? 2 * words : words;
  CK(ws.get(&bplane, (size_t)swords));
  CK(ws.get(&iplane, (size_t)words));
  CK(ws.get(&toggles, (size_t)togg));
  CK(ws.get(&wcnt, (size_t)swords));
  CK(ws.get(&wpre, (size_t)swords));
  CK(ws.get(&wtot, 4));
  CK(ws.get(&stmp, (size_t)scan_temp_words(swords)));
  // the boundary-voxel total: past the boundary plane's words in the prefix when both are scanned
  const uint32_t *btot = kmark ? wpre + words : wtot;
  CK(ws.get(&queue, 1 + kMaxSlabs));  // [0] Level1 tickets, [1 + k] Level2 tickets of slab k
  // z slabs of the Level2 launch when the outputs go to the host (one mesh): the boundary ranks
  // at up to kMaxSlabs fine slab starts are read with the first phase's counts; the launch then
  // groups fine slabs into as many slabs as the Level2 output size calls for
  int fslab = 1, fz = 0, nslab = 1, zslab = 0;
  uint32_t *d_slab = nullptr;
  if (sink && gh[0].level2) {
    fslab = std::min(kMaxSlabs, gh[0].n[2]);
    fz = (gh[0].n[2] + fslab - 1) / fslab;
    fslab = (gh[0].n[2] + fz - 1) / fz;
    CK(ws.get(&d_slab, kMaxSlabs + 1));
  }
  CK(ws.get(&stats, (size_t)n));
  CK(ws.get(&d_md, (size_t)n));
  uint32_t *stg = nullptr;  // stencil fill: Level1 sample-column toggles
  if (stencil) CK(ws.get(&stg, (size_t)stgw));
  float4 *fnorm = nullptr;
  if (nmode) CK(ws.get(&fnorm, (size_t)std::max<int64_t>(tris, 1)));

  // result arenas (shared by the batch's results, freed when the last one is released)
  auto set = std::make_shared<ResultSet>();
  set->stream = s;
  CK(ctx_malloc_async(ctx, &set->l1, std::max<int64_t>(res_l1[n], 16), s));
  CK(ctx_malloc_async(ctx, &set->prefix, 4 * std::max<int64_t>(res_pre[n], 16), s));
  if (res_hier[n] > 0) CK(ctx_malloc_async(ctx, &set->hier, sizeof(gpv_box) * res_hier[n], s));
  if (nmode) {
    // voxels without recorded triangles keep the zero normal: 0.0f, or byte 127 (0 * scale + 127)
    CK(ctx_malloc_async(ctx, &set->l1n, std::max<int64_t>(res_l1n[n], 16), s));
    CK(cudaMemsetAsync(set->l1n, nmode == GPV_NORMALS_FLOAT ? 0 : 127, res_l1n[n], s));
  }

  int64_t togg_off = 0, stg_off = 0;
  for (int m = 0; m < n; ++m) {
    MeshDesc &d = md[m];
    const GridHost &g = gh[m];
    d.g = make_griddev(g, d_tab + tab_off[m]);
    d.tris = d_tris[m];
    d.ptri = ptri + 3 * d.tri_base;
    d.rng = rng + d.tri_base;
    d.fbox = fbox + d.tri_base;
    d.bplane = bplane + d.word_base;
    d.iplane = iplane + d.word_base;
    d.toggles = toggles + togg_off;
    togg_off += (int64_t)g.n[0] * g.n[1] * g.nzw;
    if (stg) {
      d.stg = stg + stg_off;
      stg_off += 4 * (int64_t)g.n[0] * g.n[1] * g.nzw;
    }
    d.stats = stats + m;
    d.l1 = static_cast<uint8_t *>(set->l1) + res_l1[m];
    d.prefix = static_cast<int32_t *>(set->prefix) + res_pre[m];
    d.ch = g.level2 ? level2_chunk(d.g, ctx->l2_chunk_cap) : 1;
    d.has_l2 = g.level2 ? 1 : 0;
    d.fnorm = fnorm ? fnorm + d.tri_base : nullptr;
    d.l1n = nmode ? static_cast<uint8_t *>(set->l1n) + res_l1n[m] : nullptr;
    if (g.level2)
      warp_words = std::max(warp_words, level2_warp_words(d.g, ctx->l2_chunk_cap, stencil));
  }
  BatchDev bd;
  bd.md = d_md;
  bd.nmesh = n;
  bd.tile = tile;
  bd.total_tris = tris;
  bd.total_tiles = tiles;
  bd.total_fwarps = fwarps;
  bd.total_rows = rows;
  bd.total_xchunks = xchunks;
  bd.total_words = words;
  bd.queue = queue;
  bd.normals = nmode;
  bd.fill = ctx->fill;
  bd.stp = nullptr;
  bd.stp_words = 0;
  bd.kmask = kmark ? bplane + words : nullptr;
  bd.wait_limit = ctx->wait_limit;
  bd.fail_wait = ctx->fail_wait;
  CK(ctx_ensure_host(ctx, (size_t)n));
  std::memcpy(ctx->h_md, md.data(), n * sizeof(MeshDesc));

  bool capturing = false;
  auto mark = [&](int i) {
    if (!ctx->timing) return;
    if (capturing) cudaEventRecordWithFlags(ctx->ev[i], s, cudaEventRecordExternal);
    else cudaEventRecord(ctx->ev[i], s);
  };
  auto fail_all = [&](int code, const char *msg) {
    cudaFreeAsync(set->l1, s);
    cudaFreeAsync(set->prefix, s);
    if (set->bindex) cudaFreeAsync(set->bindex, s);
    if (set->l2 && !set->l2_external) cudaFreeAsync(set->l2, s);
    if (set->l1n) cudaFreeAsync(set->l1n, s);
    if (set->l2n) cudaFreeAsync(set->l2n, s);
    if (set->hier) cudaFreeAsync(set->hier, s);
    set->l1 = set->prefix = set->bindex = set->l2 = set->l1n = set->l2n = set->hier = nullptr;
    return ctx_fail(ctx, code, msg);
  };

  // ---- phase 1 (one recording): prep, per-mesh pair bases on the device (no host round trip:
  // the pair buffer has the context's capacity hint; a mesh that does not fit raises
  // ST_PAIR_OVERFLOW and the call re-runs with the exact capacity), Level1, fill finish,
  // boundary scan.
  int64_t pair_cap = std::max<int64_t>(ctx->pair_hint, std::max<int64_t>(16 * tris, 1 << 16));
  if (ctx->debug_pair_cap > 0) {  // failure-detection hook: a first capacity that overflows
    pair_cap = ctx->debug_pair_cap;
    ctx->debug_pair_cap = 0;
  }
  uint32_t *keys, *vals;
  CK(ws.get(&keys, (size_t)pair_cap));
  CK(ws.get(&vals, (size_t)pair_cap));
  ht[1] = HClock::now();
  // every value the phase's launches take (the per-mesh data reaches the kernels through d_md)
  auto bd_sig = [&](std::vector<uint64_t> &v) {
    for (uint64_t x : {(uint64_t)(uintptr_t)bd.md, (uint64_t)bd.nmesh, (uint64_t)bd.tile,
                       (uint64_t)bd.total_tris, (uint64_t)bd.total_tiles, (uint64_t)bd.total_fwarps,
                       (uint64_t)bd.total_rows, (uint64_t)bd.total_words, (uint64_t)bd.total_xchunks,
                       (uint64_t)(uintptr_t)bd.queue, (uint64_t)bd.normals, (uint64_t)bd.fill,
                       (uint64_t)(uintptr_t)bd.stp, (uint64_t)bd.stp_words,
                       (uint64_t)ctx->timing, (uint64_t)ctx->num_sms, (uint64_t)bd.wait_limit,
                       (uint64_t)bd.fail_wait})
      v.push_back(x);
  };
  std::vector<uint64_t> sig0;
  bd_sig(sig0);
  for (uint64_t x : {(uint64_t)(uintptr_t)d_md, (uint64_t)(uintptr_t)keys, (uint64_t)(uintptr_t)vals,
                     (uint64_t)pair_cap, (uint64_t)(uintptr_t)bplane, (uint64_t)words,
                     (uint64_t)(uintptr_t)wcnt, (uint64_t)(uintptr_t)wpre, (uint64_t)(uintptr_t)wtot,
                     (uint64_t)(uintptr_t)stmp, (uint64_t)(uintptr_t)d_slab,
                     (uint64_t)(d_slab ? (int64_t)gh[0].n[1] * gh[0].nxw : 0),
                     (uint64_t)(d_slab ? gh[0].n[2] : 0), (uint64_t)fz, (uint64_t)fslab,
                     (uint64_t)(uintptr_t)d_tab, (uint64_t)(uintptr_t)ctx->h_tables,
                     (uint64_t)tab_off[n], (uint64_t)(uintptr_t)ctx->h_md,
                     (uint64_t)(uintptr_t)ctx->h_stats, (uint64_t)(uintptr_t)ctx->h_u32,
                     (uint64_t)(uintptr_t)stats, (uint64_t)(uintptr_t)toggles, (uint64_t)togg,
                     (uint64_t)(uintptr_t)stg, (uint64_t)stgw})
    sig0.push_back(x);
  // the first half: prep, pair segments, Level1, fill finish, boundary scan (one-graph calls
  // also clear the second half's voxel counts, clr_words words, and its completed-voxel counter)
  auto phase1_launches = [&](uint32_t *clr, int64_t clr_words) {
    // this call's tables and descriptors in (read from page-locked staging), the accumulators
    // cleared: one kernel
    StageList in(ctx->num_sms, s);
    in.copy(d_tab, ctx->h_tables, tab_off[n] * sizeof(float));
    in.copy(d_md, ctx->h_md, n * sizeof(MeshDesc));
    in.clear(stats, n * sizeof(MeshStats));
    in.clear(bplane, swords * 4);
    in.clear(toggles, togg * 4);
    if (stg) in.clear(stg, stgw * 4);
    if (clr) {
      in.clear(clr, clr_words * 4);
      in.clear(wtot + 1, 4);
    }
    in.launch();
    mark(0);
    launch_prep(bd, s);
    mark(1);
    launch_pair_bases(bd, d_md, keys, vals, pair_cap, s);
    mark(2);
    launch_level1(bd, ctx->num_sms, s);
    if (stencil) launch_stencil1(bd, s);
    mark(3);
    launch_fill_finish(bd, s);
    launch_popc(bplane, swords, wcnt, s);
    scan_u32(wcnt, wpre, swords, wtot, stmp, s);
    launch_boundary_counts(bd, wpre, btot, s);
    if (d_slab)
      launch_slab_offsets(wpre, btot, (int64_t)gh[0].n[1] * gh[0].nxw, gh[0].n[2], fz, fslab,
                          d_slab, s);
    mark(4);
  };
  // the ray fill's u/v-passing items queued before their per-voxel work: measured faster with
  // Level2 grids of up to 8^3 cells (the Level2 kernel on torus262k 0.596 -> 0.550 ms, on a 16k
  // sphere at 4^3 0.146 -> 0.129 ms, on 512 meshes of the batched workload 36.6 -> 36.0 ms) and
  // slower at 16^3 (star1310k 3.94 -> 4.21 ms)
  bool l2_fillq = !stencil && any_l2;
  for (int m = 0; m < n; ++m)
    if (gh[m].level2 && gh[m].cells > kFillQueueCells) l2_fillq = false;
  // per-stage event times of this call (timing on)
  auto take_stage_times = [&] {
    if (!ctx->timing) return;
    // stages: 0 prep, 1 level1, 2 fill finish + boundary scan, 3 expand, 4 sort + lists,
    // 5 level2 (work items + kernel), 6 the Level2 kernel alone, 7 per-mesh pair bases,
    // 8 between the halves (counts out, host planning, second launch, uploads in; one-graph
    // calls: the planning kernel)
    const int pr[9][2] = {{0, 1}, {2, 3}, {3, 4}, {5, 6}, {6, 7}, {7, 8}, {9, 8}, {1, 2}, {4, 5}};
    for (int k = 0; k < 9; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ctx->ev[pr[k][0]], ctx->ev[pr[k][1]]) == cudaSuccess)
        ctx->stage_ms[k] += ms;
    }
    ctx->stage_calls++;
  };
  // results: per-mesh slices of the result arrays, given the boundary-index and Level2 offsets
  auto assemble = [&](const std::vector<int64_t> &boff, const std::vector<int64_t> &l2off) {
    uint64_t handle;
    {
      std::lock_guard<std::mutex> lk(ctx->owned_mu);
      handle = ctx->next_handle++;
      set->refs = n;
      ctx->owned[handle] = set;
    }
    for (int m = 0; m < n; ++m) {
      const MeshStats &st = ctx->h_stats[m];
      gpv_result &r = out[m];
      std::memset(&r, 0, sizeof(r));
      r.spec = specs[m];
      for (int a = 0; a < 3; ++a) {
        r.grid_size[a] = gh[m].g[a];
        r.grid_size2[a] = gh[m].level2 ? gh[m].g2[a] : 0.f;
      }
      r.num_level1 = gh[m].N1;
      r.num_boundary = (int64_t)st.boundary;
      r.num_level1_inside = (int64_t)st.l1_inside;
      r.num_level2_inside = (int64_t)st.l2_inside;
      r.num_level2_boundary = (int64_t)st.l2_boundary;
      r.num_pairs = (int64_t)st.pairs;
      r.work.sat1 = (int64_t)st.sat1;
      r.work.sat2 = gh[m].level2 ? (int64_t)st.pairs * gh[m].cells : 0;
      r.work.ray1 = (int64_t)st.ray1;
      r.work.ray2 = (int64_t)st.ray2;
      r.level1_inout = static_cast<uint8_t *>(set->l1) + res_l1[m];
      r.level1_prefix = static_cast<int32_t *>(set->prefix) + res_pre[m];
      r.boundary_index = static_cast<int32_t *>(set->bindex) + boff[m];
      r.level2_inout = static_cast<uint8_t *>(set->l2) + l2off[m];
      r.handle = handle;
      r.normal_mode = nmode;
      if (res_hier[m + 1] > res_hier[m]) {
        r.hierarchy = static_cast<gpv_box *>(set->hier) + res_hier[m];
        r.hierarchy_levels = hierarchy_levels(gh[m].N1);
      }
      if (nmode) {
        r.level1_normal = static_cast<uint8_t *>(set->l1n) + res_l1n[m];
        r.level2_normal = static_cast<uint8_t *>(set->l2n) + 3 * l2off[m] * nsz;
      }
    }
  };
  auto take_host_times = [&] {
    if (!ctx->timing) return;
    ht[5] = HClock::now();
    for (int k = 0; k < 5; ++k)
      ctx->host_ms[k] += std::chrono::duration<double, std::milli>(ht[k + 1] - ht[k]).count();
  };

  // ---- one graph for the whole call, when the meshes and grids repeat the previous call's
  const uint64_t key = call_key(n, T, specs);
  const bool og_path = ctx->graphs && ctx->one_graph && !sink && nmode == 0 && !stencil &&
                       res_hier[n] == 0;
  const bool og_skip = ctx->og_skip;  // (one-shot: the re-run of a call that did not fit)
  ctx->og_skip = false;
  if (og_path && !og_skip && ctx->og_key == key && ctx->og_caps.B > 0) {
    PlanCaps cap = ctx->og_caps;
    if (ctx->debug_og_cap > 0) {  // failure-detection hook: a boundary capacity that overflows
      cap.B = ctx->debug_og_cap;
      ctx->debug_og_cap = 0;
    }
    DevPlan *d_plan;
    uint32_t *kalt = nullptr, *valt = nullptr, *cnt = nullptr, *useg = nullptr, *sortmp = nullptr,
             *l2tmp = nullptr;
    CK(ws.get(&d_plan, 1));
    if (any_l2) {
      CK(ws.get(&kalt, (size_t)cap.P));
      CK(ws.get(&valt, (size_t)cap.P));
      CK(ws.get(&cnt, (size_t)cap.U + 1));
      CK(ws.get(&useg, (size_t)cap.U + 1));
      CK(ws.get(&sortmp, (size_t)scan_temp_words(cap.U + 1)));
      CK(ws.get(&l2tmp, (size_t)level2_temp_words(cap.U)));
    }
    CK(ctx_malloc_async(ctx, &set->bindex, 4 * std::max<int64_t>(cap.B, 4), s));
    CK(ctx_malloc_async(ctx, &set->l2, std::max<int64_t>(cap.l2bytes, 16), s));
    BatchDev bdp = bd;
    bdp.plan = d_plan;
    std::vector<uint64_t> sig2 = sig0;
    for (uint64_t x : {(uint64_t)cap.B, (uint64_t)cap.U, (uint64_t)cap.l2bytes, (uint64_t)cap.tiles,
                       (uint64_t)cap.P,
                       (uint64_t)(uintptr_t)d_plan, (uint64_t)(uintptr_t)kalt,
                       (uint64_t)(uintptr_t)valt, (uint64_t)(uintptr_t)cnt, (uint64_t)(uintptr_t)useg,
                       (uint64_t)(uintptr_t)sortmp, (uint64_t)(uintptr_t)l2tmp,
                       (uint64_t)(uintptr_t)set->l1, (uint64_t)(uintptr_t)set->prefix,
                       (uint64_t)(uintptr_t)set->bindex, (uint64_t)(uintptr_t)set->l2,
                       (uint64_t)warp_words, (uint64_t)l2_fillq, (uint64_t)ctx->l2_mode,
                       (uint64_t)any_l2})
      sig2.push_back(x);
    CK(run_phase(ctx, 2, s, capturing, [&] {
      phase1_launches(cnt, any_l2 ? cap.U + 1 : 0);
      // the second half's bases and sizes, on the device
      launch_plan(bdp, d_md, static_cast<int32_t *>(set->bindex), static_cast<uint8_t *>(set->l2),
                  cap, ctx->l2_mode, d_plan, s);
      mark(5);
      launch_expand(bdp, wpre, s);
      mark(6);
      if (any_l2) {
        count_sort_pairs(bdp, nullptr, cap.tiles, keys, vals, wpre + words, cap.U, cap.P, cnt,
                         useg, kalt, valt, wtot + 1, sortmp, s);
        mark(7);
        launch_level2(bdp, kalt, valt, useg, cap.U, l2tmp, warp_words, ctx->num_sms, s,
                      [&] { mark(9); }, 0, 1, {}, 0, nullptr, true, l2_fillq);
      } else {
        mark(7);
        mark(9);
      }
      mark(8);
      StageList out(ctx->num_sms, s);
      out.copy(ctx->h_stats, stats, n * sizeof(MeshStats));
      out.copy(ctx->h_u32, wtot, 8);
      out.copy(ctx->h_u32 + kPlanWord, d_plan, sizeof(DevPlan));
      out.launch();
    }, true, &sig2));
    CK(cudaStreamSynchronize(s));
    ht[2] = ht[3] = ht[4] = HClock::now();
    DevPlan pl;
    std::memcpy(&pl, ctx->h_u32 + kPlanWord, sizeof(DevPlan));
    bool overflow = false, raised = false;
    int64_t need = 0;
    for (int m = 0; m < n; ++m) {
      const MeshStats &st = ctx->h_stats[m];
      if (st.status & ST_BAD_INPUT) return fail_all(GPV_ERR_INVALID, "non-finite vertex");
      overflow = overflow || (st.status & ST_PAIR_OVERFLOW);
      raised = raised || st.status;
      need += (int64_t)st.sat1;
    }
    if (overflow || !pl.ok) {
      // a record buffer or a recorded capacity too small: the call runs again with exact sizes
      // (two halves), which also records this call's sizes for the next one-graph call
      if (overflow) {
        if (pair_cap >= need) return fail_all(GPV_ERR_DEVICE, "pair buffer overflow");
        ctx->pair_hint = std::max(ctx->pair_hint, need + need / 8);
        ctx->replans++;
      } else {
        if (raised) return fail_all(GPV_ERR_DEVICE, "device status raised in Level1");
        ctx->og_replans++;
      }
      // the re-run takes two phases (the exact sizes) and records them, merged with these
      ctx->og_skip = true;
      fail_all(GPV_OK, "");
      ctx->err.clear();
      return run_batch(ctx, n, d_tris, T, specs, out, s);
    }
    take_stage_times();
    if (any_l2 && (int64_t)ctx->h_u32[1] != (int64_t)pl.ub)
      return fail_all(GPV_ERR_DEVICE, "boundary plane and pair lists disagree");
    // the offsets the planning kernel gave each mesh
    std::vector<int64_t> l2off(n + 1, 0), boff(n + 1, 0);
    for (int m = 0; m < n; ++m) {
      const MeshStats &st = ctx->h_stats[m];
      boff[m + 1] = boff[m] + (int64_t)st.boundary;
      l2off[m + 1] = l2off[m] + (gh[m].level2 ? (int64_t)st.boundary * gh[m].cells : 0);
    }
    assemble(boff, l2off);
    ctx->og_calls++;
    take_host_times();
    return GPV_OK;
  }

  CK(run_phase(ctx, 0, s, capturing, [&] {
    phase1_launches(nullptr, 0);
    // counts out, written straight into page-locked staging
    StageList out(ctx->num_sms, s);
    if (d_slab) out.copy(ctx->h_u32 + 4, d_slab, 4 * (fslab + 1));
    out.copy(ctx->h_stats, stats, n * sizeof(MeshStats));
    out.launch();
  }, true, &sig0));
  CK(cudaStreamSynchronize(s));
  ht[2] = HClock::now();
  {
    // the same bases the device computed, for the host copy of the descriptors
    int64_t caps = 0, need = 0;
    bool overflow = false;
    for (int m = 0; m < n; ++m) {
      const MeshStats &st = ctx->h_stats[m];
      if (st.status & ST_BAD_INPUT) return fail_all(GPV_ERR_INVALID, "non-finite vertex");
      overflow = overflow || (st.status & ST_PAIR_OVERFLOW);
      const int64_t want = (int64_t)st.sat1;
      md[m].emit_base = caps;
      md[m].pair_cap = std::max<int64_t>(0, std::min<int64_t>(want, pair_cap - caps));
      md[m].keys = keys + std::min<int64_t>(caps, pair_cap);
      md[m].vals = vals + std::min<int64_t>(caps, pair_cap);
      caps += want;
      need += want;
    }
    if (overflow) {
      // a buffer that held every candidate test cannot overflow: something else is wrong
      if (pair_cap >= need) return fail_all(GPV_ERR_DEVICE, "pair buffer overflow");
      ctx->pair_hint = std::max(ctx->pair_hint, need + need / 8);
      ctx->replans++;
      fail_all(GPV_OK, "");
      ctx->err.clear();
      return run_batch(ctx, n, d_tris, T, specs, out, s);
    }
  }
  int64_t Btot = 0, l2bytes = 0, P2 = 0, ub = 0;
  std::vector<int64_t> l2off(n + 1, 0), boff(n + 1, 0);
  for (int m = 0; m < n; ++m) {
    const MeshStats &st = ctx->h_stats[m];
    if (st.status) return fail_all(GPV_ERR_DEVICE, "device status raised in Level1");
    // dense pair / boundary-voxel bases over the sorted meshes: those with a Level2 stage, and
    // every mesh when normals are on
    md[m].pair_base = P2;
    md[m].u_base = ub;
    if (gh[m].level2 || nmode) {
      P2 += (int64_t)st.pairs;
      ub += (int64_t)st.boundary;
    }
    Btot += (int64_t)st.boundary;
    boff[m + 1] = Btot;
    l2off[m + 1] = l2off[m] + (gh[m].level2 ? (int64_t)st.boundary * gh[m].cells : 0);
  }
  l2bytes = l2off[n];
  // host outputs into pinned memory: the Level2 kernel writes its bytes there itself (over the
  // CPU-GPU link while it computes) instead of into device memory followed by copies
  const bool l2_direct = sink && sink->l2_dev && gh[0].level2 && sink->l2_cap >= l2bytes;
  // packed Level2 host output (gpv_set_host_expand): the slabs in the context's mask send 2-bit
  // codes into page-locked staging, a quarter of the bytes over the link, and host threads
  // expand each finished slab into the caller's buffer while later slabs compute.  It needs the
  // 16-cell output layout (n2z 8 or 16, a multiple of 16 sub-columns per layer, an aligned
  // buffer) and pays only for large outputs.
  bool packed = l2_direct && ctx->host_threads != 0 && ctx->host_threads != 1 &&
                ctx->packed_slabs != 0 && ctx->packed_share > 0 &&
                (gh[0].n2[2] == 8 || gh[0].n2[2] == 16) &&
                ((gh[0].n2[0] * gh[0].n2[1]) & 15) == 0 && l2bytes >= ctx->packed_min_bytes &&
                sink->nslab == 0 && (reinterpret_cast<uintptr_t>(sink->l2_dev) & 15) == 0;
  if (packed) {
    const size_t words = (size_t)(l2bytes / 16);
    if (ctx->h_codes_cap < words) {
      if (ctx->h_codes) cudaFreeHost(ctx->h_codes);
      ctx->h_codes = nullptr;
      ctx->h_codes_cap = 0;
      if (cudaMallocHost(&ctx->h_codes, words * sizeof(uint32_t)) == cudaSuccess) ctx->h_codes_cap = words;
      else cudaGetLastError();
    }
    if (!ctx->pool && ctx->h_codes_cap >= words) {
      const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
      ctx->pool.reset(new ExpandPool(ctx->host_threads > 1 ? ctx->host_threads : std::min(hw, 16)));
    }
    uint32_t *dcodes = nullptr;
    packed = ctx->h_codes_cap >= words && ctx->pool &&
             cudaHostGetDevicePointer((void **)&dcodes, ctx->h_codes, 0) == cudaSuccess && dcodes;
    if (!packed) cudaGetLastError();  // the Level2 kernel writes bytes instead
    md[0].l2codes = packed ? dcodes : nullptr;
  }
  CK(ctx_malloc_async(ctx, &set->bindex, 4 * std::max<int64_t>(Btot, 4), s));
  if (l2_direct) {
    set->l2 = sink->l2_dev;
    set->l2_external = true;
  } else {
    CK(ctx_malloc_async(ctx, &set->l2, std::max<int64_t>(l2bytes, 16), s));
  }
  if (nmode) {
    CK(ctx_malloc_async(ctx, &set->l2n, std::max<int64_t>(3 * l2bytes * (int64_t)nsz, 16), s));
    for (int m = 0; m < n; ++m) md[m].l2n = static_cast<uint8_t *>(set->l2n) + 3 * l2off[m] * nsz;
  }
  for (int m = 0; m < n; ++m) {
    md[m].bindex = static_cast<int32_t *>(set->bindex) + boff[m];
    md[m].l2 = static_cast<uint8_t *>(set->l2) + l2off[m];
  }
  // sort tiles
  std::vector<SortTile> st_host;
  std::vector<int64_t> stb(n + 1, 0);
  for (int m = 0; m < n; ++m) {
    const int64_t Pm = (int64_t)ctx->h_stats[m].pairs;
    const int64_t nt = (gh[m].level2 || nmode) ? (Pm + kSortTileItems - 1) / kSortTileItems : 0;
    for (int64_t j = 0; j < nt; ++j)
      st_host.push_back({m, (int32_t)j, (int32_t)std::min<int64_t>(kSortTileItems, Pm - j * kSortTileItems), 0});
    stb[m + 1] = stb[m] + nt;
  }
  std::memcpy(ctx->h_md, md.data(), n * sizeof(MeshDesc));

  // ---- phase 2: allocations and staging first, then the recorded launch sequence
  const int64_t ntiles = (int64_t)st_host.size();
  const bool do_l2 = (any_l2 || nmode) && ntiles > 0;  // sort + lists (+ Level2, normals)
  const bool csort = do_l2 && kmark;                   // lists by the counting sort
  SortTile *d_tiles = nullptr;
  int64_t *d_tb = nullptr;
  uint32_t *kalt = nullptr, *valt = nullptr, *flags = nullptr, *uidx = nullptr, *useg = nullptr,
           *sortmp = nullptr, *l2tmp = nullptr;
  if (do_l2) {
    CK(ctx_ensure_host_tiles(ctx, (size_t)ntiles, (size_t)n + 1));
    std::memcpy(ctx->h_tiles, st_host.data(), ntiles * sizeof(SortTile));
    std::memcpy(ctx->h_tb, stb.data(), (n + 1) * sizeof(int64_t));
    CK(ws.get(&d_tiles, (size_t)ntiles));
    CK(ws.get(&d_tb, (size_t)n + 1));
    CK(ws.get(&kalt, (size_t)std::max<int64_t>(P2, 1)));
    CK(ws.get(&valt, (size_t)std::max<int64_t>(P2, 1)));
    CK(ws.get(&flags, (size_t)std::max<int64_t>(P2, ub)));  // the counting sort's counts too
    CK(ws.get(&uidx, (size_t)P2));
    CK(ws.get(&useg, (size_t)ub + 1));
    CK(ws.get(&sortmp, (size_t)std::max({sort_seg_temp_words(ntiles), scan_temp_words(P2),
                                         scan_temp_words(ub)})));
    CK(ws.get(&l2tmp, (size_t)level2_temp_words(ub)));
    if (stencil && any_l2) {  // per boundary voxel: the column prefix of sample coverage
      for (int m = 0; m < n; ++m)
        if (gh[m].level2) bd.stp_words = std::max(bd.stp_words, (4 * gh[m].n2[0] * gh[m].n2[1] + 31) / 32);
      CK(ws.get(&bd.stp, (size_t)std::max<int64_t>(ub, 1) * bd.stp_words));
    }
  }
  ht[3] = HClock::now();
  // host outputs: Level1 arrays copied as soon as the expansion has written them, Level2 slab by
  // slab, on the context's copy stream (this phase then runs without a graph)
  bool l2_copied = true;
  if (sink) {
    if (!ctx->cstream) CK(cudaStreamCreateWithFlags(&ctx->cstream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : ctx->cev)
      if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!ctx->slab_aux.st[0]) {
      for (cudaStream_t &x : ctx->slab_aux.st) CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&ctx->slab_aux.fork, cudaEventDisableTiming));
      for (cudaEvent_t &e : ctx->slab_aux.join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    l2_copied = !gh[0].level2 || l2_direct || (sink->l2 && sink->l2_cap >= l2bytes);
  }
  cudaStream_t cs = ctx->cstream;
  uint32_t slab_off[kMaxSlabs + 1] = {};
  if (d_slab) {
    // slab count: the caller's, or one per 12 MB of Level2 output (the copy of each slab then
    // overlaps the computation of the next; smaller slabs cost more than they hide)
    int want = sink->nslab > 0 ? sink->nslab
               : packed        ? kMaxSlabs
               : l2_direct     ? 1
                               : (int)std::min<int64_t>(kCopySlabs, l2bytes / (12ll << 20));
    want = std::max(1, std::min(want, fslab));
    const int gsz = (fslab + want - 1) / want;
    zslab = gsz * fz;
    nslab = (fslab + gsz - 1) / gsz;
    for (int k = 0; k <= nslab; ++k) slab_off[k] = ctx->h_u32[4 + std::min(k * gsz, fslab)];
  }
  // packed output: the first share of each masked slab's boundary voxels (output order)
  for (int k = 0; k < kMaxSlabs; ++k) {
    bd.pk_end[k] = 0;
    if (!packed || k >= std::max(nslab, 1) || !((ctx->packed_slabs >> k) & 1u)) continue;
    const uint32_t lo = d_slab ? slab_off[k] : 0u, hi = d_slab ? slab_off[k + 1] : (uint32_t)Btot;
    bd.pk_end[k] = lo + (uint32_t)(((uint64_t)(hi - lo) * (uint64_t)ctx->packed_share + 99) / 100);
  }
  // host outputs: recorded too when only page-locked Level1 copies ride along (direct Level2)
  const bool phase1_graph = !sink || (l2_direct && sink->l1_pinned && !packed);
  bool l2_queue = true;
  {
    std::unique_ptr<bool[]> has_l2(new bool[n]);
    for (int m = 0; m < n; ++m) has_l2[m] = gh[m].level2;
    l2_queue = ctx->l2_mode == GPV_LEVEL2_QUEUED   ? true
               : ctx->l2_mode == GPV_LEVEL2_INLINE ? false
                                                   : level2_queue_pays(ctx->h_stats, has_l2.get(), n);
  }
  std::vector<uint64_t> sig1;
  bool any_hier = false;
  for (int m = 0; m < n; ++m) any_hier = any_hier || res_hier[m + 1] > res_hier[m];
  bd_sig(sig1);
  for (uint64_t x : {(uint64_t)(uintptr_t)wpre, (uint64_t)do_l2, (uint64_t)(uintptr_t)d_tiles,
                     (uint64_t)(uintptr_t)d_tb, (uint64_t)ntiles, (uint64_t)(uintptr_t)keys,
                     (uint64_t)(uintptr_t)vals, (uint64_t)(uintptr_t)kalt, (uint64_t)(uintptr_t)valt,
                     (uint64_t)P2, (uint64_t)max_keybits, (uint64_t)nmode, (uint64_t)val_bits,
                     (uint64_t)(uintptr_t)sortmp, (uint64_t)(uintptr_t)flags, (uint64_t)(uintptr_t)uidx,
                     (uint64_t)(uintptr_t)wtot, (uint64_t)(uintptr_t)useg, (uint64_t)any_l2,
                     (uint64_t)ub, (uint64_t)(uintptr_t)l2tmp, (uint64_t)warp_words, (uint64_t)zslab,
                     (uint64_t)nslab, (uint64_t)gh[0].n[2], (uint64_t)(sink != nullptr),
                     (uint64_t)(uintptr_t)(sink ? sink->l1 : nullptr),
                     (uint64_t)(uintptr_t)(sink ? sink->prefix : nullptr),
                     (uint64_t)(uintptr_t)(sink ? sink->bindex : nullptr), (uint64_t)gh[0].N1,
                     (uint64_t)Btot, (uint64_t)(uintptr_t)set->l1, (uint64_t)(uintptr_t)set->prefix,
                     (uint64_t)(uintptr_t)set->bindex, (uint64_t)(uintptr_t)cs, (uint64_t)l2_queue,
                     (uint64_t)l2_fillq,
                     (uint64_t)n, (uint64_t)(uintptr_t)d_md, (uint64_t)(uintptr_t)ctx->h_md,
                     (uint64_t)(uintptr_t)ctx->h_tiles, (uint64_t)(uintptr_t)ctx->h_tb,
                     (uint64_t)(uintptr_t)stats, (uint64_t)(uintptr_t)ctx->h_stats,
                     (uint64_t)(uintptr_t)ctx->h_u32})
    sig1.push_back(x);
  CK(run_phase(ctx, 1, s, capturing, [&] {
    // the descriptors with their output bases, and the sort tiles, read from page-locked staging
    StageList in(ctx->num_sms, s);
    in.copy(d_md, ctx->h_md, n * sizeof(MeshDesc));
    if (do_l2) {
      in.copy(d_tiles, ctx->h_tiles, ntiles * sizeof(SortTile));
      in.copy(d_tb, ctx->h_tb, (n + 1) * sizeof(int64_t));
    }
    if (csort) {
      in.clear(flags, ub * 4);  // the voxel counts
      in.clear(wtot + 1, 4);    // voxels completed
    }
    in.launch();
    mark(5);
    launch_expand(bd, wpre, s);
    if (sink) {
      cudaEventRecord(ctx->cev[0], s);
      cudaStreamWaitEvent(cs, ctx->cev[0], 0);
      if (sink->l1) cudaMemcpyAsync(sink->l1, set->l1, gh[0].N1, cudaMemcpyDeviceToHost, cs);
      if (sink->prefix)
        cudaMemcpyAsync(sink->prefix, set->prefix, 4 * gh[0].N1, cudaMemcpyDeviceToHost, cs);
      if (sink->bindex && Btot)
        cudaMemcpyAsync(sink->bindex, set->bindex, 4 * Btot, cudaMemcpyDeviceToHost, cs);
    }
    for (int m = 0; m < n; ++m)
      if (res_hier[m + 1] > res_hier[m])
        launch_hierarchy(md[m].g, md[m].iplane, static_cast<gpv_box *>(set->hier) + res_hier[m], s);
    mark(6);
    if (do_l2) {
      const uint32_t *sk = kalt, *sv = valt;
      if (csort) {
        // lists in any triangle order: counting sort by voxel rank, segment starts from its scan
        count_sort_pairs(bd, d_tiles, ntiles, keys, vals, wpre + words, ub, P2, flags, useg, kalt,
                         valt, wtot + 1, sortmp, s);
      } else {
        // normals sum in ascending triangle order: radix sort by (voxel, triangle)
        const bool in_alt = sort_pairs_seg(bd, d_tiles, d_tb, ntiles, keys, vals, kalt, valt, P2,
                                           max_keybits, nmode ? val_bits : 0, sortmp, s);
        sk = in_alt ? kalt : keys;
        sv = in_alt ? valt : vals;
        launch_heads(sk, P2, flags, bd, s);
        scan_u32(flags, uidx, P2, wtot + 1, sortmp, s);
        launch_useg(flags, uidx, P2, useg, s);
      }
      mark(7);
      if (any_l2)
        launch_level2(bd, sk, sv, useg, ub, l2tmp, warp_words, ctx->num_sms, s, [&] { mark(9); },
                      zslab, nslab, [&](int k, cudaStream_t ls) {
                        if (packed) {  // the host expands this slab's codes once it is done
                          cudaEventRecord(ctx->cev[1 + k], ls);
                          return;
                        }
                        if (!sink || !l2_copied || l2_direct) return;
                        cudaEventRecord(ctx->cev[1 + k], ls);
                        cudaStreamWaitEvent(cs, ctx->cev[1 + k], 0);
                        const int64_t a = (int64_t)slab_off[k] * gh[0].cells;
                        const int64_t b = (int64_t)slab_off[k + 1] * gh[0].cells;
                        if (b > a)
                          cudaMemcpyAsync(sink->l2 + a, static_cast<uint8_t *>(set->l2) + a, b - a,
                                          cudaMemcpyDeviceToHost, cs);
                      }, gh[0].n[2], sink ? &ctx->slab_aux : nullptr, l2_queue, l2_fillq);
      else
        mark(9);
      if (nmode) {
        launch_face_normals(bd, s);
        launch_normals(bd, sk, sv, useg, ub, any_l2, ctx->num_sms, s);
      }
    } else {
      mark(7);
      mark(9);
    }
    mark(8);
    if (sink) {  // join the copy stream back
      cudaEventRecord(ctx->cev[kMaxSlabs + 1], cs);
      cudaStreamWaitEvent(s, ctx->cev[kMaxSlabs + 1], 0);
    }
    StageList out(ctx->num_sms, s);
    out.copy(ctx->h_stats, stats, n * sizeof(MeshStats));
    out.copy(ctx->h_u32, wtot, 8);
    out.launch();
  }, phase1_graph, any_hier ? nullptr : &sig1));
  if (packed) {
    // each finished slab's codes -> the caller's bytes, while later slabs compute
    for (int k = 0; k < nslab; ++k) {
      const uint32_t lo = d_slab ? slab_off[k] : 0u;
      if (bd.pk_end[k] <= lo) continue;
      CK(cudaEventSynchronize(ctx->cev[1 + k]));
      const int64_t a = (int64_t)lo * gh[0].cells, b = (int64_t)bd.pk_end[k] * gh[0].cells;
      if (b > a) ctx->pool->run(ctx->h_codes + a / 16, sink->l2 + a, (size_t)((b - a) / 16));
    }
  }
  CK(cudaStreamSynchronize(s));
  ht[4] = HClock::now();
  take_stage_times();
  for (int m = 0; m < n; ++m)
    if (ctx->h_stats[m].status) return fail_all(GPV_ERR_DEVICE, "device status raised in Level2");
  if (do_l2) {
    if ((int64_t)ctx->h_u32[1] != ub)
      return fail_all(GPV_ERR_DEVICE, "boundary plane and pair lists disagree");
  }
  assemble(boff, l2off);
  if (!l2_copied) {
    ctx_fail(ctx, GPV_ERR_BUDGET, "host Level2 buffer too small: nothing copied there (result kept)");
    return GPV_ERR_BUDGET;
  }
  if (og_path) {
    // this call's sizes, for a next call with the same meshes and grids as one graph (a little
    // room for triangles that move between calls; with the key unchanged, the larger of the old
    // and new sizes, so that two meshes sharing a key do not re-run each other's calls)
    PlanCaps c;
    c.B = Btot + Btot / 64 + 64;
    c.U = ub + ub / 64 + 64;
    c.l2bytes = l2bytes + l2bytes / 64 + 4096;
    c.tiles = ntiles + ntiles / 64 + 4;
    c.P = P2 + P2 / 64 + 1024;
    if (ctx->og_key == key) {
      c.B = std::max(c.B, ctx->og_caps.B);
      c.U = std::max(c.U, ctx->og_caps.U);
      c.l2bytes = std::max(c.l2bytes, ctx->og_caps.l2bytes);
      c.tiles = std::max(c.tiles, ctx->og_caps.tiles);
      c.P = std::max(c.P, ctx->og_caps.P);
    }
    ctx->og_key = key;
    ctx->og_caps = c;
  }
  take_host_times();
  return GPV_OK;
#undef CK
}

}  // namespace gpv

namespace gpv {

// Grid search over (Level1 tile, Level2 chunk cap) on a sample batch; each candidate runs once
// to warm up and `reps` times timed with CUDA events on the stream.  The fastest pair is kept.
int autotune(gpv_ctx *ctx, int n, const float *const *d_tris, const int64_t *T,
             const gpv_grid_spec *specs, cudaStream_t s, int reps, int *best_tile,
             int *best_chunk, float *best_ms) {
  static const int tiles[] = {32, 64, 128, 256};
  static const int chunks[] = {4, 8, 16, 32};
  std::vector<gpv_result> res(n);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return ctx_fail(ctx, GPV_ERR_CUDA, "event creation failed");
  float best = 1e30f;
  int bt = ctx->tile, bc = ctx->l2_chunk_cap;
  int rc = GPV_OK;
  for (int ti : tiles)
    for (int ch : chunks) {
      ctx->tile = ti;
      ctx->l2_chunk_cap = ch;
      float total = 0.f;
      for (int r = 0; r <= reps && rc == GPV_OK; ++r) {
        cudaEventRecord(e0, s);
        rc = run_batch(ctx, n, d_tris, T, specs, res.data(), s);
        cudaEventRecord(e1, s);
        if (rc != GPV_OK) break;
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0) total += ms;
        for (int m = 0; m < n; ++m) gpv_result_release(ctx, &res[m]);
      }
      if (rc != GPV_OK) break;
      if (total < best) {
        best = total;
        bt = ti;
        bc = ch;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tile = bt;
  ctx->l2_chunk_cap = bc;
  if (best_tile) *best_tile = bt;
  if (best_chunk) *best_chunk = bc;
  if (best_ms) *best_ms = best / std::max(reps, 1);
  return rc;
}

}  // namespace gpv
