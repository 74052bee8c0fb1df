// gpv_noalloc.cu -- Level1 voxelization that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs inside another allocator's or memory
// pool's hooks (a call back into the allocator would recurse or deadlock), host paths that must
// not take the implicit device synchronisation that cudaMalloc/cudaFree can cause, and plugin
// hosts that hand a library its buffers and forbid it to acquire device memory of its own.
// gpv_voxelize_level1_noalloc serves them: the caller passes the triangles and the three Level1
// outputs, and every intermediate lives in g_noalloc_scratch, a file-scope __device__ array of
// fixed size (kScratchBytes, 32 MiB) that every GPU loading this library holds until the
// process exits.
//
// Rules of use:
//   * Host code cannot use the array's name as a device address.  Every call looks the address
//     up with cudaGetSymbolAddress while the caller's device is current and checks the result
//     (a lookup costs far less than the call's own stream synchronisation, and it stays right
//     after a device reset, which loads the module -- and the array -- again).
//   * A call copies its tables from host memory and waits for its stream, so it cannot be
//     recorded into a graph: a call on a stream that is capturing is refused.
//   * All calls share the one array, which keeps the previous call's contents.  Each call clears
//     the regions that must start at zero.  Calls whose GPU work overlaps -- on different
//     streams or host threads -- race on the array; serialise them.
//   * Sizes whose intermediates do not fit the array are rejected with GPV_ERR_INVALID and a
//     message from gpv_noalloc_last_error() (kept per host thread); nothing is launched then.
//   * No cudaMalloc, cudaFree, host heap or library allocation is made.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "gpv_internal.h"

namespace gpv {
namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;
constexpr int kMaxTableFloats = 12288;  // nx + ny + nz
// Scratch bytes per triangle (packed vertices 48, SAT box 16, ray box 16).  Triangle counts are
// checked against the array with this before any size is formed, so no size can wrap.
constexpr size_t kBytesPerTriangle = 80;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

thread_local char g_err[256] = "";

void set_err(const char *msg) {
  std::snprintf(g_err, sizeof(g_err), "%s", msg);
}

// Variant of the Level1 kernel without the (voxel, triangle) records: one warp per triangle,
// whose lanes share its SAT candidate columns (boundary bits) and its fill columns (parity
// toggles).  Inputs are the packed triangles written by the prep kernel.  A triangle's work is
// its candidate box plus its fill columns times nz, spread over 32 lanes: a triangle whose box
// spans the whole grid (or an ill-conditioned one, whose fill box is the whole grid) costs about
// nx*ny*nz/32 tests per lane.
__global__ void k_level1_nopairs(const MeshDesc *__restrict__ md) {
  const MeshDesc &b = *md;
  const GridDev &g = b.g;
  const int lane = threadIdx.x & 31;
  const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // warp-uniform
  if (t >= b.T) return;
  const float4 a0 = b.ptri[3 * t], a1 = b.ptri[3 * t + 1], a2 = b.ptri[3 * t + 2];
  const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
  const int4 rg = b.rng[t];
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const int x0 = (int)(rg.x & 0xffff), x1 = (int)((unsigned)rg.x >> 16);
  const int y0 = (int)(rg.y & 0xffff), y1 = (int)((unsigned)rg.y >> 16);
  const int z0 = (int)(rg.z & 0xffff), z1 = (int)((unsigned)rg.z >> 16);
  const int sx = max(x1 - x0 + 1, 0), sy = max(y1 - y0 + 1, 0);
  for (int c = lane; c < sx * sy; c += 32) {
    const int p = x0 + c % sx, q = y0 + c / sx;
    SatCol sc;
    if (!sat_col(V, g.c1[0][p], g.c1[1][q], g.e1, sc)) continue;
    for (int r = z0; r <= z1; ++r)
      if (sat_z(sc, V, g.c1[2][r], g.e1))
        atomicOr(&b.bplane[((size_t)r * ny + q) * g.nxw + (p >> 5)], 1u << (p & 31));
  }
  const uint32_t fxr = __float_as_uint(a0.w), fyr = __float_as_uint(a1.w);
  const int fx0 = (int)(fxr & 0xffff), fx1 = (int)(fxr >> 16);
  const int fy0 = (int)(fyr & 0xffff), fy1 = (int)(fyr >> 16);
  const int fsx = max(fx1 - fx0 + 1, 0), fsy = max(fy1 - fy0 + 1, 0);
  RayTri rt;
  ray_tri_pre(V, a2.w, rt);
  for (int c = lane; c < fsx * fsy; c += 32) {
    const int i = fx0 + c % fsx, j = fy0 + c / fsx;
    RayCol rc;
    if (!ray_col(rt, g.c1[0][i], g.c1[1][j], rc)) continue;
    const size_t col = (size_t)j * nx + i;
    uint32_t carry = 0;
    for (int w = g.nzw - 1; w >= 0; --w) {
      uint32_t h = 0;
      for (int bb = 0; bb < 32; ++bb) {
        const int k = 32 * w + bb;
        if (k < nz && ray_t(rt, rc, g.c1[2][k], g.thr)) h |= 1u << bb;
      }
      const uint32_t d = h ^ ((h >> 1) | (carry << 31));
      carry = h & 1u;
      if (d) atomicXor(&b.toggles[col * g.nzw + w], d);
    }
  }
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace
}  // namespace gpv

using namespace gpv;

extern "C" const char *gpv_noalloc_last_error(void) { return g_err; }

extern "C" int gpv_voxelize_level1_noalloc(const float *d_tris, int64_t num_triangles,
                                           const gpv_grid_spec *spec, uint8_t *d_level1_inout,
                                           int32_t *d_level1_prefix, int32_t *d_boundary_index,
                                           int64_t *num_boundary, cudaStream_t stream) {
  if (!spec || !d_level1_inout || !d_level1_prefix || !d_boundary_index || !num_boundary ||
      num_triangles < 0 || (num_triangles > 0 && !d_tris)) {
    set_err("null argument or negative triangle count");
    return GPV_ERR_INVALID;
  }
  if (num_triangles > 0 && (reinterpret_cast<uintptr_t>(d_tris) & 15u)) {
    set_err("triangle buffer must be 16-byte aligned");
    return GPV_ERR_INVALID;
  }
  {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
      cudaGetLastError();
      set_err("stream is capturing (the call copies from host memory and waits for the stream)");
      return GPV_ERR_INVALID;
    }
  }
  if (num_triangles > (int64_t)(kScratchBytes / kBytesPerTriangle)) {
    char msg[160];
    std::snprintf(msg, sizeof(msg),
                  "%lld triangles exceed the fixed no-alloc scratch (%zu bytes, %zu per triangle)",
                  (long long)num_triangles, kScratchBytes, kBytesPerTriangle);
    set_err(msg);
    return GPV_ERR_INVALID;
  }
  // Level2 divisions are not used here, but a specification gpv_voxelize would reject is
  // rejected here too: each in 0..32, all zero or all positive.
  {
    const int32_t *n2 = spec->ndiv2;
    const bool any2 = n2[0] || n2[1] || n2[2], all2 = n2[0] && n2[1] && n2[2];
    if (n2[0] < 0 || n2[1] < 0 || n2[2] < 0 || n2[0] > 32 || n2[1] > 32 || n2[2] > 32 ||
        (any2 && !all2)) {
      set_err("invalid grid specification (Level2 divisions)");
      return GPV_ERR_INVALID;
    }
  }
  // ---- grid, derived exactly as the plain path does (no host heap: tables on the stack)
  GridDev g;
  std::memset(&g, 0, sizeof(g));
  int64_t N1 = 1;
  int ntab = 0;
  for (int a = 0; a < 3; ++a) {
    const int n = spec->ndiv[a];
    if (n < 1 || n > 65535 || !std::isfinite(spec->bbox_min[a]) ||
        !std::isfinite(spec->bbox_max[a]) || !(spec->bbox_max[a] > spec->bbox_min[a])) {
      set_err("invalid grid specification");
      return GPV_ERR_INVALID;
    }
    N1 *= n;
    ntab += n;
  }
  if (ntab > kMaxTableFloats || N1 >= ((int64_t)1 << 31)) {
    set_err("grid exceeds the no-alloc limits (nx+ny+nz <= 12288)");
    return GPV_ERR_INVALID;
  }
  float tab[kMaxTableFloats];
  int off = 0;
  for (int a = 0; a < 3; ++a) {
    const int n = spec->ndiv[a];
    const float span = spec->bbox_max[a] - spec->bbox_min[a];
    g.bmin[a] = spec->bbox_min[a];
    g.bmax[a] = spec->bbox_max[a];
    g.n[a] = n;
    g.n2[a] = 0;
    g.g[a] = (float)(span / (n * 1.0));
    g.e1[a] = (float)(g.g[a] / 2.0);
    for (int i = 0; i < n; ++i) tab[off + i] = (float)((i + 0.5) * g.e1[a] * 2 + (double)spec->bbox_min[a]);
    off += n;
  }
  g.nxw = (g.n[0] + 31) / 32;
  g.nzw = (g.n[2] + 31) / 32;
  g.thr = eps_threshold();
  const int64_t T = num_triangles;
  const int64_t N1w = (int64_t)g.n[2] * g.n[1] * g.nxw;
  const int64_t ncol = (int64_t)g.n[0] * g.n[1];

  // ---- scratch layout and limit
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o = align256(o + bytes); return at; };
  const size_t o_tab = take(sizeof(float) * ntab);
  const size_t o_ptri = take(48 * (size_t)T);
  const size_t o_rng = take(16 * (size_t)T);
  const size_t o_fbox = take(16 * (size_t)T);
  const size_t o_bp = take(4 * (size_t)N1w);
  const size_t o_ip = take(4 * (size_t)N1w);
  const size_t o_tg = take(4 * (size_t)(ncol * g.nzw));
  const size_t o_wc = take(4 * (size_t)N1w);
  const size_t o_wp = take(4 * (size_t)N1w);
  const size_t o_sc = take(4 * (size_t)scan_temp_words(N1w));
  const size_t o_st = take(sizeof(MeshStats));
  const size_t o_tot = take(16);
  const size_t o_md = take(sizeof(MeshDesc));
  if (o > kScratchBytes) {
    char msg[160];
    std::snprintf(msg, sizeof(msg),
                  "inputs need %zu bytes of scratch; the fixed no-alloc scratch holds %zu", o,
                  kScratchBytes);
    set_err(msg);
    return GPV_ERR_INVALID;
  }

  // ---- the array's device address on the current device (looked up on every call)
  unsigned char *base = nullptr;
  {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      set_err("cudaGetSymbolAddress failed for the no-alloc scratch array (no usable device?)");
      return GPV_ERR_CUDA;
    }
    base = static_cast<unsigned char *>(p);
  }

  float *d_tab = reinterpret_cast<float *>(base + o_tab);
  for (int a = 0, oo = 0; a < 3; ++a) { g.c1[a] = d_tab + oo; oo += g.n[a]; }
  MeshDesc md;
  std::memset(&md, 0, sizeof(md));
  md.g = g;
  md.tris = d_tris;
  md.T = T;
  md.ptri = reinterpret_cast<float4 *>(base + o_ptri);
  md.rng = reinterpret_cast<int4 *>(base + o_rng);
  md.fbox = reinterpret_cast<float4 *>(base + o_fbox);
  md.bplane = reinterpret_cast<uint32_t *>(base + o_bp);
  md.iplane = reinterpret_cast<uint32_t *>(base + o_ip);
  md.toggles = reinterpret_cast<uint32_t *>(base + o_tg);
  md.stats = reinterpret_cast<MeshStats *>(base + o_st);
  md.l1 = d_level1_inout;
  md.prefix = d_level1_prefix;
  md.bindex = d_boundary_index;
  MeshDesc *d_md = reinterpret_cast<MeshDesc *>(base + o_md);
  uint32_t *wcnt = reinterpret_cast<uint32_t *>(base + o_wc);
  uint32_t *wpre = reinterpret_cast<uint32_t *>(base + o_wp);
  uint32_t *stmp = reinterpret_cast<uint32_t *>(base + o_sc);
  uint32_t *d_tot = reinterpret_cast<uint32_t *>(base + o_tot);
  BatchDev bd;
  std::memset(&bd, 0, sizeof(bd));
  bd.md = d_md;
  bd.nmesh = 1;
  bd.tile = 128;
  bd.total_tris = T;
  bd.total_fwarps = (int64_t)g.n[1] * g.nxw * g.nzw;
  bd.total_rows = (int64_t)g.n[2] * g.n[1];
  bd.total_xchunks = (N1 + 127) / 128;
  bd.total_words = N1w;

  // The array keeps the last call's data: clear everything that must start at zero.  The
  // descriptor and the tables are copied from this function's stack (pageable memory: the copy
  // has been staged by the time cudaMemcpyAsync returns).
  cudaError_t e = cudaMemcpyAsync(d_tab, tab, sizeof(float) * ntab, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_md, &md, sizeof(md), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(md.stats, 0, sizeof(MeshStats), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(md.bplane, 0, 4 * (size_t)N1w, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(md.toggles, 0, 4 * (size_t)(ncol * g.nzw), stream);
  if (e != cudaSuccess) {
    set_err(cudaGetErrorString(e));
    return GPV_ERR_CUDA;
  }
  launch_prep(bd, stream);
  if (T > 0) {
    k_level1_nopairs<<<(unsigned)((T + 3) / 4), 128, 0, stream>>>(d_md);  // a warp per triangle
    count_launch();
  }
  launch_fill_finish(bd, stream);
  launch_popc(md.bplane, N1w, wcnt, stream);
  scan_u32(wcnt, wpre, N1w, d_tot, stmp, stream);
  launch_expand(bd, wpre, stream);
  uint32_t nb = 0;
  MeshStats hs;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nb, d_tot, sizeof(nb), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, md.stats, sizeof(hs), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    set_err(cudaGetErrorString(e));
    return GPV_ERR_CUDA;
  }
  if (hs.status & ST_BAD_INPUT) {
    set_err("non-finite vertex");
    return GPV_ERR_INVALID;
  }
  *num_boundary = (int64_t)nb;
  set_err("");
  return GPV_OK;
}
