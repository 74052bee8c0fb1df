// gpv_shims.cu -- the reference-named C entry points of GPView's CUDA library (GPViewCUDA, built
// from cuda/CUDAClassifyTessellation.cu and cuda/THRUSTUtilities.cu), with the same signatures,
// caller-owned device buffers, legacy default stream and return conventions, so that GPView
// relinks against libgpview.so in place of GPViewCUDA:
//   CUDAClassifyTessellation, CUDAClassifyTessellationLevel2, CUDAClassifyInOutLevel2
//     (includes/CUDAUtilities.h:87-89);
//   THRUSTDeviceFindMax, THRUSTDeviceFindMaxFloat4, THRUSTDeviceMinMaxSort
//     (includes/CUDAUtilities.h:72-74; src/CUDAUtilities.cpp:121-132 calls the first).
// InitializeCUDA and CUDACheckErrors are not here: the reference declares them with C++ linkage
// (includes/CUDAUtilities.h:63-64) and defines them in the application (src/CUDAUtilities.cpp).
//
// Arithmetic follows the reference's CPU code, not its CUDA-8 kernels: box centres are the CPU's
// double-then-float expressions, predicates run without contraction (the reference kernels let
// nvcc fuse multiply-adds, so their results could differ from its own CPU path).  Where a shim's
// inputs do not carry what the CPU formula needs (the Level2 ray origins of
// CUDAClassifyInOutLevel2), the reference kernel's own FP32 formula is used, evaluated without
// contraction.
//
// CUDAClassifyTessellation runs on the library's Level1 engine (the prep kernel, the persistent
// TMA-staged Level1 kernel's SAT units, then a scatter of its (voxel, triangle) records into the
// caller's arrays).  All shims share one grow-only device workspace kept for the process, so a
// call allocates only when it needs more room than any earlier call.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "gpv_internal.h"

namespace gpv {
namespace {

// Grow-only workspace of the shims (process-wide; the reference's callers are single-threaded,
// and a mutex serialises calls from several threads).  Growth frees the old block after a
// device synchronisation, so work still queued on it has finished.
struct ShimSpace {
  std::mutex mu;
  void *dev = nullptr;
  size_t cap = 0;
  MeshStats *h_stats = nullptr;  // page-locked
  float *h_tab = nullptr;        // page-locked staging of tables
  size_t h_tab_cap = 0;
  int device = -1, num_sms = 0;
};
ShimSpace g_shim;

size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

// Room for `bytes` in the workspace; false if it cannot be had.
bool shim_reserve(size_t bytes) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (dev != g_shim.device) {  // another device: start over there
    g_shim.dev = nullptr;
    g_shim.cap = 0;
    g_shim.device = dev;
    cudaDeviceGetAttribute(&g_shim.num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  if (!g_shim.h_stats && cudaMallocHost(&g_shim.h_stats, sizeof(MeshStats)) != cudaSuccess) {
    g_shim.h_stats = nullptr;
    return false;
  }
  if (bytes <= g_shim.cap) return true;
  if (g_shim.dev) {
    cudaDeviceSynchronize();
    cudaFree(g_shim.dev);
  }
  g_shim.dev = nullptr;
  g_shim.cap = 0;
  const size_t want = std::max(bytes + bytes / 4, size_t(1) << 20);
  if (cudaMalloc(&g_shim.dev, want) != cudaSuccess) {
    cudaGetLastError();
    g_shim.dev = nullptr;
    return false;
  }
  g_shim.cap = want;
  return true;
}

bool shim_tables(size_t floats) {
  if (floats <= g_shim.h_tab_cap) return true;
  if (g_shim.h_tab) cudaFreeHost(g_shim.h_tab);
  g_shim.h_tab = nullptr;
  g_shim.h_tab_cap = 0;
  if (cudaMallocHost(&g_shim.h_tab, std::max<size_t>(floats, 4096) * sizeof(float)) != cudaSuccess) {
    g_shim.h_tab = nullptr;
    return false;
  }
  g_shim.h_tab_cap = std::max<size_t>(floats, 4096);
  return true;
}

// The Level1 engine's (voxel, triangle) records into the reference's arrays: inOut[v] = 2,
// voxelTriCount[v] += 1 and the triangle id in the next free slot of voxelTriIndex[v * buf ..]
// (never past buf; the count keeps the true number).  keys are column-major voxel keys
// ((y * nx + x) * nz + z); the top bit of a value flags a column's topmost record.
__global__ void k_shim_scatter(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                               const MeshStats *__restrict__ st, int nx, int ny, int nz,
                               float *__restrict__ inOut, int *__restrict__ cnt,
                               int *__restrict__ idx, int buf) {
  const uint64_t P = st->pairs < st->pair_cap ? st->pairs : st->pair_cap;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < P;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t key = keys[e];
    const int r = (int)(key % (uint32_t)nz);
    const uint32_t col = key / (uint32_t)nz;
    const int p = (int)(col % (uint32_t)nx), q = (int)(col / (uint32_t)nx);
    const size_t v = ((size_t)r * ny + q) * nx + p;
    inOut[v] = 2.0f;
    const int slot = atomicAdd(&cnt[v], 1);
    if (slot >= 0 && slot < buf) idx[v * (size_t)buf + slot] = (int)(vals[e] & 0x7fffffffu);
  }
}

// CUDAClassifyTessellationKernel's launch shape (cuda/CUDAClassifyTessellation.cu:320-401): one
// thread per triangle over its candidate box; the per-voxel list never writes past
// triBufferLen.  Used only for triangle buffers that are not 16-byte aligned (the engine's
// prep kernel reads them as such).
__global__ void k_shim_level1(const float *__restrict__ tris, int T, float *__restrict__ inOut,
                              int *__restrict__ cnt, int *__restrict__ idx, GridDev g, int buf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  float V[9];
  for (int k = 0; k < 9; ++k) V[k] = tris[9 * (size_t)t + k];
  int lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    const int c0 = cell_of(V[a], g.bmin[a], g.bmax[a], g.n[a]);
    const int c1 = cell_of(V[3 + a], g.bmin[a], g.bmax[a], g.n[a]);
    const int c2 = cell_of(V[6 + a], g.bmin[a], g.bmax[a], g.n[a]);
    lo[a] = max(min(c0, min(c1, c2)), 0);
    hi[a] = min(max(c0, max(c1, c2)), g.n[a] - 1);
  }
  for (int p = lo[0]; p <= hi[0]; ++p)
    for (int q = lo[1]; q <= hi[1]; ++q) {
      SatCol sc;
      if (!sat_col(V, g.c1[0][p], g.c1[1][q], g.e1, sc)) continue;
      for (int r = lo[2]; r <= hi[2]; ++r) {
        if (!sat_z(sc, V, g.c1[2][r], g.e1)) continue;
        const size_t v = ((size_t)r * g.n[1] + q) * g.n[0] + p;
        inOut[v] = 2.0f;
        const int slot = atomicAdd(&cnt[v], 1);
        if (slot >= 0 && slot < buf) idx[v * (size_t)buf + slot] = t;
      }
    }
}

// ---- the THRUSTUtilities entry points, without Thrust --------------------------------------
// thrust::max_element's answer, the first index of the largest value under operator<, for a
// sequence read from the start: the first element stays the answer while nothing compares
// greater, so a NaN first element is the answer and later NaNs never are; -0 and +0 compare
// equal.  One 64-bit key per element orders by value, then by lower index.
__device__ unsigned long long g_thrust_max_key;

__device__ __forceinline__ unsigned long long max_key(float v, uint64_t i, bool first_nan) {
  if (first_nan) return ~0ull;  // element 0 is NaN: it is the answer
  if (v != v) return 0ull;      // later NaNs never are
  uint32_t b = __float_as_uint(v == 0.0f ? 0.0f : v);
  b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
  return ((unsigned long long)b << 32) | (0xffffffffull - (uint32_t)i);
}

// Values at x[i * stride] (stride 1: floats; stride 4 with x pointing at .w: float4's w).
__global__ void k_thrust_max(const float *__restrict__ x, int64_t n, int stride) {
  unsigned long long best = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = x[i * stride];
    const unsigned long long k = max_key(v, (uint64_t)i, i == 0 && v != v);
    best = k > best ? k : best;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, best, d);
    best = o > best ? o : best;
  }
  if ((threadIdx.x & 31) == 0 && best) atomicMax(&g_thrust_max_key, best);
}

// Index of the answer of k_thrust_max over n values, or -1 (n <= 0 or failure).
int64_t thrust_argmax(const float *x, int64_t n, int stride, int num_sms) {
  if (n <= 0 || n > 0xffffffffll) return -1;
  const unsigned long long zero = 0ull;
  if (cudaMemcpyToSymbolAsync(g_thrust_max_key, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, 0) !=
      cudaSuccess)
    return -1;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)std::max(num_sms, 1) * 8);
  k_thrust_max<<<(unsigned)blocks, 256>>>(x, n, stride);
  count_launch();
  unsigned long long key = 0ull;
  if (cudaMemcpyFromSymbol(&key, g_thrust_max_key, sizeof(key)) != cudaSuccess) return -1;
  if (key == ~0ull) return 0;
  if (key == 0ull) return 0;  // every value NaN after a non-NaN first: the first stays
  return (int64_t)(0xffffffffull - (key & 0xffffffffull));
}

int shim_num_sms() {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

// THRUSTDeviceMinMaxSort's keys: rows >= 0 by value, then every negative row, in input order
// (the reference's comparator -- a < b when a.row >= 0 and a.row < b.row -- leaves the negative
// rows unordered; stable placement after the others is this library's choice).
__global__ void k_minmax_keys(const int *__restrict__ row, int64_t n, uint32_t *__restrict__ keys,
                              uint32_t *__restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = row[i];
  keys[i] = r >= 0 ? (uint32_t)r : 0xffffffffu;
  vals[i] = (uint32_t)i;
}

__global__ void k_minmax_gather(const int *__restrict__ row, const uint32_t *__restrict__ order,
                                int64_t n, int *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = row[order[i]];
}

// Unit face normal as the loaders compute it (VectorCrossProduct then VectorNormalize,
// includes/FloatVector.h:293-342).
__device__ __forceinline__ void face_normal(const float *V, float n[3]) {
  const float a0 = fs(V[3], V[0]), a1 = fs(V[4], V[1]), a2 = fs(V[5], V[2]);
  const float b0 = fs(V[6], V[0]), b1 = fs(V[7], V[1]), b2 = fs(V[8], V[2]);
  n[0] = fs(fm(a1, b2), fm(b1, a2));
  n[1] = fs(fm(a2, b0), fm(b2, a0));
  n[2] = fs(fm(a0, b1), fm(b0, a1));
  const float mag = __fsqrt_rn(fa(fa(fm(n[0], n[0]), fm(n[1], n[1])), fm(n[2], n[2])));
  if (mag != 0.f) {
    n[0] = __fdiv_rn(n[0], mag);
    n[1] = __fdiv_rn(n[1], mag);
    n[2] = __fdiv_rn(n[2], mag);
  }
}

// The SAT's z-invariant axes (sat_col) with the box x and y axes first.  The result is the same
// conjunction of the same axis tests, each evaluated with the same operations, so it is
// identical; a voxel's list is tested against every sub-column of the voxel, and most
// (triangle, sub-column) pairs already fail the box axes.
__device__ __forceinline__ bool box_range_fails(float a, float b, float c, float h) {
  float mn = a, mx = a;
  if (b < mn) mn = b;
  if (b > mx) mx = b;
  if (c < mn) mn = c;
  if (c > mx) mx = c;
  return mn > h || mx < -h;
}
__device__ __forceinline__ bool sat_col_box_first(const float *V, float cx, float cy,
                                                  const float h[3], SatCol &s) {
  s.v0x = fs(V[0], cx); s.v1x = fs(V[3], cx); s.v2x = fs(V[6], cx);
  if (box_range_fails(s.v0x, s.v1x, s.v2x, h[0])) return false;
  s.v0y = fs(V[1], cy); s.v1y = fs(V[4], cy); s.v2y = fs(V[7], cy);
  if (box_range_fails(s.v0y, s.v1y, s.v2y, h[1])) return false;
  return sat_col(V, cx, cy, h, s);
}
// The z-dependent part (sat_z) with the box z axis first, identical for the same reason.
__device__ __forceinline__ bool sat_z_box_first(const SatCol &s, const float *V, float cz,
                                                const float h[3]) {
  if (box_range_fails(fs(V[2], cz), fs(V[5], cz), fs(V[8], cz), h[2])) return false;
  return sat_z(s, V, cz, h);
}

// CUDAClassifyTessellationLevel2Kernel (.cu:403-448), one warp per boundary voxel walking the
// voxel's list in order.  For each triangle the lanes take the sub-columns of the triangle's
// Level2 cell range (l2_cell_range: outside it the SAT's own box axes reject, so nothing is
// skipped that could pass), run the z-invariant axes once per sub-column and the z-dependent part
// per cell of the range.  Within one triangle every cell has at most one lane; a __syncwarp
// between triangles orders the updates, so each cell sums the CPU's unit face normals in list
// order, as a per-cell thread would.  Centres come from `cen` ([b][n2x | n2y | n2z] floats,
// formed on the host as the CPU does: float(((p+0.5)*gridSize2 + mid) - ext1) in double,
// src/Object.cpp:2389-2391).  (One thread per (voxel, sub-column), most lanes left each
// triangle at its box test: 6.4 of 32 lanes active, 1.50 ms on torus262k.)
__global__ void k_shim_level2_sat(const float *__restrict__ tris, float *__restrict__ l2,
                                  float *__restrict__ nrm, const float *__restrict__ cen,
                                  const int *__restrict__ l2index, const int *__restrict__ cnt,
                                  const int *__restrict__ flatIndex, const int *__restrict__ flat,
                                  int B, int3 n2, float3 e2) {
  const int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= B) return;  // the whole warp
  const int lane = (int)(threadIdx.x & 31u);
  const int ncol2 = n2.x * n2.y, cells = ncol2 * n2.z;
  const int v = l2index[b];
  const float *cx = cen + (size_t)b * (n2.x + n2.y + n2.z);
  const float *cy = cx + n2.x, *cz = cy + n2.y;
  const float h[3] = {e2.x, e2.y, e2.z};
  const float ig[3] = {1.0f / (2.0f * e2.x), 1.0f / (2.0f * e2.y), 1.0f / (2.0f * e2.z)};
  const bool sized = e2.x > 0.f && e2.y > 0.f && e2.z > 0.f && isfinite(ig[0]) &&
                     isfinite(ig[1]) && isfinite(ig[2]);
  const int n = cnt[v], f0 = flatIndex[v];
  for (int k = 0; k < n; ++k) {
    const int t = flat[f0 + k];
    float V[9];
    for (int j = 0; j < 9; ++j) V[j] = tris[9 * (size_t)t + j];
    int p0 = 0, p1 = n2.x - 1, q0 = 0, q1 = n2.y - 1, r0 = 0, r1 = n2.z - 1;
    if (sized) {  // (cells of no size: every cell of the voxel is tested)
      l2_cell_range(fminf(V[0], fminf(V[3], V[6])), fmaxf(V[0], fmaxf(V[3], V[6])), cx[0], h[0],
                    ig[0], n2.x, p0, p1);
      l2_cell_range(fminf(V[1], fminf(V[4], V[7])), fmaxf(V[1], fmaxf(V[4], V[7])), cy[0], h[1],
                    ig[1], n2.y, q0, q1);
      l2_cell_range(fminf(V[2], fminf(V[5], V[8])), fmaxf(V[2], fmaxf(V[5], V[8])), cz[0], h[2],
                    ig[2], n2.z, r0, r1);
    }
    if (p0 <= p1 && q0 <= q1 && r0 <= r1) {
      const int np = p1 - p0 + 1, items = np * (q1 - q0 + 1);
      for (int it = lane; it < items; it += 32) {
        const int qq = it / np, p = p0 + (it - qq * np), q = q0 + qq;
        SatCol sc;
        if (!sat_col_box_first(V, cx[p], cy[q], h, sc)) continue;
        bool have_fn = false;
        float fn[3];
        for (int r = r0; r <= r1; ++r) {
          if (!sat_z_box_first(sc, V, cz[r], h)) continue;
          if (!have_fn) {
            face_normal(V, fn);
            have_fn = true;
          }
          const size_t o = (size_t)b * cells + (size_t)r * ncol2 + (size_t)q * n2.x + p;
          l2[o] = 2.0f;
          nrm[4 * o + 0] = fa(nrm[4 * o + 0], fn[0]);
          nrm[4 * o + 1] = fa(nrm[4 * o + 1], fn[1]);
          nrm[4 * o + 2] = fa(nrm[4 * o + 2], fn[2]);
          nrm[4 * o + 3] = fa(nrm[4 * o + 3], 1.0f);
        }
      }
    }
    __syncwarp();  // this triangle's updates before the next triangle's
  }
}

// End of the x/y-column lists (the largest xyTriFlatIndex + xyTriCount over the columns).
__global__ void k_shim_list_end(const int *__restrict__ cnt, const int *__restrict__ index,
                                int ncols, int *__restrict__ end) {
  int e = 0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncols; c += gridDim.x * blockDim.x)
    if (cnt[c] > 0) e = max(e, index[c] + cnt[c]);
  e = __reduce_max_sync(0xffffffffu, e);
  if ((threadIdx.x & 31u) == 0 && e) atomicMax(end, e);
}

// The +z ray test's per-triangle constants (RayTri: v1, the edges, 1/det and the |det| test) of
// every entry of the x/y-column lists, once per entry instead of once per (entry, sub-column):
// three float4 per entry, the w of the second holding the det test.  One warp per column walks
// the column's own entries, so only entries a column references are read (as the fill does).
__global__ void k_shim_ray_entries(const float *__restrict__ tris, const int *__restrict__ cnt,
                                   const int *__restrict__ index, const int *__restrict__ flat,
                                   int ncols, float thr, float4 *__restrict__ out) {
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= ncols) return;
  const int n = cnt[c], f0 = index[c];
  for (int k = (int)(threadIdx.x & 31u); k < n; k += 32) {
    const int64_t e = (int64_t)f0 + k;
    const int t = flat[e];
    float V[9];
    for (int j = 0; j < 9; ++j) V[j] = tris[9 * (size_t)t + j];
    RayTri rt;
    ray_tri(V, thr, rt);
    out[3 * e + 0] = make_float4(rt.v1x, rt.v1y, rt.v1z, rt.inv_det);
    out[3 * e + 1] = make_float4(rt.e1x, rt.e1y, rt.e1z, rt.ok ? 1.f : 0.f);
    out[3 * e + 2] = make_float4(rt.e2x, rt.e2y, rt.e2z, 0.f);
  }
}

// CUDAClassifyInOutLevel2Kernel (.cu:450-504), one thread per (boundary voxel, sub-column)
// instead of per cell: the ray test's u/v part depends only on the origin's x and y, so it runs
// once per (triangle, sub-column), and t per cell; the +z parity of every cell of the sub-column
// against the x/y-column list is kept in one bit each.  Origins: (2p+1)*ext2 + mid - ext1 in
// float, left to right, as the reference kernel forms them.
__global__ void k_shim_level2_fill(const float4 *__restrict__ ray, float *__restrict__ l2,
                                   const float *__restrict__ mid, const int *__restrict__ l2index,
                                   const int *__restrict__ xycnt, const int *__restrict__ xyIndex,
                                   int B, int3 nd, int3 n2, float3 e1, float3 e2, float thr) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ncol2 = n2.x * n2.y, cells = ncol2 * n2.z;
  if (gid >= (int64_t)B * ncol2) return;
  const int b = (int)(gid / ncol2), pq = (int)(gid % ncol2);
  const int q = pq / n2.x, p = pq - q * n2.x;
  const int v = l2index[b];
  const int xy = v % (nd.x * nd.y);
  const float ox = fs(fa(fm((float)(2 * p + 1), e2.x), mid[3 * b + 0]), e1.x);
  const float oy = fs(fa(fm((float)(2 * q + 1), e2.y), mid[3 * b + 1]), e1.y);
  const float mz = mid[3 * b + 2];
  uint32_t par = 0;  // one bit per cell (n2z <= 32)
  const int n = xycnt[xy], f0 = xyIndex[xy];
  for (int k = 0; k < n; ++k) {
    const float4 *re = ray + 3 * (size_t)(f0 + k);
    const float4 a = re[0], b1 = re[1], b2 = re[2];
    if (b1.w == 0.f) continue;  // |det| test failed
    RayTri rt;
    rt.v1x = a.x; rt.v1y = a.y; rt.v1z = a.z; rt.inv_det = a.w;
    rt.e1x = b1.x; rt.e1y = b1.y; rt.e1z = b1.z;
    rt.e2x = b2.x; rt.e2y = b2.y; rt.e2z = b2.z;
    rt.ok = true;
    RayCol rc;
    if (!ray_col(rt, ox, oy, rc)) continue;
    for (int r = 0; r < n2.z; ++r) {
      const float oz = fs(fa(fm((float)(2 * r + 1), e2.z), mz), e1.z);
      if (ray_t(rt, rc, oz, thr)) par ^= 1u << r;
    }
  }
  for (int r = 0; r < n2.z; ++r)
    if ((par >> r) & 1u) l2[(size_t)b * cells + (size_t)r * ncol2 + pq] = 1.0f;
}

}  // namespace
}  // namespace gpv

using namespace gpv;

extern "C" {

int CUDAClassifyTessellation(float *trianglesCUDAData, int numTriangles, float *inOutCUDAData,
                             int *voxelTriCountCUDAData, int *voxelTriIndexCUDAData,
                             float3 objBoxMin, float3 objBoxMax, float3 boxExtents, int3 numDiv,
                             int triBufferLen) {
  gpv_grid_spec spec;
  spec.bbox_min[0] = objBoxMin.x; spec.bbox_min[1] = objBoxMin.y; spec.bbox_min[2] = objBoxMin.z;
  spec.bbox_max[0] = objBoxMax.x; spec.bbox_max[1] = objBoxMax.y; spec.bbox_max[2] = objBoxMax.z;
  spec.ndiv[0] = numDiv.x; spec.ndiv[1] = numDiv.y; spec.ndiv[2] = numDiv.z;
  spec.ndiv2[0] = spec.ndiv2[1] = spec.ndiv2[2] = 0;
  const float ext[3] = {boxExtents.x, boxExtents.y, boxExtents.z};
  GridHost gh;
  if (grid_derive(spec, gh, ext) != GPV_OK || numTriangles <= 0) return 1;
  std::lock_guard<std::mutex> lk(g_shim.mu);
  const int64_t T = numTriangles;
  const int64_t N1w = (int64_t)gh.n[2] * gh.n[1] * gh.nxw;
  const int64_t tog = (int64_t)gh.n[0] * gh.n[1] * gh.nzw;
  const int64_t ntab = table_floats(gh);
  // workspace: tables, packed triangles, SAT ranges, ray boxes, planes, toggles, stats,
  // descriptor, queue, then the records (sized after the prep kernel has counted them)
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t at = off; off = al256(off + bytes); return at; };
  const size_t o_tab = take(4 * (size_t)ntab), o_ptri = take(48 * (size_t)T),
               o_rng = take(16 * (size_t)T), o_fbox = take(16 * (size_t)T),
               o_bp = take(4 * (size_t)N1w), o_ip = take(4 * (size_t)N1w),
               o_tg = take(4 * (size_t)tog), o_st = take(sizeof(MeshStats)),
               o_md = take(sizeof(MeshDesc)), o_q = take(64);
  const size_t fixed = off;
  const bool aligned = (reinterpret_cast<uintptr_t>(trianglesCUDAData) & 15u) == 0;
  if (!shim_reserve(fixed) || !shim_tables((size_t)ntab)) return 1;
  char *base = static_cast<char *>(g_shim.dev);
  pack_tables(gh, g_shim.h_tab);
  float *d_tab = reinterpret_cast<float *>(base + o_tab);
  cudaMemcpyAsync(d_tab, g_shim.h_tab, 4 * (size_t)ntab, cudaMemcpyHostToDevice, 0);
  GridDev g = make_griddev(gh, d_tab);
  if (!aligned) {
    k_shim_level1<<<(numTriangles + 127) / 128, 128>>>(trianglesCUDAData, numTriangles,
                                                        inOutCUDAData, voxelTriCountCUDAData,
                                                        voxelTriIndexCUDAData, g, triBufferLen);
    count_launch();
    cudaStreamSynchronize(0);  // the staged tables may be rewritten by the next call
    return 1;
  }
  MeshDesc md;
  std::memset(&md, 0, sizeof(md));
  md.g = g;
  md.tris = trianglesCUDAData;
  md.T = T;
  md.ptri = reinterpret_cast<float4 *>(base + o_ptri);
  md.rng = reinterpret_cast<int4 *>(base + o_rng);
  md.fbox = reinterpret_cast<float4 *>(base + o_fbox);
  md.bplane = reinterpret_cast<uint32_t *>(base + o_bp);
  md.iplane = reinterpret_cast<uint32_t *>(base + o_ip);
  md.toggles = reinterpret_cast<uint32_t *>(base + o_tg);
  md.stats = reinterpret_cast<MeshStats *>(base + o_st);
  md.ch = 1;
  MeshDesc *d_md = reinterpret_cast<MeshDesc *>(base + o_md);
  int tile = 256;
  while (tile > 32 && T < (int64_t)tile * 3 * g_shim.num_sms) tile >>= 1;
  BatchDev bd;
  std::memset(&bd, 0, sizeof(bd));
  bd.md = d_md;
  bd.nmesh = 1;
  bd.tile = tile;
  bd.total_tris = T;
  bd.total_tiles = (T + tile - 1) / tile;
  bd.total_fwarps = (int64_t)gh.n[1] * gh.nxw * gh.nzw;
  bd.total_rows = (int64_t)gh.n[2] * gh.n[1];
  bd.total_words = N1w;
  bd.queue = reinterpret_cast<uint32_t *>(base + o_q);
  bd.fill = kFillNone;  // SAT units only: ClassifyTessellation marks boundaries, nothing fills
  cudaMemsetAsync(md.stats, 0, sizeof(MeshStats), 0);
  cudaMemsetAsync(md.bplane, 0, 4 * (size_t)N1w, 0);
  cudaMemcpyAsync(d_md, &md, sizeof(md), cudaMemcpyHostToDevice, 0);
  launch_prep(bd, 0);
  // the records' room: one per candidate-box test at most (sat1), read back once
  cudaMemcpyAsync(g_shim.h_stats, md.stats, sizeof(MeshStats), cudaMemcpyDeviceToHost, 0);
  if (cudaStreamSynchronize(0) != cudaSuccess) return 1;
  const int64_t cap = std::max<int64_t>((int64_t)g_shim.h_stats->sat1, 1);
  const size_t o_keys = al256(fixed), o_vals = al256(o_keys + 4 * (size_t)cap);
  const size_t need = al256(o_vals + 4 * (size_t)cap);
  if (need > g_shim.cap) {
    // growing frees the block: copy what the prep kernel produced to the new one
    void *old = g_shim.dev;
    g_shim.dev = nullptr;
    g_shim.cap = 0;
    if (!shim_reserve(need)) {
      g_shim.dev = old;  // keep the old block; give up on this call
      return 1;
    }
    cudaMemcpy(g_shim.dev, old, fixed, cudaMemcpyDeviceToDevice);
    cudaFree(old);
    base = static_cast<char *>(g_shim.dev);
    md.g = make_griddev(gh, reinterpret_cast<float *>(base + o_tab));
    md.ptri = reinterpret_cast<float4 *>(base + o_ptri);
    md.rng = reinterpret_cast<int4 *>(base + o_rng);
    md.fbox = reinterpret_cast<float4 *>(base + o_fbox);
    md.bplane = reinterpret_cast<uint32_t *>(base + o_bp);
    md.iplane = reinterpret_cast<uint32_t *>(base + o_ip);
    md.toggles = reinterpret_cast<uint32_t *>(base + o_tg);
    md.stats = reinterpret_cast<MeshStats *>(base + o_st);
    d_md = reinterpret_cast<MeshDesc *>(base + o_md);
    bd.md = d_md;
    bd.queue = reinterpret_cast<uint32_t *>(base + o_q);
  }
  uint32_t *keys = reinterpret_cast<uint32_t *>(base + o_keys);
  uint32_t *vals = reinterpret_cast<uint32_t *>(base + o_vals);
  md.keys = keys;
  md.vals = vals;
  md.pair_cap = cap;
  md.emit_base = 0;
  cudaMemcpyAsync(d_md, &md, sizeof(md), cudaMemcpyHostToDevice, 0);
  {
    // the pair capacity the Level1 kernel checks its records against
    const unsigned long long c = (unsigned long long)cap;
    cudaMemcpyAsync(&md.stats->pair_cap, &c, sizeof(c), cudaMemcpyHostToDevice, 0);
  }
  launch_level1(bd, g_shim.num_sms, 0);
  const int64_t blocks = std::min<int64_t>((cap + 255) / 256, (int64_t)g_shim.num_sms * 8);
  k_shim_scatter<<<(unsigned)std::max<int64_t>(blocks, 1), 256>>>(
      keys, vals, md.stats, gh.n[0], gh.n[1], gh.n[2], inOutCUDAData, voxelTriCountCUDAData,
      voxelTriIndexCUDAData, triBufferLen);
  count_launch();
  // the workspace is reused by the next call: let this one finish first (the reference's
  // caller synchronises right after anyway, src/Object.cpp:2116-2120)
  cudaStreamSynchronize(0);
  return 1;
}

int CUDAClassifyTessellationLevel2(float *trianglesCUDAData, float *level2InOutCUDAData,
                                   float *level2NormalCUDAData, float *level1MidPointCUDAData,
                                   int *level2IndexCUDAData, int *voxelTriCountCUDAData,
                                   int *level1TriFlatIndexCUDAData, int *level1TriFlatCUDAData,
                                   int numBoundary, int3 numDiv2, float3 boxExtentsLevel1,
                                   float3 boxExtentsLevel2) {
  const int cells = numDiv2.x * numDiv2.y * numDiv2.z;
  if (numBoundary <= 0 || cells <= 0) return 1;
  std::lock_guard<std::mutex> lk(g_shim.mu);
  // Midpoints are device data: bring them over (page-locked staging) and form the centre table
  // in double on the host, as the CPU path does; the table goes to the shared workspace.
  const int nn = numDiv2.x + numDiv2.y + numDiv2.z;
  const size_t nmid = (size_t)numBoundary * 3, ncen = (size_t)numBoundary * nn;
  if (!shim_reserve(4 * ncen) || !shim_tables(nmid + ncen)) return 1;
  float *mid = g_shim.h_tab, *cen = g_shim.h_tab + nmid;
  if (cudaMemcpy(mid, level1MidPointCUDAData, nmid * sizeof(float), cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return 1;
  const float e1[3] = {boxExtentsLevel1.x, boxExtentsLevel1.y, boxExtentsLevel1.z};
  const float e2[3] = {boxExtentsLevel2.x, boxExtentsLevel2.y, boxExtentsLevel2.z};
  const int n2[3] = {numDiv2.x, numDiv2.y, numDiv2.z};
  // (p + 0.5) * gridSize2 in double, per axis and cell (the same for every voxel)
  std::vector<double> off(nn);
  for (int a = 0, o = 0; a < 3; o += n2[a], ++a) {
    const float g2 = e2[a] * 2.0f;  // gridSize2 (exact: ext2 = gridSize2 / 2)
    for (int p = 0; p < n2[a]; ++p) off[o + p] = (p + 0.5) * g2;
  }
  auto centres = [&](int b0, int b1) {
    for (int b = b0; b < b1; ++b)
      for (int a = 0, o = 0; a < 3; o += n2[a], ++a) {
        const double m = (double)mid[3 * (size_t)b + a];
        for (int p = 0; p < n2[a]; ++p)
          cen[(size_t)b * nn + o + p] = (float)(off[o + p] + m - e1[a]);
      }
  };
  // large calls on up to 16 host threads (110k boundary voxels at 8^3: ~2.6 M centres)
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::min(std::min(hw, 16), std::max(1, numBoundary / 4096));
  if (nt <= 1) {
    centres(0, numBoundary);
  } else {
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k)
      th.emplace_back(centres, (int)((int64_t)numBoundary * k / nt),
                      (int)((int64_t)numBoundary * (k + 1) / nt));
    for (std::thread &x : th) x.join();
  }
  float *d_cen = static_cast<float *>(g_shim.dev);
  cudaMemcpyAsync(d_cen, cen, ncen * sizeof(float), cudaMemcpyHostToDevice, 0);
  const int64_t n = (int64_t)numBoundary * 32;  // a warp per boundary voxel
  k_shim_level2_sat<<<(unsigned)((n + 127) / 128), 128>>>(
      trianglesCUDAData, level2InOutCUDAData, level2NormalCUDAData, d_cen, level2IndexCUDAData,
      voxelTriCountCUDAData, level1TriFlatIndexCUDAData, level1TriFlatCUDAData, numBoundary,
      numDiv2, boxExtentsLevel2);
  count_launch();
  cudaStreamSynchronize(0);  // the staging and the workspace are reused by the next call
  return 1;
}

int CUDAClassifyInOutLevel2(float *trianglesCUDAData, float *level2InOutCUDAData,
                            float *level1MidPointCUDAData, int *level2IndexCUDAData,
                            int *xyTriCountCUDAData, int *xyTriFlatIndexCUDAData,
                            int *xyTriFlatCUDAData, int numBoundary, int3 numDiv, int3 numDiv2,
                            float3 boxExtentsLevel1, float3 boxExtentsLevel2) {
  const int cells = numDiv2.x * numDiv2.y * numDiv2.z;
  if (numBoundary <= 0 || cells <= 0) return 1;
  if (numDiv2.z > 32) return 1;  // one parity bit per cell of a sub-column
  std::lock_guard<std::mutex> lk(g_shim.mu);
  // the end of the column lists, then the ray constants of every list entry (workspace)
  const int ncols = numDiv.x * numDiv.y;
  if (ncols <= 0 || !shim_reserve(256)) return 1;
  int *d_end = static_cast<int *>(g_shim.dev);
  cudaMemsetAsync(d_end, 0, sizeof(int), 0);
  k_shim_list_end<<<std::min((ncols + 255) / 256, 4 * shim_num_sms()), 256>>>(
      xyTriCountCUDAData, xyTriFlatIndexCUDAData, ncols, d_end);
  int nE = 0;
  if (cudaMemcpy(&nE, d_end, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  if (!shim_reserve(256 + 48 * (size_t)std::max(nE, 1))) return 1;
  float4 *ray = reinterpret_cast<float4 *>(static_cast<char *>(g_shim.dev) + 256);
  const float thr = eps_threshold();
  if (nE > 0)
    k_shim_ray_entries<<<(unsigned)((ncols + 7) / 8), 256>>>(
        trianglesCUDAData, xyTriCountCUDAData, xyTriFlatIndexCUDAData, xyTriFlatCUDAData, ncols,
        thr, ray);
  const int64_t n = (int64_t)numBoundary * numDiv2.x * numDiv2.y;  // a thread per sub-column
  k_shim_level2_fill<<<(unsigned)((n + 127) / 128), 128>>>(
      ray, level2InOutCUDAData, level1MidPointCUDAData, level2IndexCUDAData, xyTriCountCUDAData,
      xyTriFlatIndexCUDAData, numBoundary, numDiv, numDiv2, boxExtentsLevel1, boxExtentsLevel2, thr);
  count_launch(nE > 0 ? 3 : 2);
  cudaStreamSynchronize(0);  // the workspace is reused by the next call
  return 1;
}

// cuda/THRUSTUtilities.cu:44-60: the largest of w*h device floats (thrust::max_element's answer,
// first index on ties), copied to the host.  0 when w*h <= 0 (the reference then reads one past
// the end).
float THRUSTDeviceFindMax(float *dataCUDAPointer, int w, int h) {
  const int64_t n = (int64_t)w * h;
  const int64_t i = thrust_argmax(dataCUDAPointer, n, 1, shim_num_sms());
  float v = 0.0f;
  if (i >= 0) cudaMemcpy(&v, dataCUDAPointer + i, sizeof(v), cudaMemcpyDeviceToHost);
  return v;
}

// cuda/THRUSTUtilities.cu:82-102: the float4 with the largest w (first on ties); its x, y, z and
// w = 1 into *maxVal, its index into *maxLoc (host pointers), its w returned.  With
// numValues <= 0: *maxLoc = 0, *maxVal = (0, 0, 0, 1), 0 returned.
float THRUSTDeviceFindMaxFloat4(float4 *dataCUDAPointer, int numValues, float4 *maxVal, int *maxLoc) {
  const int64_t i = thrust_argmax(reinterpret_cast<const float *>(dataCUDAPointer) + 3, numValues, 4,
                                  shim_num_sms());
  float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
  if (i >= 0) cudaMemcpy(&e, dataCUDAPointer + i, sizeof(e), cudaMemcpyDeviceToHost);
  if (maxLoc) *maxLoc = i >= 0 ? (int)i : 0;
  if (maxVal) *maxVal = make_float4(e.x, e.y, e.z, 1.0f);
  return e.w;
}

// cuda/THRUSTUtilities.cu:128-160: sorts copies of the (row, min, max) triples by row and copies
// the sorted rows to the host array rowNumbers (n ints); the device inputs are not changed and,
// as in the reference, minData / maxData are not written.  Rows >= 0 come first in ascending
// order, then the negative rows in input order.
void THRUSTDeviceMinMaxSort(float *minDataCUDAPointer, float *maxDataCUDAPointer,
                            int *rowDataCUDAPointer, int n, float *minData, float *maxData,
                            int *rowNumbers) {
  (void)minDataCUDAPointer; (void)maxDataCUDAPointer; (void)minData; (void)maxData;
  if (n <= 0 || !rowNumbers) return;
  std::lock_guard<std::mutex> lk(g_shim.mu);
  const size_t w = al256(4 * (size_t)n) / 4;
  const size_t words = 5 * w + (size_t)sort_temp_words(n);
  if (!shim_reserve(4 * words)) return;
  uint32_t *keys = static_cast<uint32_t *>(g_shim.dev), *vals = keys + w, *kalt = vals + w,
           *valt = kalt + w, *out = valt + w, *temp = out + w;
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_minmax_keys<<<nb, 256>>>(rowDataCUDAPointer, n, keys, vals);
  const bool alt = sort_pairs(keys, vals, kalt, valt, n, 32, temp, 0);
  k_minmax_gather<<<nb, 256>>>(rowDataCUDAPointer, alt ? valt : vals, n, reinterpret_cast<int *>(out));
  count_launch(2);
  cudaMemcpy(rowNumbers, out, 4 * (size_t)n, cudaMemcpyDeviceToHost);
}

}  // extern "C"
