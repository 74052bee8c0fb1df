// gpv_shims.cu -- the reference-named C entry points GPView's Object class binds
// (includes/CUDAUtilities.h:63-64, :87-89), with the same signatures, caller-owned device
// buffers, legacy default stream and "return 1" convention.
//
// Arithmetic follows the reference's CPU code, not its CUDA-8 kernels: box centres are the CPU's
// double-then-float expressions, predicates run without contraction (the reference kernels let
// nvcc fuse multiply-adds, so their results could differ from its own CPU path).  Where a shim's
// inputs do not carry what the CPU formula needs (the Level2 ray origins of
// CUDAClassifyInOutLevel2), the reference kernel's own FP32 formula is used, evaluated without
// contraction.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gpv_internal.h"

namespace gpv {
namespace {

// CUDAClassifyTessellationKernel (cuda/CUDAClassifyTessellation.cu:320-401), one thread per
// triangle over its candidate box; the per-voxel list never writes past triBufferLen.
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

// CUDAClassifyTessellationLevel2Kernel (.cu:403-448): one thread per (boundary voxel, cell).
// Centres come from `cen` ([b][n2x | n2y | n2z] floats, formed on the host as the CPU does:
// float(((p+0.5)*gridSize2 + mid) - ext1) in double, src/Object.cpp:2389-2391); the CPU's unit
// face normals are summed in list order.
__global__ void k_shim_level2_sat(const float *__restrict__ tris, float *__restrict__ l2,
                                  float *__restrict__ nrm, const float *__restrict__ cen,
                                  const int *__restrict__ l2index, const int *__restrict__ cnt,
                                  const int *__restrict__ flatIndex, const int *__restrict__ flat,
                                  int B, int3 n2, float3 e2) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cells = n2.x * n2.y * n2.z;
  if (gid >= (int64_t)B * cells) return;
  const int b = (int)(gid / cells), c = (int)(gid % cells);
  const int r = c / (n2.x * n2.y), q = (c / n2.x) % n2.y, p = c % n2.x;
  const int v = l2index[b];
  const float *cb = cen + (size_t)b * (n2.x + n2.y + n2.z);
  const float cc[3] = {cb[p], cb[n2.x + q], cb[n2.x + n2.y + r]};
  const float h[3] = {e2.x, e2.y, e2.z};
  const int n = cnt[v], f0 = flatIndex[v];
  for (int k = 0; k < n; ++k) {
    const int t = flat[f0 + k];
    float V[9];
    for (int j = 0; j < 9; ++j) V[j] = tris[9 * (size_t)t + j];
    if (!tri_box(V, cc, h)) continue;
    float fn[3];
    face_normal(V, fn);
    const size_t o = (size_t)b * cells + c;
    l2[o] = 2.0f;
    nrm[4 * o + 0] = fa(nrm[4 * o + 0], fn[0]);
    nrm[4 * o + 1] = fa(nrm[4 * o + 1], fn[1]);
    nrm[4 * o + 2] = fa(nrm[4 * o + 2], fn[2]);
    nrm[4 * o + 3] = fa(nrm[4 * o + 3], 1.0f);
  }
}

// CUDAClassifyInOutLevel2Kernel (.cu:450-504): one thread per (boundary voxel, cell), +z parity
// against the x/y-column list.  Origin: (2p+1)*ext2 + mid - ext1 in float, left to right.
__global__ void k_shim_level2_fill(const float *__restrict__ tris, float *__restrict__ l2,
                                   const float *__restrict__ mid, const int *__restrict__ l2index,
                                   const int *__restrict__ xycnt, const int *__restrict__ xyIndex,
                                   const int *__restrict__ xyflat, int B, int3 nd, int3 n2,
                                   float3 e1, float3 e2, float thr) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cells = n2.x * n2.y * n2.z;
  if (gid >= (int64_t)B * cells) return;
  const int b = (int)(gid / cells), c = (int)(gid % cells);
  const int r = c / (n2.x * n2.y), q = (c / n2.x) % n2.y, p = c % n2.x;
  const int v = l2index[b];
  const int xy = v % (nd.x * nd.y);
  const float ox = fs(fa(fm((float)(2 * p + 1), e2.x), mid[3 * b + 0]), e1.x);
  const float oy = fs(fa(fm((float)(2 * q + 1), e2.y), mid[3 * b + 1]), e1.y);
  const float oz = fs(fa(fm((float)(2 * r + 1), e2.z), mid[3 * b + 2]), e1.z);
  int hits = 0;
  const int n = xycnt[xy], f0 = xyIndex[xy];
  for (int k = 0; k < n; ++k) {
    const int t = xyflat[f0 + k];
    float V[9];
    for (int j = 0; j < 9; ++j) V[j] = tris[9 * (size_t)t + j];
    RayTri rt;
    ray_tri(V, thr, rt);
    if (!rt.ok) continue;
    RayCol rc;
    if (!ray_col(rt, ox, oy, rc)) continue;
    hits += ray_t(rt, rc, oz, thr) ? 1 : 0;
  }
  if (hits % 2 == 1) l2[(size_t)b * cells + c] = 1.0f;
}

}  // namespace
}  // namespace gpv

using namespace gpv;

extern "C" {

void InitializeCUDA(void) {
  // CUTGetMaxGflopsDeviceID (includes/CUDAUtilities.h:32-61): most SMs x clock.
  int n = 0;
  cudaGetDeviceCount(&n);
  int best = 0;
  long long best_score = -1;
  for (int d = 0; d < n; ++d) {
    int sms = 0, clk = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, d);
    if ((long long)sms * clk > best_score) {
      best_score = (long long)sms * clk;
      best = d;
    }
  }
  cudaSetDevice(best);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, best) == cudaSuccess) std::printf("Device in use : %s\n", prop.name);
  CUDACheckErrors(" Init ");
}

void CUDACheckErrors(char const *label) {
  // src/CUDAUtilities.cpp:33-49: synchronise, read the last error, print it, continue.
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) std::printf("CUDA Error: %s %s\n", label ? label : "", cudaGetErrorString(e));
}

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
  std::vector<float> tab;
  for (int a = 0; a < 3; ++a) tab.insert(tab.end(), gh.c1[a].begin(), gh.c1[a].end());
  float *d_tab = nullptr;
  if (cudaMalloc(&d_tab, tab.size() * sizeof(float)) != cudaSuccess) return 1;
  cudaMemcpy(d_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice);
  GridDev g;
  std::memset(&g, 0, sizeof(g));
  for (int a = 0; a < 3; ++a) {
    g.bmin[a] = spec.bbox_min[a];
    g.bmax[a] = spec.bbox_max[a];
    g.n[a] = gh.n[a];
    g.e1[a] = gh.e1[a];
  }
  g.c1[0] = d_tab;
  g.c1[1] = d_tab + gh.n[0];
  g.c1[2] = d_tab + gh.n[0] + gh.n[1];
  k_shim_level1<<<(numTriangles + 127) / 128, 128>>>(trianglesCUDAData, numTriangles,
                                                      inOutCUDAData, voxelTriCountCUDAData,
                                                      voxelTriIndexCUDAData, g, triBufferLen);
  count_launch();
  cudaFree(d_tab);  // ordered after the kernel on the legacy stream
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
  // Midpoints are device data: bring them over, form the centre table in double on the host.
  const int nn = numDiv2.x + numDiv2.y + numDiv2.z;
  std::vector<float> mid((size_t)numBoundary * 3), cen((size_t)numBoundary * nn);
  if (cudaMemcpy(mid.data(), level1MidPointCUDAData, mid.size() * sizeof(float),
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    return 1;
  const float e1[3] = {boxExtentsLevel1.x, boxExtentsLevel1.y, boxExtentsLevel1.z};
  const float e2[3] = {boxExtentsLevel2.x, boxExtentsLevel2.y, boxExtentsLevel2.z};
  const int n2[3] = {numDiv2.x, numDiv2.y, numDiv2.z};
  for (int b = 0; b < numBoundary; ++b)
    for (int a = 0, o = 0; a < 3; o += n2[a], ++a) {
      const float g2 = e2[a] * 2.0f;  // gridSize2 (exact: ext2 = gridSize2 / 2)
      for (int p = 0; p < n2[a]; ++p)
        cen[(size_t)b * nn + o + p] = (float)((p + 0.5) * g2 + (double)mid[3 * (size_t)b + a] - e1[a]);
    }
  float *d_cen = nullptr;
  if (cudaMalloc(&d_cen, cen.size() * sizeof(float)) != cudaSuccess) return 1;
  cudaMemcpy(d_cen, cen.data(), cen.size() * sizeof(float), cudaMemcpyHostToDevice);
  const int64_t n = (int64_t)numBoundary * cells;
  k_shim_level2_sat<<<(unsigned)((n + 127) / 128), 128>>>(
      trianglesCUDAData, level2InOutCUDAData, level2NormalCUDAData, d_cen, level2IndexCUDAData,
      voxelTriCountCUDAData, level1TriFlatIndexCUDAData, level1TriFlatCUDAData, numBoundary,
      numDiv2, boxExtentsLevel2);
  count_launch();
  cudaFree(d_cen);
  return 1;
}

int CUDAClassifyInOutLevel2(float *trianglesCUDAData, float *level2InOutCUDAData,
                            float *level1MidPointCUDAData, int *level2IndexCUDAData,
                            int *xyTriCountCUDAData, int *xyTriFlatIndexCUDAData,
                            int *xyTriFlatCUDAData, int numBoundary, int3 numDiv, int3 numDiv2,
                            float3 boxExtentsLevel1, float3 boxExtentsLevel2) {
  const int cells = numDiv2.x * numDiv2.y * numDiv2.z;
  if (numBoundary <= 0 || cells <= 0) return 1;
  const int64_t n = (int64_t)numBoundary * cells;
  k_shim_level2_fill<<<(unsigned)((n + 127) / 128), 128>>>(
      trianglesCUDAData, level2InOutCUDAData, level1MidPointCUDAData, level2IndexCUDAData,
      xyTriCountCUDAData, xyTriFlatIndexCUDAData, xyTriFlatCUDAData, numBoundary, numDiv, numDiv2,
      boxExtentsLevel1, boxExtentsLevel2, eps_threshold());
  count_launch();
  return 1;
}

}  // extern "C"
