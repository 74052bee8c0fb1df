// gpv_stencil.cu -- the stencil (rasterised) inside fill of Level1, ClassifyInOut2x
// (src/Object.cpp:1446-1649), as a CUDA kernel.
//
// The reference renders the whole mesh once per z slice into a 2nx x 2ny stencil buffer
// (orthographic over the bounding box, clip plane z <= slice centre, GL_INCR per fragment) and
// reads the buffer back.  Per (triangle, sample) the set of slices that count the fragment is
// a suffix k >= k0 (the clip heights increase with k), so one toggle bit at k0 in the sample's
// column replaces the nz renderings: the prefix XOR of a sample column's toggles is the parity
// of its stencil count in every slice.  k_fill_finish (gpv_kernels.cu) takes the prefix XORs
// of the four sample columns of each voxel column and keeps the voxels where at least three are
// odd (numInsideCount > 2, :1586-1600), which gives the same inside plane as the ray fill path.
//
// Work: each warp takes 32 triangles; their (triangle, sample) items -- the samples whose centres
// lie in the triangle's snapped box -- are flattened by a warp scan and processed 32 at a time.
#include "gpv_internal.h"

namespace gpv {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kStWarps = 8;

__device__ __forceinline__ int mesh_of_tri(const MeshDesc *md, int nmesh, int64_t gi) {
  int lo = 0, hi = nmesh - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (md[mid].tri_base <= gi) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kStWarps * 32) k_stencil1(BatchDev bd) {
  __shared__ StTri s_t[kStWarps][32];
  __shared__ unsigned long long s_pre[kStWarps][32];
  __shared__ int s_m[kStWarps][32];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const int64_t gi = ((int64_t)blockIdx.x * kStWarps + warp) * 32 + lane;
  unsigned long long cnt = 0;
  if (gi < bd.total_tris) {
    const int m = mesh_of_tri(bd.md, bd.nmesh, gi);
    const MeshDesc &d = bd.md[m];
    const GridDev &g = d.g;
    const int64_t t = gi - d.tri_base;
    const float4 a0 = __ldg(d.ptri + 3 * t), a1 = __ldg(d.ptri + 3 * t + 1), a2 = __ldg(d.ptri + 3 * t + 2);
    const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 9; ++k) finite = finite && isfinite(V[k]);
    StTri st;
    if (finite && st_setup(V, g.bmin[0], g.bmax[0], g.bmin[1], g.bmax[1], 2 * g.n[0], 2 * g.n[1], st)) {
      s_t[warp][lane] = st;
      s_m[warp][lane] = m;
      cnt = (unsigned long long)(st.sx1 - st.sx0 + 1) * (unsigned long long)(st.sy1 - st.sy0 + 1);
    }
  }
  unsigned long long inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long v = __shfl_up_sync(FULL, inc, o);
    if (lane >= (unsigned)o) inc += v;
  }
  s_pre[warp][lane] = inc - cnt;
  const unsigned long long tot = __shfl_sync(FULL, inc, 31);
  __syncwarp();
  for (unsigned long long w = lane; w < tot; w += 32) {
    int tl = 0;  // last triangle slot whose items start at or before w
#pragma unroll
    for (int st = 16; st > 0; st >>= 1)
      if (s_pre[warp][tl + st] <= w) tl += st;
    const StTri &t = s_t[warp][tl];
    const unsigned long long loc = w - s_pre[warp][tl];
    const unsigned nsx = (unsigned)(t.sx1 - t.sx0 + 1);
    unsigned long long row;
    unsigned colo;
    if (loc < 0xffffffffull) {
      row = (unsigned)loc / nsx;
      colo = (unsigned)loc - (unsigned)row * nsx;
    } else {
      row = loc / nsx;
      colo = (unsigned)(loc - row * nsx);
    }
    const int sx = t.sx0 + (int)colo, sy = t.sy0 + (int)row;
    float zs;
    if (!st_cover(t, sx, sy, zs)) continue;
    const MeshDesc &d = bd.md[s_m[warp][tl]];
    const int nz = d.g.n[2];
    const int k0 = st_first_slice(d.g.sp1, nz, zs);
    if (k0 < nz) {
      const size_t scol = (size_t)sy * (size_t)(2 * d.g.n[0]) + (size_t)sx;
      atomicXor(&d.stg[scol * d.g.nzw + (k0 >> 5)], 1u << (k0 & 31));
    }
  }
}

}  // namespace

void launch_stencil1(const BatchDev &bd, cudaStream_t s) {
  if (bd.total_tris <= 0) return;
  const int64_t per_block = kStWarps * 32;
  k_stencil1<<<(unsigned)((bd.total_tris + per_block - 1) / per_block), kStWarps * 32, 0, s>>>(bd);
  count_launch();
}

}  // namespace gpv
