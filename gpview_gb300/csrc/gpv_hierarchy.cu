// gpv_hierarchy.cu -- the voxel box hierarchy of Object::BuildHierarchy (src/Object.cpp:2790-2867)
// on the device, one launch per level.
//
// Leaves are the Level1 voxel boxes as PerformVoxelization initialises them (src/Object.cpp:
// 3176-3187): centre = the Level1 centre table, half size = the Level1 extents, solid = the inside
// fill's parity (taken before the boundary marks, as the reference sets it right after the fill).
// Level 1 combines x-neighbour leaves (2i, 2i+1); level L >= 2 combines node pairs of level L-1
// along x, y or z by L % 3, with the reference's fallback when that axis is one box wide.
// CombineBBox (src/Object.cpp:2750-2788): two empty boxes give an empty box, one solid box is
// copied, two solid boxes give their bounding box ((max+min)/2, (max-min)/2, float).
#include "gpv_internal.h"

namespace gpv {

namespace {

__device__ __forceinline__ void combine(const gpv_box &a, const gpv_box &b, gpv_box &o) {
  float mid[3] = {0.f, 0.f, 0.f}, half[3] = {0.f, 0.f, 0.f};
  if (a.solid == 0 && b.solid == 0) {
    o.solid = 0;
  } else if (a.solid == 0) {
    o.solid = 1;
    for (int c = 0; c < 3; ++c) { mid[c] = b.mid[c]; half[c] = b.half[c]; }
  } else if (b.solid == 0) {
    o.solid = 1;
    for (int c = 0; c < 3; ++c) { mid[c] = a.mid[c]; half[c] = a.half[c]; }
  } else {
    o.solid = 1;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float amn = fs(a.mid[c], a.half[c]), amx = fa(a.mid[c], a.half[c]);
      const float bmn = fs(b.mid[c], b.half[c]), bmx = fa(b.mid[c], b.half[c]);
      const float mx = (amx < bmx) ? bmx : amx;  // std::max
      const float mn = (bmn < amn) ? bmn : amn;  // std::min
      mid[c] = __fdiv_rn(fa(mx, mn), 2.0f);
      half[c] = __fdiv_rn(fs(mx, mn), 2.0f);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) { o.mid[c] = mid[c]; o.half[c] = half[c]; }
  o.child1 = a.index;
  o.child2 = b.index;
}

__global__ void __launch_bounds__(256) k_hier_leaves(GridDev g, const uint32_t *__restrict__ iplane,
                                                     int64_t half_n, gpv_box *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= half_n) return;
  const int nx = g.n[0], ny = g.n[1];
  gpv_box leaf[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int64_t v = 2 * i + h;
    const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((int64_t)nx * ny));
    leaf[h].mid[0] = __ldg(g.c1[0] + x);
    leaf[h].mid[1] = __ldg(g.c1[1] + y);
    leaf[h].mid[2] = __ldg(g.c1[2] + z);
#pragma unroll
    for (int c = 0; c < 3; ++c) leaf[h].half[c] = g.e1[c];
    leaf[h].solid = (int)((iplane[((int64_t)z * ny + y) * g.nxw + (x >> 5)] >> (x & 31)) & 1u);
    leaf[h].index = (int32_t)v;
  }
  gpv_box o;
  combine(leaf[0], leaf[1], o);
  o.index = (int32_t)i;
  out[i] = o;
}

__global__ void __launch_bounds__(256) k_hier_level(gpv_box *__restrict__ nodes, int64_t prev,
                                                    int64_t cur, int dx, int dy, int dz, int is,
                                                    int js, int ks) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ox = dx / is, oy = dy / js, oz = dz / ks;
  if (t >= (int64_t)ox * oy * oz) return;
  const int ii = (int)(t % ox), jj = (int)((t / ox) % oy), kk = (int)(t / ((int64_t)ox * oy));
  const int i = ii * is, j = jj * js, k = kk * ks;
  const int64_t i1 = (int64_t)k * dy * dx + (int64_t)j * dx + i;
  const int64_t sk = (int64_t)(ks - 1) * dy * dx + (int64_t)(js - 1) * dx + (is - 1);
  gpv_box o;
  combine(nodes[prev + i1], nodes[prev + i1 + sk], o);
  o.index = (int32_t)(cur + t);
  nodes[cur + t] = o;
}

}  // namespace

int hierarchy_levels(int64_t N1) {
  if (N1 < 2 || (N1 & (N1 - 1))) return 0;
  int lv = 0;
  for (int64_t x = N1; x > 1; x >>= 1) ++lv;
  return lv;
}

// Level-by-level launches for one mesh (N1 a power of two); `out` holds N1 - 1 boxes.
void launch_hierarchy(const GridDev &g, const uint32_t *iplane, gpv_box *out, cudaStream_t s) {
  const int64_t N1 = (int64_t)g.n[0] * g.n[1] * g.n[2];
  const int levels = hierarchy_levels(N1);
  if (!levels) return;
  int64_t nlev = N1 / 2;
  k_hier_leaves<<<(unsigned)((nlev + 255) / 256), 256, 0, s>>>(g, iplane, nlev, out);
  count_launch();
  int dx = g.n[0] / 2, dy = g.n[1], dz = g.n[2];
  int64_t prev = 0, cur = nlev;
  nlev /= 2;
  for (int level = 2; level <= levels; ++level) {
    int is = (level % 3 == 1 && dx > 1) ? 2 : 1;
    int js = (level % 3 == 2 && dy > 1) ? 2 : 1;
    int ks = (level % 3 == 0 && dz > 1) ? 2 : 1;
    if (is == 1 && js == 1 && ks == 1) {
      if (dx > 1) is = 2;
      else if (dy > 1) js = 2;
      else if (dz > 1) ks = 2;
    }
    const int64_t cnt = (int64_t)(dx / is) * (dy / js) * (dz / ks);
    k_hier_level<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(out, prev, cur, dx, dy, dz, is, js, ks);
    count_launch();
    if (is == 2) dx /= 2;
    if (js == 2) dy /= 2;
    if (ks == 2) dz /= 2;
    prev += nlev * 2;
    cur += nlev;
    nlev /= 2;
  }
}

}  // namespace gpv
