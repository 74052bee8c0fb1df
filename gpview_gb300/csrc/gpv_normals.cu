// gpv_normals.cu -- Level1 and Level2 voxel normals (optional; gpv_set_normals).
//
// Reference semantics (the CPU path):
//   face normal   VectorCrossProduct(v1 - v0, v2 - v0), VectorNormalize (src/Object.cpp:522-526,
//                 includes/FloatVector.h:293-296,333-342), float arithmetic, IEEE sqrt/divide.
//   Level1        for every voxel with recorded triangles: the float sum of their face normals in
//                 list order, divided by the count, normalised (src/Object.cpp:3219-3253);
//                 other voxels 0 (:3151-3152).
//   Level2        every SAT pass of (triangle, sub-cell) adds the face normal and 1 to the cell
//                 (AddPointToVoxel, :2715-2719), triangles in list order; sum / count,
//                 normalised (:2402-2424); cells without a pass 0 (:3309-3310).
// The list order of the CPU path is ascending triangle id (ClassifyTessellation records the
// triangles in file order, :2267-2340); with normals on, the pair sort also orders each voxel's
// triangles by id, so every float sum runs in the reference's order.
//
// Outputs per mode: GPV_NORMALS_BYTES writes the .raw encoding uint8(n * float(256/3) + 127)
// (src/Object.cpp:2940-2941, :3033-3035), three bytes per voxel / cell; GPV_NORMALS_FLOAT writes
// the three floats.
#include "gpv_internal.h"

namespace gpv {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kNWarps = 4;
constexpr int kNTileCells = 512;  // Level2 cells accumulated at once per warp (float4 each)

__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
  const float mag = __fsqrt_rn(fa(fa(fm(x, x), fm(y, y)), fm(z, z)));
  if (mag != 0.f) {
    x = __fdiv_rn(x, mag);
    y = __fdiv_rn(y, mag);
    z = __fdiv_rn(z, mag);
  }
}

__device__ __forceinline__ void store_normal(void *base, int mode, int64_t idx, float x, float y,
                                             float z) {
  if (mode == GPV_NORMALS_FLOAT) {
    float *o = static_cast<float *>(base) + 3 * idx;
    o[0] = x; o[1] = y; o[2] = z;
  } else {
    const float sc = (float)(256.0 / 3.0);
    uint8_t *o = static_cast<uint8_t *>(base) + 3 * idx;
    o[0] = (uint8_t)__float2int_rz(fa(fm(x, sc), 127.f));
    o[1] = (uint8_t)__float2int_rz(fa(fm(y, sc), 127.f));
    o[2] = (uint8_t)__float2int_rz(fa(fm(z, sc), 127.f));
  }
}

template <int64_t MeshDesc::*F>
__device__ __forceinline__ int mesh_by(const MeshDesc *md, int nmesh, int64_t idx) {
  int lo = 0, hi = nmesh - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (md[mid].*F <= idx) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_face_normals(BatchDev bd) {
  const int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= bd.total_tris) return;
  const MeshDesc &d = bd.md[mesh_by<&MeshDesc::tri_base>(bd.md, bd.nmesh, gi)];
  const int64_t t = gi - d.tri_base;
  const float *v = d.tris + 9 * t;
  const float a0 = fs(v[3], v[0]), a1 = fs(v[4], v[1]), a2 = fs(v[5], v[2]);
  const float b0 = fs(v[6], v[0]), b1 = fs(v[7], v[1]), b2 = fs(v[8], v[2]);
  float x = fs(fm(a1, b2), fm(b1, a2));
  float y = fs(fm(a2, b0), fm(b2, a0));
  float z = fs(fm(a0, b1), fm(b0, a1));
  normalize3(x, y, z);
  d.fnorm[t] = make_float4(x, y, z, 0.f);
}

// One thread per boundary voxel of the sorted meshes: sum in list order, average, normalise.
__global__ void __launch_bounds__(256) k_level1_normals(BatchDev bd, const uint32_t *__restrict__ keys,
                                                        const uint32_t *__restrict__ vals,
                                                        const uint32_t *__restrict__ useg, int64_t U) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= U) return;
  const MeshDesc &d = bd.md[mesh_by<&MeshDesc::u_base>(bd.md, bd.nmesh, u)];
  const uint32_t e0 = useg[u], e1 = useg[u + 1];
  float sx = 0.f, sy = 0.f, sz = 0.f;
  for (uint32_t e = e0; e < e1; ++e) {
    const float4 f = __ldg(d.fnorm + (vals[e] & 0x7fffffffu));
    sx = fa(sx, f.x);
    sy = fa(sy, f.y);
    sz = fa(sz, f.z);
  }
  const float cnt = (float)(e1 - e0);
  float x = __fdiv_rn(sx, cnt), y = __fdiv_rn(sy, cnt), z = __fdiv_rn(sz, cnt);
  normalize3(x, y, z);
  const int nx = d.g.n[0], ny = d.g.n[1], nz = d.g.n[2];
  const uint32_t key = keys[e0];  // column-major: (j*nx + i)*nz + k
  const uint32_t col = key / (uint32_t)nz;
  const int64_t vlin = ((int64_t)(key - col * (uint32_t)nz) * ny + col / (uint32_t)nx) * nx +
                       col % (uint32_t)nx;
  store_normal(d.l1n, bd.normals, vlin, x, y, z);
}

// One warp per boundary voxel of a Level2 mesh (grid-stride).  The voxel's cells are taken in
// tiles of kNTileCells consecutive cells (cell order r, q, p); for each tile the voxel's triangles
// run in list order, each one's candidate cells (the triangle's box, clipped to the tile's z
// layers) tested by the exact SAT across the lanes and accumulated in shared memory (one triangle
// at a time, so each cell's sum follows the list order).
__global__ void __launch_bounds__(kNWarps * 32) k_level2_normals(BatchDev bd,
                                                                 const uint32_t *__restrict__ keys,
                                                                 const uint32_t *__restrict__ vals,
                                                                 const uint32_t *__restrict__ useg,
                                                                 int64_t U) {
  __shared__ float4 s_acc[kNWarps][kNTileCells];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  float4 *acc = s_acc[warp];
  const int64_t nwarps = (int64_t)gridDim.x * kNWarps;
  for (int64_t u = (int64_t)blockIdx.x * kNWarps + warp; u < U; u += nwarps) {
    const MeshDesc &d = bd.md[mesh_by<&MeshDesc::u_base>(bd.md, bd.nmesh, u)];
    if (!d.has_l2) continue;  // warp-uniform
    const GridDev &g = d.g;
    const int nx = g.n[0], nz = g.n[2];
    const int n2x = g.n2[0], n2y = g.n2[1], n2z = g.n2[2];
    const int ncol2 = n2x * n2y, cells = ncol2 * n2z;
    const uint32_t e0 = useg[u], e1 = useg[u + 1];
    const uint32_t key = keys[e0];
    const uint32_t col = key / (uint32_t)nz;
    const int k = (int)(key - col * (uint32_t)nz);
    const int ci = (int)(col % (uint32_t)nx), cj = (int)(col / (uint32_t)nx);
    const int64_t vlin = ((int64_t)k * g.n[1] + cj) * nx + ci;
    const int64_t obase = (int64_t)d.prefix[vlin] * cells;
    const float *sx = g.c2s[0] + (size_t)ci * n2x, *sy = g.c2s[1] + (size_t)cj * n2y,
                *szt = g.c2s[2] + (size_t)k * n2z;
    const float sx0 = __ldg(sx), sy0 = __ldg(sy), sz0 = __ldg(szt);
    for (int c0 = 0; c0 < cells; c0 += kNTileCells) {
      const int c1 = min(cells, c0 + kNTileCells), tc = c1 - c0;
      const int rz0 = c0 / ncol2, rz1 = (c1 - 1) / ncol2;
      for (int c = lane; c < tc; c += 32) acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      __syncwarp();
      for (uint32_t e = e0; e < e1; ++e) {
        const uint32_t t = vals[e] & 0x7fffffffu;
        const float4 a0 = __ldg(d.ptri + 3 * (size_t)t), a1 = __ldg(d.ptri + 3 * (size_t)t + 1),
                     a2 = __ldg(d.ptri + 3 * (size_t)t + 2);
        const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
        const float4 fnv = __ldg(d.fnorm + t);
        int p0, p1, q0, q1, r0, r1;
        l2_cell_range(fminf(V[0], fminf(V[3], V[6])), fmaxf(V[0], fmaxf(V[3], V[6])), sx0,
                      g.e2[0], g.inv_g2[0], n2x, p0, p1);
        l2_cell_range(fminf(V[1], fminf(V[4], V[7])), fmaxf(V[1], fmaxf(V[4], V[7])), sy0,
                      g.e2[1], g.inv_g2[1], n2y, q0, q1);
        l2_cell_range(fminf(V[2], fminf(V[5], V[8])), fmaxf(V[2], fmaxf(V[5], V[8])), sz0,
                      g.e2[2], g.inv_g2[2], n2z, r0, r1);
        r0 = max(r0, rz0);
        r1 = min(r1, rz1);
        const int np = p1 - p0 + 1, nq = q1 - q0 + 1, nr = r1 - r0 + 1;
        if (np > 0 && nq > 0 && nr > 0) {
          const int tot = np * nq * nr;
          for (int w = lane; w < tot; w += 32) {
            const int pr = w / np, p = p0 + (w - pr * np);
            const int qq = pr / nr, r = r0 + (pr - qq * nr), q = q0 + qq;
            const int c = r * ncol2 + q * n2x + p;
            if (c < c0 || c >= c1) continue;
            const float c3[3] = {__ldg(sx + p), __ldg(sy + q), __ldg(szt + r)};
            if (tri_box(V, c3, g.e2)) {
              float4 &a = acc[c - c0];
              a.x = fa(a.x, fnv.x);
              a.y = fa(a.y, fnv.y);
              a.z = fa(a.z, fnv.z);
              a.w = fa(a.w, 1.f);
            }
          }
        }
        __syncwarp();
      }
      for (int c = lane; c < tc; c += 32) {
        const float4 a = acc[c];
        float x = 0.f, y = 0.f, z = 0.f;
        if (a.w > 0.f) {
          x = __fdiv_rn(a.x, a.w);
          y = __fdiv_rn(a.y, a.w);
          z = __fdiv_rn(a.z, a.w);
          normalize3(x, y, z);
        }
        store_normal(d.l2n, bd.normals, obase + c0 + c, x, y, z);
      }
      __syncwarp();
    }
  }
}

}  // namespace

void launch_face_normals(const BatchDev &bd, cudaStream_t s) {
  if (bd.total_tris <= 0) return;
  k_face_normals<<<(unsigned)((bd.total_tris + 255) / 256), 256, 0, s>>>(bd);
  count_launch();
}

void launch_normals(const BatchDev &bd, const uint32_t *keys, const uint32_t *vals,
                    const uint32_t *useg, int64_t U, bool any_l2, int num_sms, cudaStream_t s) {
  if (U <= 0) return;
  k_level1_normals<<<(unsigned)((U + 255) / 256), 256, 0, s>>>(bd, keys, vals, useg, U);
  count_launch();
  if (!any_l2) return;
  const int64_t grid = std::min<int64_t>((U + kNWarps - 1) / kNWarps, (int64_t)num_sms * 8);
  k_level2_normals<<<(unsigned)grid, kNWarps * 32, 0, s>>>(bd, keys, vals, useg, U);
  count_launch();
}

}  // namespace gpv
