// gpv_common.cuh -- device predicates, grid parameters and small PTX helpers shared by the
// voxelization kernels.
//
// Every predicate is written with __fadd_rn/__fsub_rn/__fmul_rn so that no multiply-add is
// contracted whatever the compiler flags, and follows the operation order of the reference's
// CPU code (src/TriBoxIntersection.cpp:64-210, src/TriRayIntersection.cpp:78-131).  The two
// double-precision comparisons of the ray test (det against +-1e-6, t > 1e-6) are evaluated
// exactly in float against `thr`, the largest float below 1e-6:  for a float x,
// (double)x < 1e-6  <=>  x <= thr,  and  (double)x > 1e-6  <=>  x > thr.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gpv {

// Status bits a kernel may raise in MeshStats::status (read back by the host).
enum : uint32_t {
  ST_WAIT_TIMEOUT = 1u,     // a bounded mbarrier / queue wait gave up
  ST_PAIR_OVERFLOW = 2u,    // pair buffer capacity exceeded (host re-plans)
  ST_BAD_INPUT = 4u,        // non-finite vertex
};

struct MeshStats {
  unsigned long long sat1;        // algorithmic Level1 SAT tests (candidate boxes)
  unsigned long long sat_units;   // (triangle, column) SAT units
  unsigned long long fill_units;  // (triangle, column) fill units
  unsigned long long ray1;        // exact-box (column, triangle) pairs * nz
  unsigned long long pairs;       // emitted (voxel, triangle) records
  unsigned long long boundary;    // Level1 boundary voxels
  unsigned long long l1_inside;   // Level1 voxels with state 1
  unsigned long long l2_inside;   // Level2 cells with state 1
  unsigned long long l2_boundary; // Level2 cells with state 2
  unsigned long long ray2;        // sum |U(b)| * cells
  unsigned long long pair_cap;    // capacity of the pair buffer
  unsigned long long xycells;     // sum over triangles of (x extent + 1)(y extent + 1) in Level2
                                  // cells, times 16: with pairs, the density of Level2 SAT items
  unsigned int status;
  unsigned int pad;
};

// Grid of one mesh, passed by value to the kernels.
struct GridDev {
  float bmin[3], bmax[3];
  int n[3];
  int n2[3];
  float e1[3], e2[3], g[3], g2[3];
  const float *c1[3];   // Level1 centres per axis
  const float *c2s[3];  // Level2 SAT centres [i*n2+p]
  const float *o2[3];   // Level2 ray origins [i*n2+p]
  int nxw;              // 32-bit words per x row of the Level1 bit planes
  int nzw;              // 32-bit words per column of the toggle plane
  int key_bits;         // bits of the column-major voxel key
  float thr;            // largest float below 1e-6
  int oz_monotone;      // Level2 ray-origin heights strictly increase along every column
  float inv_g2[3];      // 1 / gridSize2 (range arithmetic only, never inside a predicate)
  const float *sp1;     // stencil fill: Level1 slice clip heights [k] (Level2 uses o2[2])
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

// Level1 cell of a coordinate: int(((v-min)/(max-min))*n) with the decrement at v == max
// (src/Object.cpp:2280-2306).  The quotient is clamped to [-1, n+1] before the conversion so
// that vertices outside the grid (undefined in the reference) give a defined index.
__device__ __forceinline__ int cell_of(float v, float mn, float mx, int n) {
  float q = fm(__fdiv_rn(fs(v, mn), fs(mx, mn)), (float)n);
  q = fminf(fmaxf(q, -1.0f), (float)n + 1.0f);
  int c = __float2int_rz(q);
  if (c == n && v == mx) c--;
  return c;
}

// One edge-cross-axis test; true when the axis separates.
__device__ __forceinline__ bool sep(float pa, float pb, float rad) {
  float mn = pa < pb ? pa : pb;
  float mx = pa < pb ? pb : pa;
  return (mn > rad) || (mx < -rad);
}

// ---- SAT split into the part that depends only on the box's x/y centre and the part that
// depends on its z centre.  The boolean result is the conjunction of all axis tests, so testing
// the z-invariant axes once per column is exact.
struct SatCol {
  float v0x, v1x, v2x, v0y, v1y, v2y;
  float e0x, e0y, e1x, e1y, e2x, e2y;
};

// The translated x/y vertex coordinates and edges of sat_col, without its tests (for a column
// already known to pass them).
__device__ __forceinline__ void sat_col_values(const float *V, float cx, float cy, SatCol &s) {
  s.v0x = fs(V[0], cx); s.v1x = fs(V[3], cx); s.v2x = fs(V[6], cx);
  s.v0y = fs(V[1], cy); s.v1y = fs(V[4], cy); s.v2y = fs(V[7], cy);
  s.e0x = fs(s.v1x, s.v0x); s.e0y = fs(s.v1y, s.v0y);
  s.e1x = fs(s.v2x, s.v1x); s.e1y = fs(s.v2y, s.v1y);
  s.e2x = fs(s.v0x, s.v2x); s.e2y = fs(s.v0y, s.v2y);
}

// z-invariant part: the three Z-axis edge tests and the x/y box axes.  False = separated.
__device__ __forceinline__ bool sat_col(const float *V, float cx, float cy, const float h[3],
                                        SatCol &s) {
  sat_col_values(V, cx, cy, s);
  float fx, fy;
  // edge 0, Z12: a = e0y, b = e0x on v1, v2
  fx = fabsf(s.e0x); fy = fabsf(s.e0y);
  if (sep(fs(fm(s.e0y, s.v1x), fm(s.e0x, s.v1y)), fs(fm(s.e0y, s.v2x), fm(s.e0x, s.v2y)),
          fa(fm(fy, h[0]), fm(fx, h[1])))) return false;
  // edge 1, Z0: a = e1y, b = e1x on v0, v1
  fx = fabsf(s.e1x); fy = fabsf(s.e1y);
  if (sep(fs(fm(s.e1y, s.v0x), fm(s.e1x, s.v0y)), fs(fm(s.e1y, s.v1x), fm(s.e1x, s.v1y)),
          fa(fm(fy, h[0]), fm(fx, h[1])))) return false;
  // edge 2, Z12: a = e2y, b = e2x on v1, v2
  fx = fabsf(s.e2x); fy = fabsf(s.e2y);
  if (sep(fs(fm(s.e2y, s.v1x), fm(s.e2x, s.v1y)), fs(fm(s.e2y, s.v2x), fm(s.e2x, s.v2y)),
          fa(fm(fy, h[0]), fm(fx, h[1])))) return false;
  // box x and y axes
  float mn = s.v0x, mx = s.v0x;
  if (s.v1x < mn) mn = s.v1x;
  if (s.v1x > mx) mx = s.v1x;
  if (s.v2x < mn) mn = s.v2x;
  if (s.v2x > mx) mx = s.v2x;
  if (mn > h[0] || mx < -h[0]) return false;
  mn = s.v0y; mx = s.v0y;
  if (s.v1y < mn) mn = s.v1y;
  if (s.v1y > mx) mx = s.v1y;
  if (s.v2y < mn) mn = s.v2y;
  if (s.v2y > mx) mx = s.v2y;
  if (mn > h[1] || mx < -h[1]) return false;
  return true;
}

// z-dependent part: X and Y edge tests, box z axis, triangle plane.  True = overlap.
__device__ __forceinline__ bool sat_z(const SatCol &s, const float *V, float cz,
                                      const float h[3]) {
  const float v0z = fs(V[2], cz), v1z = fs(V[5], cz), v2z = fs(V[8], cz);
  const float e0z = fs(v1z, v0z), e1z = fs(v2z, v1z), e2z = fs(v0z, v2z);
  float fx, fy, fz;
  // edge 0: X01 (a=e0z, b=e0y; v0, v2), Y02 (a=e0z, b=e0x; v0, v2)
  fx = fabsf(s.e0x); fy = fabsf(s.e0y); fz = fabsf(e0z);
  if (sep(fs(fm(e0z, s.v0y), fm(s.e0y, v0z)), fs(fm(e0z, s.v2y), fm(s.e0y, v2z)),
          fa(fm(fz, h[1]), fm(fy, h[2])))) return false;
  if (sep(fa(fm(-e0z, s.v0x), fm(s.e0x, v0z)), fa(fm(-e0z, s.v2x), fm(s.e0x, v2z)),
          fa(fm(fz, h[0]), fm(fx, h[2])))) return false;
  // edge 1: X01 (v0, v2), Y02 (v0, v2)
  fx = fabsf(s.e1x); fy = fabsf(s.e1y); fz = fabsf(e1z);
  if (sep(fs(fm(e1z, s.v0y), fm(s.e1y, v0z)), fs(fm(e1z, s.v2y), fm(s.e1y, v2z)),
          fa(fm(fz, h[1]), fm(fy, h[2])))) return false;
  if (sep(fa(fm(-e1z, s.v0x), fm(s.e1x, v0z)), fa(fm(-e1z, s.v2x), fm(s.e1x, v2z)),
          fa(fm(fz, h[0]), fm(fx, h[2])))) return false;
  // edge 2: X2 (v0, v1), Y1 (v0, v1)
  fx = fabsf(s.e2x); fy = fabsf(s.e2y); fz = fabsf(e2z);
  if (sep(fs(fm(e2z, s.v0y), fm(s.e2y, v0z)), fs(fm(e2z, s.v1y), fm(s.e2y, v1z)),
          fa(fm(fz, h[1]), fm(fy, h[2])))) return false;
  if (sep(fa(fm(-e2z, s.v0x), fm(s.e2x, v0z)), fa(fm(-e2z, s.v1x), fm(s.e2x, v1z)),
          fa(fm(fz, h[0]), fm(fx, h[2])))) return false;
  // box z axis
  float mn = v0z, mx = v0z;
  if (v1z < mn) mn = v1z;
  if (v1z > mx) mx = v1z;
  if (v2z < mn) mn = v2z;
  if (v2z > mx) mx = v2z;
  if (mn > h[2] || mx < -h[2]) return false;
  // plane: normal = e0 x e1, planeBoxOverlap(normal, v0, h)
  const float nx = fs(fm(s.e0y, e1z), fm(e0z, s.e1y));
  const float ny = fs(fm(e0z, s.e1x), fm(s.e0x, e1z));
  const float nz = fs(fm(s.e0x, s.e1y), fm(s.e0y, s.e1x));
  float lo0, hi0, lo1, hi1, lo2, hi2;
  if (nx > 0.0f) { lo0 = fs(-h[0], s.v0x); hi0 = fs(h[0], s.v0x); }
  else           { lo0 = fs(h[0], s.v0x);  hi0 = fs(-h[0], s.v0x); }
  if (ny > 0.0f) { lo1 = fs(-h[1], s.v0y); hi1 = fs(h[1], s.v0y); }
  else           { lo1 = fs(h[1], s.v0y);  hi1 = fs(-h[1], s.v0y); }
  if (nz > 0.0f) { lo2 = fs(-h[2], v0z);   hi2 = fs(h[2], v0z); }
  else           { lo2 = fs(h[2], v0z);    hi2 = fs(-h[2], v0z); }
  if (fa(fa(fm(nx, lo0), fm(ny, lo1)), fm(nz, lo2)) > 0.0f) return false;
  return fa(fa(fm(nx, hi0), fm(ny, hi1)), fm(nz, hi2)) >= 0.0f;
}

// Sub-cells along one axis whose box can meet [tmin, tmax].  Cell p spans
// [c2s[p] - h, c2s[p] + h] ~ [vmin + p g2, vmin + (p+1) g2]; a cell whose box misses
// [tmin - delta, tmax + delta] is rejected by the SAT's own box-axis test (delta covers the
// rounding of the coordinates and of this computation, the 1e-3 cell margin that of the
// quotient).
__device__ __forceinline__ void l2_cell_range(float tmin, float tmax, float c0, float h,
                                              float inv_g2, int n2, int &lo, int &hi) {
  const float vmin = c0 - h;
  const float delta = 8.f * 5.9604644775390625e-08f * (fabsf(tmin) + fabsf(tmax) + fabsf(vmin) + h) + 1e-30f;
  // first p with vmin + (p+1) g2 >= tmin - delta, last p with vmin + p g2 <= tmax + delta
  // (the reciprocal's rounding moves the quotients by far less than the 1e-3 cell margin)
  float f0 = (tmin - delta - vmin) * inv_g2 - 1e-3f;
  float f1 = (tmax + delta - vmin) * inv_g2 + 1e-3f;
  f0 = fminf(fmaxf(f0, -4.f), (float)n2 + 4.f);
  f1 = fminf(fmaxf(f1, -4.f), (float)n2 + 4.f);
  lo = max((int)floorf(f0), 0);
  hi = min((int)floorf(f1), n2 - 1);
}

__device__ __forceinline__ bool tri_box(const float *V, const float c[3], const float h[3]) {
  SatCol s;
  if (!sat_col(V, c[0], c[1], h, s)) return false;
  return sat_z(s, V, c[2], h);
}

// ---- +z Moller-Trumbore split into the column part (u, v) and the height part (t).  With the
// direction (0,0,1) the reference's products with the zero components only add signed zeros.
struct RayTri {  // per-triangle constants
  float v1x, v1y, v1z, e1x, e1y, e1z, e2x, e2y, e2z, inv_det;
  bool ok;       // det passed the |det| > 1e-6 test
};

__device__ __forceinline__ void ray_tri(const float *V, float thr, RayTri &r) {
  r.v1x = V[0]; r.v1y = V[1]; r.v1z = V[2];
  r.e1x = fs(V[3], V[0]); r.e1y = fs(V[4], V[1]); r.e1z = fs(V[5], V[2]);
  r.e2x = fs(V[6], V[0]); r.e2y = fs(V[7], V[1]); r.e2z = fs(V[8], V[2]);
  const float det = fa(fm(r.e1x, -r.e2y), fm(r.e1y, r.e2x));
  r.ok = (det < -thr) || (det > thr);
  r.inv_det = __fdiv_rn(1.0f, det);
}

// Same constants with 1/det taken from the per-triangle record written by the prep kernel
// (computed there with the same __fdiv_rn(1, det)); `ok` is not evaluated here -- callers skip
// triangles whose conservative ray box is empty, which is the case exactly when det fails.
__device__ __forceinline__ void ray_tri_pre(const float *V, float inv_det, RayTri &r) {
  r.v1x = V[0]; r.v1y = V[1]; r.v1z = V[2];
  r.e1x = fs(V[3], V[0]); r.e1y = fs(V[4], V[1]); r.e1z = fs(V[5], V[2]);
  r.e2x = fs(V[6], V[0]); r.e2y = fs(V[7], V[1]); r.e2z = fs(V[8], V[2]);
  r.inv_det = inv_det;
  r.ok = true;
}

struct RayCol { float Tx, Ty; };

// u/v tests of one column; true when the column passes.
__device__ __forceinline__ bool ray_col(const RayTri &r, float ox, float oy, RayCol &c) {
  c.Tx = fs(ox, r.v1x);
  c.Ty = fs(oy, r.v1y);
  const float u = fm(fa(fm(c.Tx, -r.e2y), fm(c.Ty, r.e2x)), r.inv_det);
  if (u < 0.f || u > 1.f) return false;
  const float v = fm(fs(fm(c.Tx, r.e1y), fm(c.Ty, r.e1x)), r.inv_det);
  if (v < 0.f || fa(u, v) > 1.f) return false;
  return true;
}

// t > 1e-6 for one origin height.
__device__ __forceinline__ bool ray_t(const RayTri &r, const RayCol &c, float oz, float thr) {
  const float Tz = fs(oz, r.v1z);
  const float q0 = fs(fm(c.Ty, r.e1z), fm(Tz, r.e1y));
  const float q1 = fs(fm(Tz, r.e1x), fm(c.Tx, r.e1z));
  const float q2 = fs(fm(c.Tx, r.e1y), fm(c.Ty, r.e1x));
  const float t = fm(fa(fa(fm(r.e2x, q0), fm(r.e2y, q1)), fm(r.e2z, q2)), r.inv_det);
  return t > thr;
}

// ---- PTX helpers: mbarrier + bulk async copy (TMA, non-tensor) into this CTA's shared memory.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` polls and returns false (the caller raises
// ST_WAIT_TIMEOUT and leaves the tile).  Never traps.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// ---- stencil fill (ClassifyInOut2x, src/Object.cpp:1446-1649; ClassifyInOut2xLevel2,
// :1210-1444): the triangles are drawn into an orthographic viewport of SW x SH pixels over
// [lx, hx] x [ly, hy]; a pixel (sample) counts a triangle when its centre is covered and the
// surface there lies at or below the slice's clip height (glClipPlane (0, 0, -1, c) keeps
// z <= c).  Window coordinates are snapped to 1/256 pixel (8 sub-pixel bits, clamped to
// +-2^21 pixels), coverage is decided by exact integer edge functions with a top-left rule
// (a sample on an edge shared by two triangles counts once), and the height is interpolated
// from the barycentric weights in float.
struct StTri {
  int32_t X[3], Y[3];  // snapped window coordinates, counter-clockwise
  float z[3];
  float rA;            // 1 / (twice the snapped area)
  int sx0, sx1, sy0, sy1;  // samples whose centres lie in the snapped bounding box
};

__device__ __forceinline__ int32_t st_snap(float v, float lo, float hi, int npx) {
  float w = fm(__fdiv_rn(fs(v, lo), fs(hi, lo)), (float)npx);
  w = (w > -2097152.0f) ? fminf(w, 2097152.0f) : -2097152.0f;  // NaN to the low clamp
  return (int32_t)__float2ll_rn(fm(w, 256.0f));
}

// false: zero snapped area, or no sample centre inside the viewport and the triangle's box.
__device__ __forceinline__ bool st_setup(const float *V, float lx, float hx, float ly, float hy,
                                         int SW, int SH, StTri &t) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    t.X[i] = st_snap(V[3 * i], lx, hx, SW);
    t.Y[i] = st_snap(V[3 * i + 1], ly, hy, SH);
    t.z[i] = V[3 * i + 2];
  }
  long long A = (long long)(t.X[1] - t.X[0]) * (t.Y[2] - t.Y[0]) -
                (long long)(t.Y[1] - t.Y[0]) * (t.X[2] - t.X[0]);
  if (A == 0) return false;
  if (A < 0) {
    int32_t a = t.X[1]; t.X[1] = t.X[2]; t.X[2] = a;
    a = t.Y[1]; t.Y[1] = t.Y[2]; t.Y[2] = a;
    const float f = t.z[1]; t.z[1] = t.z[2]; t.z[2] = f;
    A = -A;
  }
  t.rA = __frcp_rn(__ll2float_rn(A));
  const int32_t xmn = min(t.X[0], min(t.X[1], t.X[2])), xmx = max(t.X[0], max(t.X[1], t.X[2]));
  const int32_t ymn = min(t.Y[0], min(t.Y[1], t.Y[2])), ymx = max(t.Y[0], max(t.Y[1], t.Y[2]));
  // sample centres 256 s + 128 within [mn, mx]: ceil((mn - 128) / 256) .. floor((mx - 128) / 256)
  t.sx0 = max(-((128 - xmn) >> 8), 0);
  t.sx1 = min((xmx - 128) >> 8, SW - 1);
  t.sy0 = max(-((128 - ymn) >> 8), 0);
  t.sy1 = min((ymx - 128) >> 8, SH - 1);
  return t.sx0 <= t.sx1 && t.sy0 <= t.sy1;
}

__device__ __forceinline__ bool st_edge_in(long long w, int32_t dx, int32_t dy) {
  return w > 0 || (w == 0 && (dy < 0 || (dy == 0 && dx > 0)));
}

// Coverage of sample (sx, sy) and the interpolated surface height there.
__device__ __forceinline__ bool st_cover(const StTri &t, int sx, int sy, float &zs) {
  const long long px = (long long)sx * 256 + 128, py = (long long)sy * 256 + 128;
  const int32_t dx0 = t.X[2] - t.X[1], dy0 = t.Y[2] - t.Y[1];
  const long long w0 = (long long)dx0 * (py - t.Y[1]) - (long long)dy0 * (px - t.X[1]);
  if (!st_edge_in(w0, dx0, dy0)) return false;
  const int32_t dx1 = t.X[0] - t.X[2], dy1 = t.Y[0] - t.Y[2];
  const long long w1 = (long long)dx1 * (py - t.Y[2]) - (long long)dy1 * (px - t.X[2]);
  if (!st_edge_in(w1, dx1, dy1)) return false;
  const int32_t dx2 = t.X[1] - t.X[0], dy2 = t.Y[1] - t.Y[0];
  const long long w2 = (long long)dx2 * (py - t.Y[0]) - (long long)dy2 * (px - t.X[0]);
  if (!st_edge_in(w2, dx2, dy2)) return false;
  zs = fa(fa(fm(fm(__ll2float_rn(w0), t.rA), t.z[0]), fm(fm(__ll2float_rn(w1), t.rA), t.z[1])),
          fm(fm(__ll2float_rn(w2), t.rA), t.z[2]));
  return true;
}

// First index in [0, n] with tab[i] >= x (tab increasing): the lowest slice whose clip height
// keeps a surface point at height x.
__device__ __forceinline__ int st_first_slice(const float *tab, int n, float x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(tab + mid) >= x) hi = mid; else lo = mid + 1;
  }
  return lo;
}

}  // namespace gpv
