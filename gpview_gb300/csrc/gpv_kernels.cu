// gpv_kernels.cu -- sm_103a kernels of the plain voxelization path.
//
// Pipeline for one mesh (all on one stream):
//   k_prep        per triangle: pack vertices as 3 float4, Level1 SAT candidate box (the
//                 reference's own range, src/Object.cpp:2280-2325), conservative x/y box for the
//                 ray tests, work counts.
//   k_level1      per tile of triangles staged in shared memory by a bulk async copy (TMA):
//                 (a) SAT units = (triangle, column) running the z run top-down; passes set the
//                     boundary bit (atomicOr) and emit (column-major voxel key, triangle|top) pairs;
//                 (b) fill units = (triangle, column) running the column part of the +z
//                     Moller-Trumbore test; passing pairs are queued per warp and the whole warp
//                     evaluates t over the column (one voxel per lane, __ballot_sync), XOR-ing
//                     parity toggles d(k) = hit(k) ^ hit(k+1) into a column-major plane.
//   k_fill_finish warp-level suffix XOR of the toggles per column -> parity, transposed to
//                 the linear (x fastest) inside plane.
//   sort          radix sort of the pairs by column-major voxel key (gpv_sort.cu).
//   k_expand      .raw bytes of Level1, boundaryPrefixSum, boundaryIndex.
//   Level2        gpv_level2.cu.
#include "gpv_internal.h"

namespace gpv {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr float EPS24 = 5.9604644775390625e-08f;  // 2^-24

__device__ __forceinline__ uint32_t pack2(int lo, int hi) {
  return (uint32_t)(lo & 0xffff) | ((uint32_t)(hi & 0xffff) << 16);
}
__device__ __forceinline__ int lo16(uint32_t v) { return (int)(v & 0xffffu); }
__device__ __forceinline__ int hi16(uint32_t v) { return (int)(v >> 16); }

// smallest i in [0,n] with tab[i] >= x (tab nondecreasing); approximate start then adjust.
__device__ __forceinline__ int first_ge(const float *tab, int n, float x, float c0, float g) {
  float f = (x - c0) / g;
  int i;
  if (!(f > 0.f)) i = 0;
  else if (f >= (float)n) i = n;
  else i = (int)ceilf(f);
  while (i > 0 && __ldg(tab + i - 1) >= x) --i;
  while (i < n && __ldg(tab + i) < x) ++i;
  return i;
}
// largest i in [-1,n-1] with tab[i] <= x.
__device__ __forceinline__ int last_le(const float *tab, int n, float x, float c0, float g) {
  float f = (x - c0) / g;
  int i;
  if (!(f > 0.f)) i = -1;
  else if (f >= (float)n) i = n - 1;
  else i = (int)floorf(f);
  while (i < n - 1 && __ldg(tab + i + 1) <= x) ++i;
  while (i >= 0 && __ldg(tab + i) > x) --i;
  return i;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t o = __shfl_up_sync(FULL, v, d);
    if (lane >= (unsigned)d) v += o;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
  return v;
}

// Conservative x/y box of the columns whose +z ray can pass the u/v tests of this triangle.
// Outside the box every column fails them in float arithmetic; ill-conditioned projections get
// the whole plane; triangles failing the |det| test get an empty box.
__device__ __forceinline__ float4 ray_box(const float *V, const GridDev &g) {
  const float e1x = fs(V[3], V[0]), e1y = fs(V[4], V[1]);
  const float e2x = fs(V[6], V[0]), e2y = fs(V[7], V[1]);
  const float det = fa(fm(e1x, -e2y), fm(e1y, e2x));
  const float inf = __int_as_float(0x7f800000);
  if (!(det < -g.thr || det > g.thr)) return make_float4(inf, inf, -inf, -inf);
  const float adet = fabsf(det);
  const float sd = fabsf(e1x * e2y) + fabsf(e1y * e2x);
  const float rel = 4.f * EPS24 * sd / adet;
  if (!(rel <= 0.125f)) return make_float4(-inf, -inf, inf, inf);
  float G = fmaxf(fmaxf(fabsf(g.bmin[0] - V[0]), fabsf(g.bmax[0] - V[0])),
                  fmaxf(fabsf(g.bmin[1] - V[1]), fabsf(g.bmax[1] - V[1])));
  G = G * 1.0001f + 1e-30f;
  const float au = 4.f * EPS24 * G * (fabsf(e2x) + fabsf(e2y)) / adet;
  const float av = 4.f * EPS24 * G * (fabsf(e1x) + fabsf(e1y)) / adet;
  const float mu = 2.f * (rel + au + av) + 1e-6f;
  float lo[2], hi[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    float mn = fminf(V[a], fminf(V[3 + a], V[6 + a]));
    float mx = fmaxf(V[a], fmaxf(V[3 + a], V[6 + a]));
    float w = mx - mn;
    float m = 2.f * mu * w + 8.f * EPS24 * (fabsf(mn) + fabsf(mx) + w) + 1e-30f;
    lo[a] = mn - m;
    hi[a] = mx + m;
  }
  return make_float4(lo[0], lo[1], hi[0], hi[1]);
}

// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_prep(GridDev g, Level1Bufs b) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long sat1 = 0, su = 0, fu = 0, r1 = 0;
  if (t < b.T) {
    float V[9];
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      V[k] = __ldg(b.tris + 9 * t + k);
      finite = finite && isfinite(V[k]);
    }
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int c0 = cell_of(V[a], g.bmin[a], g.bmax[a], g.n[a]);
      const int c1 = cell_of(V[3 + a], g.bmin[a], g.bmax[a], g.n[a]);
      const int c2 = cell_of(V[6 + a], g.bmin[a], g.bmax[a], g.n[a]);
      lo[a] = max(min(c0, min(c1, c2)), 0);
      hi[a] = min(max(c0, max(c1, c2)), g.n[a] - 1);
    }
    float4 fb = ray_box(V, g);
    int fx0 = 1, fx1 = 0, fy0 = 1, fy1 = 0;
    if (!finite) {
      atomicOr(&b.stats->status, (unsigned)ST_BAD_INPUT);
      lo[0] = 1; hi[0] = 0;
      fb = make_float4(1.f, 1.f, 0.f, 0.f);
    } else {
      fx0 = first_ge(g.c1[0], g.n[0], fb.x, g.c1[0][0], g.g[0]);
      fx1 = last_le(g.c1[0], g.n[0], fb.z, g.c1[0][0], g.g[0]);
      fy0 = first_ge(g.c1[1], g.n[1], fb.y, g.c1[1][0], g.g[1]);
      fy1 = last_le(g.c1[1], g.n[1], fb.w, g.c1[1][0], g.g[1]);
      // exact x/y box of the triangle for the ray1 work count
      const float mnx = fminf(V[0], fminf(V[3], V[6])), mxx = fmaxf(V[0], fmaxf(V[3], V[6]));
      const float mny = fminf(V[1], fminf(V[4], V[7])), mxy = fmaxf(V[1], fmaxf(V[4], V[7]));
      const int ax = last_le(g.c1[0], g.n[0], mxx, g.c1[0][0], g.g[0]) -
                     first_ge(g.c1[0], g.n[0], mnx, g.c1[0][0], g.g[0]) + 1;
      const int ay = last_le(g.c1[1], g.n[1], mxy, g.c1[1][0], g.g[1]) -
                     first_ge(g.c1[1], g.n[1], mny, g.c1[1][0], g.g[1]) + 1;
      if (ax > 0 && ay > 0) r1 = (unsigned long long)ax * ay * g.n[2];
    }
    const bool sat_ok = lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2];
    if (sat_ok) {
      su = (unsigned long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1);
      sat1 = su * (hi[2] - lo[2] + 1);
    } else {
      lo[0] = 1; hi[0] = 0;
    }
    if (fx0 <= fx1 && fy0 <= fy1) fu = (unsigned long long)(fx1 - fx0 + 1) * (fy1 - fy0 + 1);
    else { fx0 = 1; fx1 = 0; fy0 = 1; fy1 = 0; }
    b.ptri[3 * t + 0] = make_float4(V[0], V[1], V[2], __uint_as_float(pack2(fx0, fx1)));
    b.ptri[3 * t + 1] = make_float4(V[3], V[4], V[5], __uint_as_float(pack2(fy0, fy1)));
    // 1/det of the +z ray test (src/TriRayIntersection.cpp:310), shared by every column
    const float det = fa(fm(fs(V[3], V[0]), -fs(V[7], V[1])), fm(fs(V[4], V[1]), fs(V[6], V[0])));
    b.ptri[3 * t + 2] = make_float4(V[6], V[7], V[8], __fdiv_rn(1.0f, det));
    b.rng[t] = make_int4((int)pack2(lo[0], hi[0]), (int)pack2(lo[1], hi[1]),
                         (int)pack2(lo[2], hi[2]), 0);
    b.fbox[t] = fb;
  }
  sat1 = warp_sum(sat1); su = warp_sum(su); fu = warp_sum(fu); r1 = warp_sum(r1);
  if ((threadIdx.x & 31u) == 0) {
    if (sat1) atomicAdd(&b.stats->sat1, sat1);
    if (su) atomicAdd(&b.stats->sat_units, su);
    if (fu) atomicAdd(&b.stats->fill_units, fu);
    if (r1) atomicAdd(&b.stats->ray1, r1);
  }
}

// ---------------------------------------------------------------------------------------------
constexpr int kL1Threads = 256;
constexpr int kL1Warps = kL1Threads / 32;
constexpr uint32_t kWaitLimit = 1u << 22;

// last index lt in [0,nt) with off[lt] <= u (off nondecreasing, off[0] = 0)
__device__ __forceinline__ int tile_search(const uint32_t *off, int nt, uint32_t u) {
  int lo = 0, hi = nt - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int TILE>
__global__ void __launch_bounds__(kL1Threads) k_level1(GridDev g, Level1Bufs b) {
  __shared__ __align__(16) float4 s_tri[TILE * 3];
  __shared__ __align__(16) int4 s_rng[TILE];
  __shared__ uint32_t s_soff[TILE + 1];
  __shared__ uint32_t s_foff[TILE + 1];
  __shared__ uint32_t s_q[kL1Warps][32];
  __shared__ __align__(8) uint64_t s_bar;

  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const int64_t t0 = (int64_t)blockIdx.x * TILE;
  const int nt = (int)min((int64_t)TILE, b.T - t0);

  // ---- stage the tile with bulk async copies completing on an mbarrier
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t bt = (uint32_t)nt * 48u, br = (uint32_t)nt * 16u;
    mbar_expect_tx(&s_bar, bt + br);
    bulk_g2s(s_tri, b.ptri + 3 * t0, bt, &s_bar);
    bulk_g2s(s_rng, b.rng + t0, br, &s_bar);
  }
  const bool ok = mbar_wait_bounded(&s_bar, 0, kWaitLimit);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) {
      atomicOr(&b.stats->status, (unsigned)ST_WAIT_TIMEOUT);
      mbar_wait_bounded(&s_bar, 0, kWaitLimit);  // let the copy in flight land before exiting
    }
    return;
  }

  // ---- per-triangle unit counts and their block scan
  uint32_t cs = 0, cf = 0;
  if ((int)threadIdx.x < nt) {
    const int4 r = s_rng[threadIdx.x];
    const int x0 = lo16(r.x), x1 = hi16(r.x), y0 = lo16(r.y), y1 = hi16(r.y);
    if (x0 <= x1 && y0 <= y1) cs = (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1));
    const uint32_t fxr = __float_as_uint(s_tri[3 * threadIdx.x].w);
    const uint32_t fyr = __float_as_uint(s_tri[3 * threadIdx.x + 1].w);
    if (lo16(fxr) <= hi16(fxr) && lo16(fyr) <= hi16(fyr))
      cf = (uint32_t)((hi16(fxr) - lo16(fxr) + 1) * (hi16(fyr) - lo16(fyr) + 1));
  }
  {
    __shared__ uint32_t s_ws[kL1Warps], s_wf[kL1Warps];
    const uint32_t is = warp_incl_scan(cs), iff = warp_incl_scan(cf);
    if (lane == 31) { s_ws[warp] = is; s_wf[warp] = iff; }
    __syncthreads();
    uint32_t bs = 0, bf = 0;
    for (unsigned w = 0; w < warp; ++w) { bs += s_ws[w]; bf += s_wf[w]; }
    if ((int)threadIdx.x < TILE) {
      s_soff[threadIdx.x] = bs + is - cs;
      s_foff[threadIdx.x] = bf + iff - cf;
    }
    if (threadIdx.x == kL1Threads - 1) {
      s_soff[TILE] = bs + is;
      s_foff[TILE] = bf + iff;
    }
    __syncthreads();
  }
  const uint32_t Us = s_soff[TILE], Uf = s_foff[TILE];
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const unsigned lt_mask = (1u << lane) - 1u;
  const uint64_t cap = b.stats->pair_cap;

  // ---- (a) SAT units
  for (uint32_t base = warp * 32u; base < Us; base += kL1Warps * 32u) {
    const uint32_t u = base + lane;
    int lt = 0, p = 0, q = 0, z0 = 0, zc = -1;
    float V[9];
    SatCol sc;
    if (u < Us) {
      lt = tile_search(s_soff, nt, u);
      const int4 r = s_rng[lt];
      const int x0 = lo16(r.x), x1 = hi16(r.x), y0 = lo16(r.y);
      z0 = lo16(r.z);
      const uint32_t c = u - s_soff[lt];
      const int nxr = x1 - x0 + 1;
      p = x0 + (int)(c % (uint32_t)nxr);
      q = y0 + (int)(c / (uint32_t)nxr);
      const float4 a0 = s_tri[3 * lt], a1 = s_tri[3 * lt + 1], a2 = s_tri[3 * lt + 2];
      V[0] = a0.x; V[1] = a0.y; V[2] = a0.z; V[3] = a1.x; V[4] = a1.y; V[5] = a1.z;
      V[6] = a2.x; V[7] = a2.y; V[8] = a2.z;
      if (sat_col(V, __ldg(g.c1[0] + p), __ldg(g.c1[1] + q), g.e1, sc)) zc = hi16(r.z);
    }
    bool first = true;
    const uint32_t tglob = (uint32_t)(t0 + lt);
    while (__any_sync(FULL, zc >= z0)) {
      uint32_t mask = 0;
      const int ztop = zc;
      if (zc >= z0) {
        const int nrun = min(32, zc - z0 + 1);
        for (int d = 0; d < nrun; ++d)
          if (sat_z(sc, V, __ldg(g.c1[2] + (ztop - d)), g.e1)) mask |= 1u << d;
        zc -= nrun;
      }
      const uint32_t cnt = __popc(mask);
      const uint32_t inc = warp_incl_scan(cnt);
      const uint32_t tot = __shfl_sync(FULL, inc, 31);
      unsigned long long basep = 0;
      if (lane == 31 && tot) basep = atomicAdd(&b.stats->pairs, (unsigned long long)tot);
      basep = __shfl_sync(FULL, basep, 31);
      uint64_t pos = basep + inc - cnt;
      while (mask) {
        const int d = __ffs(mask) - 1;
        mask &= mask - 1u;
        const int r = ztop - d;
        if (pos < cap) {
          b.keys[pos] = (uint32_t)(((uint64_t)q * nx + p) * nz + r);
          b.vals[pos] = tglob | (first ? 0x80000000u : 0u);
        } else {
          atomicOr(&b.stats->status, (unsigned)ST_PAIR_OVERFLOW);
        }
        first = false;
        ++pos;
        atomicOr(&b.bplane[((size_t)r * ny + q) * g.nxw + (p >> 5)], 1u << (p & 31));
      }
    }
  }

  // ---- (b) fill units
  for (uint32_t base = warp * 32u; base < Uf; base += kL1Warps * 32u) {
    const uint32_t u = base + lane;
    bool pass = false;
    if (u < Uf) {
      const int lt = tile_search(s_foff, nt, u);
      const float4 a0 = s_tri[3 * lt], a1 = s_tri[3 * lt + 1], a2 = s_tri[3 * lt + 2];
      const uint32_t fxr = __float_as_uint(a0.w), fyr = __float_as_uint(a1.w);
      const uint32_t c = u - s_foff[lt];
      const int nxr = hi16(fxr) - lo16(fxr) + 1;
      const int i = lo16(fxr) + (int)(c % (uint32_t)nxr);
      const int j = lo16(fyr) + (int)(c / (uint32_t)nxr);
      const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
      RayTri rt;
      ray_tri_pre(V, a2.w, rt);  // fill units exist only for triangles passing the det test
      RayCol rc;
      pass = ray_col(rt, __ldg(g.c1[0] + i), __ldg(g.c1[1] + j), rc);
    }
    const unsigned qm = __ballot_sync(FULL, pass);
    if (pass) s_q[warp][__popc(qm & lt_mask)] = u;
    __syncwarp();
    const int nq = __popc(qm);
    for (int e = 0; e < nq; ++e) {
      const uint32_t uu = s_q[warp][e];
      const int lt = tile_search(s_foff, nt, uu);
      const float4 a0 = s_tri[3 * lt], a1 = s_tri[3 * lt + 1], a2 = s_tri[3 * lt + 2];
      const uint32_t fxr = __float_as_uint(a0.w), fyr = __float_as_uint(a1.w);
      const uint32_t c = uu - s_foff[lt];
      const int nxr = hi16(fxr) - lo16(fxr) + 1;
      const int i = lo16(fxr) + (int)(c % (uint32_t)nxr);
      const int j = lo16(fyr) + (int)(c / (uint32_t)nxr);
      const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
      RayTri rt;
      ray_tri_pre(V, a2.w, rt);
      RayCol rc;
      ray_col(rt, __ldg(g.c1[0] + i), __ldg(g.c1[1] + j), rc);
      const size_t col = (size_t)j * nx + i;
      uint32_t carry = 0;
      for (int w = g.nzw - 1; w >= 0; --w) {
        const int k = w * 32 + (int)lane;
        const bool hit = k < nz && ray_t(rt, rc, __ldg(g.c1[2] + k), g.thr);
        const uint32_t h = __ballot_sync(FULL, hit);
        const uint32_t d = h ^ ((h >> 1) | (carry << 31));
        carry = h & 1u;
        if (lane == 0 && d) atomicXor(&b.toggles[col * g.nzw + w], d);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// One warp per (row j, 32-column group): suffix XOR of each column's toggles gives the parity
// of every voxel; 32 ballots per word transpose it into the linear inside plane.
__global__ void __launch_bounds__(256) k_fill_finish(GridDev g, Level1Bufs b) {
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned lane = threadIdx.x & 31u;
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  if (gw >= (int64_t)ny * g.nxw) return;
  const int j = (int)(gw / g.nxw), ig = (int)(gw % g.nxw);
  const int i = ig * 32 + (int)lane;
  const bool valid = i < nx;
  const size_t col = (size_t)j * nx + i;
  uint32_t carry = 0;
  for (int w = g.nzw - 1; w >= 0; --w) {
    const uint32_t D = valid ? b.toggles[col * g.nzw + w] : 0u;
    uint32_t s = D;
    s ^= s >> 1; s ^= s >> 2; s ^= s >> 4; s ^= s >> 8; s ^= s >> 16;
    if (carry) s = ~s;
    carry ^= (uint32_t)(__popc(D) & 1);
    uint32_t mine = 0;
#pragma unroll
    for (int bb = 0; bb < 32; ++bb) {
      const uint32_t m = __ballot_sync(FULL, (s >> bb) & 1u);
      if ((int)lane == bb) mine = m;
    }
    const int k = w * 32 + (int)lane;
    if (k < nz) b.iplane[((size_t)k * ny + j) * g.nxw + ig] = mine;
  }
}

__global__ void k_popc(const uint32_t *__restrict__ plane, int64_t nw, uint32_t *__restrict__ cnt) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) cnt[w] = __popc(plane[w]);
}

// One block per Level1 row (k, j): state bytes, boundaryPrefixSum, boundaryIndex.
__global__ void __launch_bounds__(128) k_expand(GridDev g, const uint32_t *__restrict__ bplane,
                                                const uint32_t *__restrict__ iplane,
                                                const uint32_t *__restrict__ wpre,
                                                uint8_t *__restrict__ l1, int32_t *__restrict__ prefix,
                                                int32_t *__restrict__ bindex, MeshStats *st) {
  const int64_t row = blockIdx.x;
  const int nx = g.n[0];
  const bool vec = (nx & 3) == 0;
  unsigned long long nin = 0;
  for (int x4 = threadIdx.x * 4; x4 < nx; x4 += blockDim.x * 4) {
    uint32_t bytes = 0;
    int32_t pre[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int x = x4 + e;
      pre[e] = 0;
      if (x >= nx) break;
      const size_t w = (size_t)row * g.nxw + (x >> 5);
      const int bit = x & 31;
      const uint32_t bw = bplane[w], iw = iplane[w];
      const uint32_t p = wpre[w] + __popc(bw & ((1u << bit) - 1u));
      const bool isb = (bw >> bit) & 1u, isi = (iw >> bit) & 1u;
      const uint32_t s = isb ? 254u : (isi ? 127u : 0u);
      nin += (!isb && isi);
      pre[e] = (int32_t)p;
      const int64_t v = row * nx + x;
      if (isb) bindex[p] = (int32_t)v;
      if (!vec) {
        l1[v] = (uint8_t)s;
        prefix[v] = (int32_t)p;
      }
      bytes |= s << (8 * e);
    }
    if (vec) {
      const int64_t v = row * nx + x4;
      *reinterpret_cast<uint32_t *>(l1 + v) = bytes;
      *reinterpret_cast<int4 *>(prefix + v) = make_int4(pre[0], pre[1], pre[2], pre[3]);
    }
  }
  nin = warp_sum(nin);
  if ((threadIdx.x & 31u) == 0 && nin) atomicAdd(&st->l1_inside, nin);
}

__global__ void k_heads(const uint32_t *__restrict__ keys, int64_t P, uint32_t *__restrict__ flags) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < P) flags[e] = (e == 0 || keys[e] != keys[e - 1]) ? 1u : 0u;
}

__global__ void k_useg(const uint32_t *__restrict__ flags, const uint32_t *__restrict__ uidx,
                       int64_t P, uint32_t *__restrict__ useg) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < P && flags[e]) useg[uidx[e]] = (uint32_t)e;
  if (e == P - 1) useg[uidx[e] + flags[e]] = (uint32_t)P;
}

}  // namespace

// ---- launchers --------------------------------------------------------------------------------
void launch_prep(const GridDev &g, const Level1Bufs &b, cudaStream_t s) {
  if (b.T <= 0) return;
  const unsigned nb = (unsigned)((b.T + 255) / 256);
  k_prep<<<nb, 256, 0, s>>>(g, b);
  count_launch();
}

void launch_level1(const GridDev &g, const Level1Bufs &b, int tile, cudaStream_t s) {
  if (b.T <= 0) return;
  const unsigned nb = (unsigned)((b.T + tile - 1) / tile);
  switch (tile) {
    case 32: k_level1<32><<<nb, kL1Threads, 0, s>>>(g, b); count_launch(); break;
    case 64: k_level1<64><<<nb, kL1Threads, 0, s>>>(g, b); count_launch(); break;
    case 128: k_level1<128><<<nb, kL1Threads, 0, s>>>(g, b); count_launch(); break;
    default: k_level1<256><<<(unsigned)((b.T + 255) / 256), kL1Threads, 0, s>>>(g, b); count_launch(); break;
  }
}

void launch_fill_finish(const GridDev &g, const Level1Bufs &b, cudaStream_t s) {
  const int64_t warps = (int64_t)g.n[1] * g.nxw;
  const unsigned nb = (unsigned)((warps * 32 + 255) / 256);
  k_fill_finish<<<nb, 256, 0, s>>>(g, b);
  count_launch();
}

void launch_popc(const GridDev &g, const uint32_t *bplane, uint32_t *cnt, cudaStream_t s) {
  const int64_t nw = (int64_t)g.n[2] * g.n[1] * g.nxw;
  k_popc<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(bplane, nw, cnt);
  count_launch();
}

void launch_expand(const GridDev &g, const uint32_t *bplane, const uint32_t *iplane,
                   const uint32_t *wpre, uint8_t *l1, int32_t *prefix, int32_t *bindex,
                   MeshStats *st, cudaStream_t s) {
  const unsigned rows = (unsigned)((int64_t)g.n[2] * g.n[1]);
  k_expand<<<rows, 128, 0, s>>>(g, bplane, iplane, wpre, l1, prefix, bindex, st);
  count_launch();
}

void launch_heads(const uint32_t *keys, int64_t P, uint32_t *flags, cudaStream_t s) {
  if (P <= 0) return;
  k_heads<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(keys, P, flags);
  count_launch();
}

void launch_useg(const uint32_t *flags, const uint32_t *uidx, int64_t P, uint32_t *useg,
                 cudaStream_t s) {
  if (P <= 0) return;
  k_useg<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(flags, uidx, P, useg);
  count_launch();
}

}  // namespace gpv
