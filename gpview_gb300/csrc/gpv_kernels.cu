// gpv_kernels.cu -- sm_103a kernels of the Level1 stage, batched over meshes.
//
// Pipeline (all on one stream; a plain voxelization is a batch of one):
//   k_prep        per triangle: pack vertices as 3 float4, Level1 SAT candidate box (the
//                 reference's own range, src/Object.cpp:2280-2325), conservative x/y box for the
//                 ray tests, 1/det of the ray test, work counts.
//   k_level1      persistent: blocks pull (mesh, triangle tile) items from a device queue; the
//                 tile is staged in shared memory by bulk async copies (TMA) on an mbarrier.
//                 (a) SAT units = (triangle, column) running the z run top-down; passes set the
//                     boundary bit (atomicOr) and emit (column-major voxel key, triangle|topmost).
//                 (b) fill units = (triangle, column) running the column part of the +z
//                     Moller-Trumbore test; passing pairs are queued per warp and the whole warp
//                     evaluates t over the column (one voxel per lane, __ballot_sync), XOR-ing
//                     parity toggles d(k) = hit(k) ^ hit(k+1) into a column-major plane.
//   k_fill_finish warp-level suffix XOR of the toggles per column -> parity, transposed to
//                 the linear (x fastest) inside plane.
//   k_popc + scan per-word boundary counts, boundaryPrefixSum.
//   k_expand      .raw bytes of Level1, boundaryPrefixSum, boundaryIndex.
//   sort / Level2 gpv_sort.cu, gpv_level2.cu.
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

// Adds v to *dst once per warp when every lane targets the same counter, else per lane.
__device__ __forceinline__ void warp_add(unsigned long long *dst, unsigned long long v) {
  const unsigned long long a = (unsigned long long)dst;
  if (__all_sync(FULL, __shfl_sync(FULL, a, 0) == a)) {
    v = warp_sum(v);
    if ((threadIdx.x & 31u) == 0 && v) atomicAdd(dst, v);
  } else if (v) {
    atomicAdd(dst, v);
  }
}

// The four prep counters of a 256-thread block: one atomic each per block when every thread of
// the block works on the same mesh (the common case), else per warp.  Thousands of per-warp
// atomics on one counter serialise at L2.
__device__ __forceinline__ void block_add_prep(MeshStats *st, unsigned long long a,
                                               unsigned long long b, unsigned long long c,
                                               unsigned long long d, unsigned long long e) {
  __shared__ unsigned long long s_acc[5][8];
  __shared__ MeshStats *s_first;
  if (threadIdx.x == 0) s_first = st;
  __syncthreads();
  if (__syncthreads_and(st == s_first)) {
    a = warp_sum(a); b = warp_sum(b); c = warp_sum(c); d = warp_sum(d); e = warp_sum(e);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0) {
      s_acc[0][warp] = a; s_acc[1][warp] = b; s_acc[2][warp] = c; s_acc[3][warp] = d;
      s_acc[4][warp] = e;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
      unsigned long long v = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) v += s_acc[threadIdx.x][w];
      unsigned long long *dst = threadIdx.x == 0 ? &st->sat1 : threadIdx.x == 1 ? &st->sat_units
                                : threadIdx.x == 2 ? &st->fill_units : threadIdx.x == 3 ? &st->ray1
                                : &st->xycells;
      if (v) atomicAdd(dst, v);
    }
  } else {
    warp_add(&st->sat1, a);
    warp_add(&st->sat_units, b);
    warp_add(&st->fill_units, c);
    warp_add(&st->ray1, d);
    warp_add(&st->xycells, e);
  }
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
__global__ void __launch_bounds__(256) k_prep(BatchDev bd) {
  const int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = gi < bd.total_tris;
  const int m = find_mesh<&MeshDesc::tri_base>(bd.md, bd.nmesh, live ? gi : bd.total_tris - 1);
  const MeshDesc &d = bd.md[m];
  const GridDev &g = d.g;
  unsigned long long sat1 = 0, su = 0, fu = 0, r1 = 0, xy = 0;
  if (live) {
    const int64_t t = gi - d.tri_base;
    float V[9];
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      V[k] = __ldg(d.tris + 9 * t + k);
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
      atomicOr(&d.stats->status, (unsigned)ST_BAD_INPUT);
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
      if (g.n2[0] > 0) {  // x/y extent in Level2 cells (the density of the Level2 SAT items)
        const float ex = fminf((mxx - mnx) * g.inv_g2[0], 1e6f), ey = fminf((mxy - mny) * g.inv_g2[1], 1e6f);
        xy = (unsigned long long)((ex + 1.f) * (ey + 1.f) * 16.f);
      }
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
    if (bd.fill != GPV_FILL_RAY) {  // the stencil kernel fills instead (or nothing fills)
      fx0 = 1; fx1 = 0; fy0 = 1; fy1 = 0;
      fu = 0;
      r1 = 0;
    }
    // 1/det of the +z ray test (src/TriRayIntersection.cpp:99), shared by every column
    const float det = fa(fm(fs(V[3], V[0]), -fs(V[7], V[1])), fm(fs(V[4], V[1]), fs(V[6], V[0])));
    d.ptri[3 * t + 0] = make_float4(V[0], V[1], V[2], __uint_as_float(pack2(fx0, fx1)));
    d.ptri[3 * t + 1] = make_float4(V[3], V[4], V[5], __uint_as_float(pack2(fy0, fy1)));
    d.ptri[3 * t + 2] = make_float4(V[6], V[7], V[8], __fdiv_rn(1.0f, det));
    d.rng[t] = make_int4((int)pack2(lo[0], hi[0]), (int)pack2(lo[1], hi[1]),
                         (int)pack2(lo[2], hi[2]), 0);
    d.fbox[t] = fb;
  }
  block_add_prep(d.stats, sat1, su, fu, r1, xy);
}

// Per-mesh pair emission segments from the candidate counts prep just produced: exclusive prefix
// of sat1 over the meshes, capped by the buffer capacity (a mesh past the end gets a short or
// empty segment; its Level1 then raises ST_PAIR_OVERFLOW).  One block; meshes in rounds of 1024.
__global__ void __launch_bounds__(1024) k_pair_bases(int nmesh, MeshDesc *md, uint32_t *keys,
                                                     uint32_t *vals, int64_t cap) {
  __shared__ unsigned long long s_w[32];
  __shared__ unsigned long long s_carry;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int m0 = 0; m0 < nmesh; m0 += 1024) {
    const int m = m0 + (int)threadIdx.x;
    const unsigned long long v = m < nmesh ? md[m].stats->sat1 : 0ull;
    unsigned long long x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long o = __shfl_up_sync(FULL, x, d);
      if (lane >= (unsigned)d) x += o;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned long long w = s_w[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long o = __shfl_up_sync(FULL, w, d);
        if (lane >= (unsigned)d) w += o;
      }
      s_w[lane] = w;
    }
    __syncthreads();
    const unsigned long long base = s_carry + (warp ? s_w[warp - 1] : 0ull) + x - v;
    if (m < nmesh) {
      const int64_t b = (int64_t)base;
      md[m].emit_base = b;
      md[m].pair_cap = max((int64_t)0, min((int64_t)v, cap - b));
      md[m].keys = keys + min(b, cap);
      md[m].vals = vals + min(b, cap);
    }
    __syncthreads();
    if (threadIdx.x == 1023) s_carry = base + v;
    __syncthreads();
  }
}

// One-graph calls: the second half's per-mesh bases and sizes from the first half's counts (one
// block; meshes in rounds of 1024, seven running sums scanned together).  The sums, per mesh:
// 0 boundary voxels (boundaryIndex slices), 1 the same for meshes with a Level2 grid (sorted
// segments), 2 their Level2 bytes, 3 their pair-sort tiles, 4 their pairs, 5 the pairs of those
// whose pairs carry many Level2 SAT items (the queued organisation's measure, as
// level2_queue_pays computes it on the host), 6 meshes with a raised status.
constexpr int kPlanSums = 7;
__global__ void __launch_bounds__(1024) k_plan(int nmesh, MeshDesc *md, int32_t *bindex,
                                               uint8_t *l2, PlanCaps caps, int mode,
                                               DevPlan *plan) {
  __shared__ unsigned long long s_w[32][kPlanSums];
  __shared__ unsigned long long s_carry[kPlanSums];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (threadIdx.x < kPlanSums) s_carry[threadIdx.x] = 0;
  __syncthreads();
  for (int m0 = 0; m0 < nmesh; m0 += 1024) {
    const int m = m0 + (int)threadIdx.x;
    unsigned long long v[kPlanSums] = {};
    if (m < nmesh) {
      const MeshStats &st = *md[m].stats;
      const bool has = md[m].has_l2 != 0;
      const unsigned long long b = st.boundary, p = st.pairs;
      const unsigned long long cells =
          (unsigned long long)md[m].g.n2[0] * md[m].g.n2[1] * md[m].g.n2[2];
      v[0] = b;
      v[1] = has ? b : 0ull;
      v[2] = has ? b * cells : 0ull;
      v[3] = has ? (p + kSortTileItems - 1) / kSortTileItems : 0ull;
      v[4] = has ? p : 0ull;
      v[5] = (has && st.xycells >= 64ull * p) ? p : 0ull;
      v[6] = st.status != 0u;
    }
    unsigned long long x[kPlanSums];
#pragma unroll
    for (int k = 0; k < kPlanSums; ++k) {
      x[k] = v[k];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long o = __shfl_up_sync(FULL, x[k], d);
        if (lane >= (unsigned)d) x[k] += o;
      }
      if (lane == 31) s_w[warp][k] = x[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
      for (int k = 0; k < kPlanSums; ++k) {
        unsigned long long w = s_w[lane][k];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const unsigned long long o = __shfl_up_sync(FULL, w, d);
          if (lane >= (unsigned)d) w += o;
        }
        s_w[lane][k] = w;
      }
    }
    __syncthreads();
    if (m < nmesh) {
      unsigned long long e[kPlanSums];
#pragma unroll
      for (int k = 0; k < kPlanSums; ++k)
        e[k] = s_carry[k] + (warp ? s_w[warp - 1][k] : 0ull) + x[k] - v[k];
      md[m].u_base = (int64_t)e[1];
      md[m].pair_base = (int64_t)e[4];
      md[m].stile_base = (int64_t)e[3];
      md[m].bindex = bindex + min((long long)e[0], (long long)caps.B);
      md[m].l2 = l2 + min((long long)e[2], (long long)caps.l2bytes);
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < kPlanSums; ++k) s_carry[k] += s_w[31][k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const unsigned long long *t = s_carry;
    DevPlan p;
    p.ok = t[6] == 0 && t[0] <= (unsigned long long)caps.B && t[1] <= (unsigned long long)caps.U &&
           t[2] <= (unsigned long long)caps.l2bytes && t[3] <= (unsigned long long)caps.tiles &&
           t[4] <= (unsigned long long)caps.P;
    p.qsel = mode == GPV_LEVEL2_QUEUED   ? 1u
             : mode == GPV_LEVEL2_INLINE ? 0u
                                         : ((double)t[5] > 0.9 * (double)t[4] ? 1u : 0u);
    p.ub = (uint32_t)min(t[1], 0xffffffffull);
    p.ntiles = (uint32_t)min(t[3], 0xffffffffull);
    p.P2 = t[4];
    p.Btot = t[0];
    p.l2bytes = t[2];
    *plan = p;
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
__global__ void __launch_bounds__(kL1Threads) k_level1(BatchDev bd) {
  __shared__ __align__(16) float4 s_tri[TILE * 3];
  __shared__ __align__(16) int4 s_rng[TILE];
  __shared__ uint32_t s_soff[TILE + 1];
  __shared__ uint32_t s_foff[TILE + 1];
  __shared__ uint32_t s_q[kL1Warps][32];
  __shared__ uint32_t s_ws[kL1Warps], s_wf[kL1Warps];
  __shared__ uint32_t s_next;  // next 32-unit chunk of the tile (SAT chunks, then fill chunks)
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int64_t s_item;

  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    fence_mbar_init();
  }
  __syncthreads();

  for (uint32_t iter = 0;; ++iter) {
    // ---- pull the next (mesh, tile) item from the queue
    if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(&bd.queue[0], 1u);
    __syncthreads();
    const int64_t item = s_item;
    if (item >= bd.total_tiles) break;
    const int m = find_mesh<&MeshDesc::tile_base>(bd.md, bd.nmesh, item);
    const MeshDesc &d = bd.md[m];
    const GridDev &g = d.g;
    const int64_t t0 = (item - d.tile_base) * TILE;
    uint32_t *const kmask = bd.kmask && d.has_l2 ? bd.kmask + d.word_base : nullptr;
    const int nt = (int)min((int64_t)TILE, d.T - t0);

    // ---- stage the tile with bulk async copies completing on the mbarrier
    if (threadIdx.x == 0) {
      const uint32_t bt = (uint32_t)nt * 48u, br = (uint32_t)nt * 16u;
      mbar_expect_tx(&s_bar, bt + br);
      bulk_g2s(s_tri, d.ptri + 3 * t0, bt, &s_bar);
      bulk_g2s(s_rng, d.rng + t0, br, &s_bar);
    }
    // bounded wait (bd.wait_limit polls, kWaitLimit when 0); bd.fail_wait makes it give up at
    // once (failure-detection tests).  On giving up, the status word is raised and thread 0
    // waits, bounded again, for the copies in flight to land before the block returns.
    const bool ok = !bd.fail_wait &&
                    mbar_wait_bounded(&s_bar, iter & 1u, bd.wait_limit ? bd.wait_limit : kWaitLimit);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(&d.stats->status, (unsigned)ST_WAIT_TIMEOUT);
        mbar_wait_bounded(&s_bar, iter & 1u, kWaitLimit);  // let the copy in flight land
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
      if (threadIdx.x == 0) s_next = 0;
      __syncthreads();
    }
    const uint32_t Us = s_soff[TILE], Uf = s_foff[TILE];
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const uint64_t cap = (uint64_t)d.pair_cap;

    // Warps take 32-unit chunks from a counter, the SAT chunks first and then the fill chunks,
    // so that a warp whose z runs or hits were short takes more chunks instead of waiting at the
    // tile's closing barrier for the others.
    const uint32_t nsc = (Us + 31u) >> 5;
    auto next_chunk = [&]() {
      uint32_t c = 0;
      if (lane == 0) c = atomicAdd(&s_next, 1u);
      return __shfl_sync(FULL, c, 0);
    };
    uint32_t chunk = next_chunk();
    // ---- (a) SAT units
    for (; chunk < nsc; chunk = next_chunk()) {
      const uint32_t base = chunk * 32u;
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
          for (int dd = 0; dd < nrun; ++dd)
            if (sat_z(sc, V, __ldg(g.c1[2] + (ztop - dd)), g.e1)) mask |= 1u << dd;
          zc -= nrun;
        }
        const uint32_t cnt = __popc(mask);
        const uint32_t inc = warp_incl_scan(cnt);
        const uint32_t tot = __shfl_sync(FULL, inc, 31);
        unsigned long long basep = 0;
        if (lane == 31 && tot) basep = atomicAdd(&d.stats->pairs, (unsigned long long)tot);
        basep = __shfl_sync(FULL, basep, 31);
        uint64_t pos = basep + inc - cnt;
        while (mask) {
          const int dd = __ffs(mask) - 1;
          mask &= mask - 1u;
          const int r = ztop - dd;
          const uint32_t key = (uint32_t)(((uint64_t)q * nx + p) * nz + r);
          if (pos < cap) {
            d.keys[pos] = key;
            d.vals[pos] = tglob | (first ? 0x80000000u : 0u);
          } else {
            atomicOr(&d.stats->status, (unsigned)ST_PAIR_OVERFLOW);
          }
          if (kmask) atomicOr(kmask + (key >> 5), 1u << (key & 31u));
          first = false;
          ++pos;
          atomicOr(&d.bplane[((size_t)r * ny + q) * g.nxw + (p >> 5)], 1u << (p & 31));
        }
      }
    }

    // ---- (b) fill units
    for (; (chunk - nsc) * 32u < Uf; chunk = next_chunk()) {
      const uint32_t base = (chunk - nsc) * 32u;
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
          const uint32_t dd = h ^ ((h >> 1) | (carry << 31));
          carry = h & 1u;
          if (lane == 0 && dd) atomicXor(&d.toggles[col * g.nzw + w], dd);
        }
      }
      __syncwarp();
    }
    __syncthreads();  // the next item overwrites the tile
  }
}

// ---------------------------------------------------------------------------------------------
// One warp per (mesh, row j, 32-column group, 32-layer word w): suffix XOR of each column's
// toggles gives the parity of every voxel (the toggles of the words above w give the carry); 32
// ballots transpose the word into the linear inside plane.
// Stencil fill: the parity of each of the voxel column's four sample columns is the prefix XOR
// of its slice toggles (lowest slice first), and a voxel is inside where at least three of the
// four are odd.
__global__ void __launch_bounds__(256) k_fill_finish(BatchDev bd) {
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned lane = threadIdx.x & 31u;
  if (gw >= bd.total_fwarps) return;
  const int m = find_mesh<&MeshDesc::fwarp_base>(bd.md, bd.nmesh, gw);
  const MeshDesc &d = bd.md[m];
  const GridDev &g = d.g;
  const int64_t lw = gw - d.fwarp_base;
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const int w = (int)(lw % g.nzw);
  const int64_t cgrp = lw / g.nzw;
  const int j = (int)(cgrp / g.nxw), ig = (int)(cgrp % g.nxw);
  const int i = ig * 32 + (int)lane;
  const bool valid = i < nx;
  const size_t col = (size_t)j * nx + i;
  const bool stencil = bd.fill == GPV_FILL_STENCIL;
  const uint32_t *sc[4] = {nullptr, nullptr, nullptr, nullptr};
  uint32_t s;
  if (stencil) {
    // bit a: toggle parity of sample column a in all words / in the words above w
    uint32_t tot = 0, above = 0;
    if (valid) {
      const size_t SW = 2 * (size_t)nx;
      sc[0] = d.stg + ((size_t)(2 * j) * SW + 2 * (size_t)i) * g.nzw;
      sc[1] = sc[0] + g.nzw;
      sc[2] = sc[0] + SW * g.nzw;
      sc[3] = sc[2] + g.nzw;
      for (int v = 0; v < g.nzw; ++v)
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const uint32_t pv = (uint32_t)(__popc(sc[a][v]) & 1) << a;
          tot ^= pv;
          if (v > w) above ^= pv;
        }
    }
    uint32_t x[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const uint32_t D = valid ? sc[a][w] : 0u;
      const uint32_t pd = (uint32_t)(__popc(D) & 1);
      uint32_t y = D;  // prefix XOR from the lowest slice of the word
      y ^= y << 1; y ^= y << 2; y ^= y << 4; y ^= y << 8; y ^= y << 16;
      if ((((tot ^ above) >> a) & 1u) ^ pd) y = ~y;  // odd toggles in the words below
      x[a] = y;
    }
    s = (x[0] & x[1] & (x[2] | x[3])) | (x[2] & x[3] & (x[0] | x[1]));
  } else {
    uint32_t carry = 0;  // toggle parity of the column in the words above w
    if (valid)
      for (int v = w + 1; v < g.nzw; ++v) carry ^= (uint32_t)(__popc(d.toggles[col * g.nzw + v]) & 1);
    const uint32_t D = valid ? d.toggles[col * g.nzw + w] : 0u;
    s = D;
    s ^= s >> 1; s ^= s >> 2; s ^= s >> 4; s ^= s >> 8; s ^= s >> 16;
    if (carry) s = ~s;
  }
  uint32_t mine = 0;
#pragma unroll
  for (int bb = 0; bb < 32; ++bb) {
    const uint32_t mm = __ballot_sync(FULL, (s >> bb) & 1u);
    if ((int)lane == bb) mine = mm;
  }
  const int k = w * 32 + (int)lane;
  if (k < nz) d.iplane[((size_t)k * ny + j) * g.nxw + ig] = mine;
}

__global__ void k_popc(const uint32_t *__restrict__ plane, int64_t nw, uint32_t *__restrict__ cnt) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) cnt[w] = __popc(plane[w]);
}

// B_m = boundary voxels of mesh m, from the exclusive scan over the batch's plane words.
__global__ void k_boundary_counts(BatchDev bd, const uint32_t *__restrict__ wpre,
                                  const uint32_t *__restrict__ wtotal) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= bd.nmesh) return;
  const uint32_t s = wpre[bd.md[m].word_base];
  const uint32_t e = m + 1 < bd.nmesh ? wpre[bd.md[m + 1].word_base] : *wtotal;
  bd.md[m].stats->boundary = e - s;
}

// One warp per chunk of 128 consecutive voxels of one mesh's linear index (x fastest),
// kExpandWarps chunks per block: state bytes, boundaryPrefixSum, boundaryIndex.  Every lane of a
// chunk works whatever the row length (a warp per row left three quarters of the lanes idle on a
// 32-voxel row), and a block whose chunks lie in one mesh looks the mesh up once.
constexpr int kExpandWarps = 8;
constexpr int kExpandVox = 128;
// One chunk by one warp; returns the lane's inside-voxel count and the chunk's mesh statistics.
__device__ __forceinline__ unsigned long long expand_chunk(const BatchDev &bd,
                                                           const uint32_t *__restrict__ wpre, int m,
                                                           int64_t gc, unsigned lane,
                                                           MeshStats *&st) {
  const MeshDesc &d = bd.md[m];
  const GridDev &g = d.g;
  st = d.stats;
  const int nx = g.n[0];
  const int64_t N1 = (int64_t)nx * g.n[1] * g.n[2];
  const int64_t v0 = (gc - d.xc_base) * kExpandVox + (int64_t)lane * 4;
  if (v0 >= N1) return 0;
  const uint32_t pbase = wpre[d.word_base];
  const uint32_t *bplane = d.bplane, *iplane = d.iplane;
  const uint32_t *wp = wpre + d.word_base;
  unsigned long long nin = 0;
  // (the 4- and 16-byte stores need aligned outputs: the batch's arenas are, a no-alloc caller's
  // buffers may not be)
  if ((nx & 3) == 0 && (reinterpret_cast<uintptr_t>(d.l1) & 3u) == 0 &&
      (reinterpret_cast<uintptr_t>(d.prefix) & 15u) == 0) {
    // the lane's four voxels share a row and a plane word (nx and v0 are multiples of 4), and
    // N1 is a multiple of 4 too
    const int64_t row = v0 / nx;
    const int x0 = (int)(v0 - row * nx);
    const size_t w = (size_t)row * g.nxw + (x0 >> 5);
    const int b0 = x0 & 31;
    const uint32_t bw = bplane[w], iw = iplane[w];
    uint32_t p = wp[w] - pbase + __popc(bw & ((1u << b0) - 1u));
    uint32_t bytes = 0;
    int32_t pre[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool isb = (bw >> (b0 + e)) & 1u, isi = (iw >> (b0 + e)) & 1u;
      pre[e] = (int32_t)p;
      if (isb) {
        d.bindex[p] = (int32_t)(v0 + e);
        ++p;
      }
      nin += (!isb && isi);
      bytes |= (isb ? 254u : (isi ? 127u : 0u)) << (8 * e);
    }
    *reinterpret_cast<uint32_t *>(d.l1 + v0) = bytes;
    *reinterpret_cast<int4 *>(d.prefix + v0) = make_int4(pre[0], pre[1], pre[2], pre[3]);
  } else {
    for (int e = 0; e < 4; ++e) {
      const int64_t v = v0 + e;
      if (v >= N1) break;
      const int64_t row = v / nx;
      const int x = (int)(v - row * nx);
      const size_t w = (size_t)row * g.nxw + (x >> 5);
      const int bit = x & 31;
      const uint32_t bw = bplane[w], iw = iplane[w];
      const uint32_t p = wp[w] - pbase + __popc(bw & ((1u << bit) - 1u));
      const bool isb = (bw >> bit) & 1u, isi = (iw >> bit) & 1u;
      nin += (!isb && isi);
      if (isb) d.bindex[p] = (int32_t)v;
      d.l1[v] = (uint8_t)(isb ? 254u : (isi ? 127u : 0u));
      d.prefix[v] = (int32_t)p;
    }
  }
  return nin;
}

// A block takes `iters` x kExpandWarps consecutive chunks; warp w the chunks c0 + w + k x
// kExpandWarps.  Thread 0 looks up the mesh of the block's first chunk once (a binary search over
// the descriptors), and each warp walks forward from it as its chunks pass mesh boundaries, so
// the search is not repeated per chunk.  A warp adds its inside count to the statistics when it
// leaves a mesh; the block adds the warps' last runs with one atomic per mesh.
__global__ void __launch_bounds__(kExpandWarps * 32) k_expand(BatchDev bd,
                                                            const uint32_t *__restrict__ wpre,
                                                            int iters) {
  __shared__ int s_mesh;
  __shared__ int s_m[kExpandWarps];
  __shared__ unsigned long long s_nin[kExpandWarps];
  // one-graph calls whose sizes did not fit: the call is re-run
  if (bd.plan && !bd.plan->ok) return;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const int64_t c0 = (int64_t)blockIdx.x * kExpandWarps * iters;
  if (threadIdx.x == 0) s_mesh = find_mesh<&MeshDesc::xc_base>(bd.md, bd.nmesh, c0);
  __syncthreads();
  int m = s_mesh;
  unsigned long long nin = 0;
  for (int k = 0; k < iters; ++k) {
    const int64_t gc = c0 + (int64_t)k * kExpandWarps + warp;
    if (gc >= bd.total_xchunks) break;  // warp-uniform
    int mn = m;
    while (mn + 1 < bd.nmesh && bd.md[mn + 1].xc_base <= gc) ++mn;
    if (mn != m) {
      const unsigned long long t = warp_sum(nin);
      if (lane == 0 && t) atomicAdd(&bd.md[m].stats->l1_inside, t);
      nin = 0;
      m = mn;
    }
    MeshStats *st = nullptr;
    nin += expand_chunk(bd, wpre, m, gc, lane, st);
  }
  // the warps' last mesh runs: one atomic per mesh of the block
  const unsigned long long t = warp_sum(nin);
  if (lane == 0) {
    s_m[warp] = m;
    s_nin[warp] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int cur = s_m[0];
    unsigned long long acc = 0;
    for (int w = 0; w < kExpandWarps; ++w) {
      if (s_m[w] != cur) {
        if (acc) atomicAdd(&bd.md[cur].stats->l1_inside, acc);
        cur = s_m[w];
        acc = 0;
      }
      acc += s_nin[w];
    }
    if (acc) atomicAdd(&bd.md[cur].stats->l1_inside, acc);
  }
}

__global__ void k_heads(const uint32_t *__restrict__ keys, int64_t P, uint32_t *__restrict__ flags) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < P) flags[e] = (e == 0 || keys[e] != keys[e - 1]) ? 1u : 0u;
}

// Every mesh's first pair starts a segment even when its key equals the previous mesh's last.
__global__ void k_mesh_pair_heads(BatchDev bd, int64_t P, uint32_t *__restrict__ flags) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= bd.nmesh) return;
  const int64_t b = bd.md[m].pair_base;
  const int64_t e = m + 1 < bd.nmesh ? bd.md[m + 1].pair_base : P;
  if (e > b) flags[b] = 1u;
}

__global__ void k_useg(const uint32_t *__restrict__ flags, const uint32_t *__restrict__ uidx,
                       int64_t P, uint32_t *__restrict__ useg) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < P && flags[e]) useg[uidx[e]] = (uint32_t)e;
  if (e == P - 1) useg[uidx[e] + flags[e]] = (uint32_t)P;
}

// Copies and clears of StageOps (see StageList): 16-byte accesses where both addresses allow,
// 4-byte ones otherwise.  Sources are read with cache-volatile loads: page-locked host staging is
// rewritten by the host between launches.
__global__ void __launch_bounds__(256) k_stage(StageOps L) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int k = 0; k < L.n; ++k) {
    const uint32_t *src = L.op[k].src;
    uint32_t *dst = L.op[k].dst;
    const int64_t w = L.op[k].words;
    int64_t i0 = 0;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
      const int64_t w4 = w >> 2;
      uint4 *d4 = reinterpret_cast<uint4 *>(dst);
      const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
      if (src)
        for (int64_t i = t; i < w4; i += stride) d4[i] = __ldcv(s4 + i);
      else
        for (int64_t i = t; i < w4; i += stride) d4[i] = make_uint4(0u, 0u, 0u, 0u);
      i0 = w4 << 2;
    }
    if (src)
      for (int64_t i = i0 + t; i < w; i += stride) dst[i] = __ldcv(src + i);
    else
      for (int64_t i = i0 + t; i < w; i += stride) dst[i] = 0u;
  }
}

}  // namespace

// ---- launchers --------------------------------------------------------------------------------
void launch_prep(const BatchDev &bd, cudaStream_t s) {
  if (bd.total_tris <= 0) return;
  k_prep<<<(unsigned)((bd.total_tris + 255) / 256), 256, 0, s>>>(bd);
  count_launch();
}

// Boundary-voxel rank at the start of each z slab of one mesh (slab k = layers [k*zslab,
// (k+1)*zslab)): the exclusive word prefix at the slab's first word, the total past the end.
__global__ void k_slab_offsets(const uint32_t *__restrict__ wpre, const uint32_t *__restrict__ wtot,
                               int64_t words_per_layer, int nz, int zslab, int nslab,
                               uint32_t *__restrict__ out) {
  const int t = (int)threadIdx.x;
  if (t > nslab) return;
  const int z0 = min(t * zslab, nz);
  out[t] = z0 >= nz ? *wtot : wpre[(int64_t)z0 * words_per_layer];
}

void launch_slab_offsets(const uint32_t *wpre, const uint32_t *wtot, int64_t words_per_layer,
                         int nz, int zslab, int nslab, uint32_t *out, cudaStream_t s) {
  k_slab_offsets<<<1, 32, 0, s>>>(wpre, wtot, words_per_layer, nz, zslab, nslab, out);
  count_launch();
}

void StageList::add(void *dst, const void *src, size_t bytes) {
  if (bytes == 0) return;
  if (bytes & 3u) {
    if (src)
      cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s_);
    else
      cudaMemsetAsync(dst, 0, bytes, s_);
    return;
  }
  if (ops_.n == StageOps::kMax) launch();
  ops_.op[ops_.n++] = {static_cast<const uint32_t *>(src), static_cast<uint32_t *>(dst),
                       (int64_t)(bytes / 4)};
}

void StageList::launch() {
  if (ops_.n == 0) return;
  int64_t w = 0;
  for (int k = 0; k < ops_.n; ++k) w = std::max(w, ops_.op[k].words);
  const int64_t blocks = std::min<int64_t>((w / 4 + 255) / 256 + 1, 2 * (int64_t)sms_);
  k_stage<<<(unsigned)blocks, 256, 0, s_>>>(ops_);
  count_launch();
  ops_.n = 0;
}

void launch_pair_bases(const BatchDev &bd, MeshDesc *d_md, uint32_t *keys, uint32_t *vals,
                       int64_t cap, cudaStream_t s) {
  k_pair_bases<<<1, 1024, 0, s>>>(bd.nmesh, d_md, keys, vals, cap);
  count_launch();
}

void launch_plan(const BatchDev &bd, MeshDesc *d_md, int32_t *bindex, uint8_t *l2,
                 const PlanCaps &caps, int level2_mode, DevPlan *plan, cudaStream_t s) {
  k_plan<<<1, 1024, 0, s>>>(bd.nmesh, d_md, bindex, l2, caps, level2_mode, plan);
  count_launch();
}

void launch_level1(const BatchDev &bd, int num_sms, cudaStream_t s) {
  if (bd.total_tiles <= 0) return;
  const int64_t grid = std::min<int64_t>(bd.total_tiles, (int64_t)num_sms * 8);
  cudaMemsetAsync(bd.queue, 0, sizeof(uint32_t), s);
  switch (bd.tile) {
    case 32: k_level1<32><<<(unsigned)grid, kL1Threads, 0, s>>>(bd); break;
    case 64: k_level1<64><<<(unsigned)grid, kL1Threads, 0, s>>>(bd); break;
    case 128: k_level1<128><<<(unsigned)grid, kL1Threads, 0, s>>>(bd); break;
    default: k_level1<256><<<(unsigned)grid, kL1Threads, 0, s>>>(bd); break;
  }
  count_launch();
}

void launch_fill_finish(const BatchDev &bd, cudaStream_t s) {
  if (bd.total_fwarps <= 0) return;
  k_fill_finish<<<(unsigned)((bd.total_fwarps * 32 + 255) / 256), 256, 0, s>>>(bd);
  count_launch();
}

void launch_popc(const uint32_t *plane, int64_t nwords, uint32_t *cnt, cudaStream_t s) {
  if (nwords <= 0) return;
  k_popc<<<(unsigned)((nwords + 255) / 256), 256, 0, s>>>(plane, nwords, cnt);
  count_launch();
}

void launch_boundary_counts(const BatchDev &bd, const uint32_t *wpre, const uint32_t *wtotal,
                            cudaStream_t s) {
  k_boundary_counts<<<(unsigned)((bd.nmesh + 127) / 128), 128, 0, s>>>(bd, wpre, wtotal);
  count_launch();
}

void launch_expand(const BatchDev &bd, const uint32_t *wpre, cudaStream_t s) {
  if (bd.total_xchunks <= 0) return;
  // up to 8 chunks per warp where the chunks are many enough to give each of the 152 SMs 64
  // warps anyway
  const int64_t spread = bd.total_xchunks / (152 * 64);
  const int iters = (int)(spread < 1 ? 1 : spread > 8 ? 8 : spread);
  const int64_t per_block = (int64_t)kExpandWarps * iters;
  k_expand<<<(unsigned)((bd.total_xchunks + per_block - 1) / per_block), kExpandWarps * 32, 0, s>>>(
      bd, wpre, iters);
  count_launch();
}

void launch_heads(const uint32_t *keys, int64_t P, uint32_t *flags, const BatchDev &bd,
                  cudaStream_t s) {
  if (P <= 0) return;
  k_heads<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(keys, P, flags);
  k_mesh_pair_heads<<<(unsigned)((bd.nmesh + 127) / 128), 128, 0, s>>>(bd, P, flags);
  count_launch(2);
}

void launch_useg(const uint32_t *flags, const uint32_t *uidx, int64_t P, uint32_t *useg,
                 cudaStream_t s) {
  if (P <= 0) return;
  k_useg<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(flags, uidx, P, useg);
  count_launch();
}

}  // namespace gpv
