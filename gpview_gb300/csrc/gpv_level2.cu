// gpv_level2.cu -- Level2 refinement of the boundary voxels, organised per Level1 column.
//
// Reference semantics (src/Object.cpp:1111-1207 and :2344-2400): for boundary voxel b at
// (i,j,k), a Level2 cell is 2 if the SAT passes for any triangle recorded in b; otherwise 1 if
// the +z ray from the cell's origin crosses an odd number of distinct triangles among those
// recorded in voxels (i,j,z) with z >= k; otherwise 0.
//
// Work unit: a chunk of up to CH consecutive boundary voxels of one Level1 column (one warp).
//   SAT   -- (triangle, sub-column) items of each voxel, flattened over the 32 lanes; the cells
//            of a sub-column are tested only inside the plane slab that can pass the SAT's own
//            plane test (PlaneSlab), and one atomic per sub-column writes the z bits.
//   fill  -- the column's triangle entries flagged as topmost occurrences are the union sets
//            of all voxels of the chunk at once (voxel k sees the triangles whose topmost z is
//            >= k).  The u/v part of each ray test depends only on the sub-column, so it runs
//            once per (triangle, sub-column) for the whole chunk.  Voxels that lie certainly below
//            the triangle (t at their top origin exceeds 1e-6 by twice a float error bound) are
//            entirely hit: one "full hit" toggle marks the highest of them and a suffix XOR over
//            the chunk's voxels expands it.  In the remaining voxels t at each origin follows
//            from t at the top origin (exact t falls by the rise of the origin); only origins
//            within the error band of the crossing evaluate their own t.
#include "gpv_internal.h"

namespace gpv {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr float EPS24 = 5.9604644775390625e-08f;  // 2^-24
constexpr int kWarps = 4;
constexpr int kMaskWords = 512;  // words of one mask kind per warp (sets the chunk length)

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

// Slab of cell centres the triangle's plane test can accept.  For a cell centre c the SAT's
// plane test (planeBoxOverlap on the box-relative, rounded edges) can only pass when
//   |n_f . (V0 - c)| <= |n_f| . h + E,
// with n_f the float normal (V1-V0) x (V2-V1) and E a bound on the float deviations of both
// sides from exact arithmetic.  With R the largest |V_i,q - c_q| over the voxel's centres and
// h the largest half size, the deviations sum to less than 736 eps R^2 (h + R); E uses 1024.
struct PlaneSlab { float nx, ny, nz, H; };

__device__ __forceinline__ PlaneSlab plane_slab(const float *V, float cx0, float cx1, float cy0,
                                                float cy1, float cz0, float cz1, const float h[3]) {
  const float a0 = fs(V[3], V[0]), a1 = fs(V[4], V[1]), a2 = fs(V[5], V[2]);
  const float b0 = fs(V[6], V[3]), b1 = fs(V[7], V[4]), b2 = fs(V[8], V[5]);
  PlaneSlab ps;
  ps.nx = fs(fm(a1, b2), fm(a2, b1));
  ps.ny = fs(fm(a2, b0), fm(a0, b2));
  ps.nz = fs(fm(a0, b1), fm(a1, b0));
  const float lo[3] = {cx0 - h[0], cy0 - h[1], cz0 - h[2]};
  const float hi[3] = {cx1 + h[0], cy1 + h[1], cz1 + h[2]};
  float R = 0.f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const float vmn = fminf(V[q], fminf(V[3 + q], V[6 + q]));
    const float vmx = fmaxf(V[q], fmaxf(V[3 + q], V[6 + q]));
    R = fmaxf(R, fmaxf(fabsf(vmx - lo[q]), fabsf(hi[q] - vmn)));
  }
  R *= 1.0001f;
  const float hm = fmaxf(h[0], fmaxf(h[1], h[2]));
  const float E = 1024.f * EPS24 * R * R * (hm + R);
  ps.H = fabsf(ps.nx) * h[0] + fabsf(ps.ny) * h[1] + fabsf(ps.nz) * h[2] + E;
  return ps;
}

// Bits of one Level2 column (n2z cells along z) start at bit (q*n2x + p)*n2z of a voxel's mask.
__device__ __forceinline__ void or_column(uint32_t *m, int colidx, int n2z, uint32_t bits) {
  const int off = colidx * n2z, sh = off & 31;
  atomicOr(&m[off >> 5], bits << sh);
  if (sh + n2z > 32) atomicOr(&m[(off >> 5) + 1], bits >> (32 - sh));
}
__device__ __forceinline__ void xor_column(uint32_t *m, int colidx, int n2z, uint32_t bits) {
  const int off = colidx * n2z, sh = off & 31;
  atomicXor(&m[off >> 5], bits << sh);
  if (sh + n2z > 32) atomicXor(&m[(off >> 5) + 1], bits >> (32 - sh));
}

// t of the +z test for one origin height (same operations as ray_t).
__device__ __forceinline__ float ray_tval(const RayTri &r, const RayCol &c, float oz) {
  const float Tz = fs(oz, r.v1z);
  const float q0 = fs(fm(c.Ty, r.e1z), fm(Tz, r.e1y));
  const float q1 = fs(fm(Tz, r.e1x), fm(c.Tx, r.e1z));
  const float q2 = fs(fm(c.Tx, r.e1y), fm(c.Ty, r.e1x));
  return fm(fa(fa(fm(r.e2x, q0), fm(r.e2y, q1)), fm(r.e2z, q2)), r.inv_det);
}

// First index i in [0, n] with tab[i] >= x, and last index in [-1, n-1] with tab[i] <= x, for an
// increasing table of spacing ~1/inv: an arithmetic estimate corrected by table comparisons
// (the result is exactly the table's, the estimate only saves the scan).
__device__ __forceinline__ int tab_first_ge(const float *tab, int n, float x, float inv) {
  const float t0 = __ldg(tab);
  if (!(x > t0)) return 0;                       // also x = -inf
  const float f = fminf((x - t0) * inv, (float)n);  // +inf and huge x clamp to n
  int i = (int)ceilf(f);
  while (i > 0 && __ldg(tab + i - 1) >= x) --i;
  while (i < n && __ldg(tab + i) < x) ++i;
  return i;
}
__device__ __forceinline__ int tab_last_le(const float *tab, int n, float x, float inv) {
  const float t0 = __ldg(tab);
  if (x < t0) return -1;
  const float f = fminf((x - t0) * inv, (float)(n - 1));
  int i = (int)floorf(f);
  while (i < n - 1 && __ldg(tab + i + 1) <= x) ++i;
  while (i >= 0 && __ldg(tab + i) > x) --i;
  return i;
}

// Number of origins r in [0, n) with otop - oz[r] > dthr (float subtraction), for an increasing
// table oz of spacing ~1/inv: the count is a prefix length because otop - oz[r] rounds
// monotonically; an arithmetic estimate is corrected by table comparisons.
__device__ __forceinline__ int count_drop_above(const float *oz, int n, float otop, float dthr,
                                                float inv) {
  const float f = (otop - dthr - __ldg(oz)) * inv;
  int i;
  if (!(f > 0.f)) i = 0;
  else if (f >= (float)n) i = n;
  else i = (int)ceilf(f);
  while (i > 0 && !(otop - __ldg(oz + i - 1) > dthr)) --i;
  while (i < n && otop - __ldg(oz + i) > dthr) ++i;
  return i;
}

// last index tl in [0,31] with pre[tl] <= it (pre nondecreasing, pre[0] = 0)
__device__ __forceinline__ int batch_search(const uint32_t *pre, uint32_t it) {
  int lo = 0, hi = 31;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct WarpScratch {
  float v[32][9];     // triangle vertices of the current batch
  float x[32][7];     // SAT: slab normal, H, 1/(sub-columns per row), 1/nz, slab bound; fill: 1/det,
                      // well-conditioned flag, 1/(sub-columns per row).  Odd row stride: no bank conflicts
  uint32_t rng[32];   // packed sub-cell ranges
  uint32_t pre[33];   // exclusive prefix of item counts
  int jm[32];         // SAT: the triangle's voxel in the chunk; fill: voxels of the chunk below
                      // the triangle's topmost voxel
  uint32_t zrec[32];  // SAT: (triangle slot, p, q) of a sub-column item
  uint32_t seg[33];   // SAT: first pair of each voxel of the chunk, and the end
  uint32_t zown[64];  // SAT: (record lane, cell) of each (triangle, cell) item of a window;
                      // queued fill: Tx of each record
  uint32_t brec[64];  // SAT: queued (triangle slot, p, q) records of sub-columns passing the
                      // z-invariant axes; queued fill: (triangle slot, sub-column) records of
                      // sub-columns passing u/v
  float fty[64];      // queued fill: Ty of each record
};

// ---- item construction -----------------------------------------------------------------------
__device__ __forceinline__ int mesh_of_u(const MeshDesc *md, int nmesh, int64_t u) {
  int lo = 0, hi = nmesh - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (md[mid].u_base <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Boundary voxels of the sorted meshes: B, or (one-graph calls, B the capacity) the device
// plan's count, none when the plan did not fit.
__device__ __forceinline__ int64_t sorted_voxels(const BatchDev &bd, int64_t B) {
  if (!bd.plan) return B;
  return bd.plan->ok ? min(B, (int64_t)bd.plan->ub) : 0;
}

// cflag[u] = 1 where a new Level1 column starts (a mesh's first boundary voxel, or a column
// change within the mesh).  One-graph calls: zero past the device count (the scans run over the
// capacity), and no work items until k_itemstarts counts them.
__global__ void k_colflags(BatchDev bd, const uint32_t *__restrict__ keys,
                           const uint32_t *__restrict__ useg, int64_t Bcap,
                           uint32_t *__restrict__ cflag, uint32_t *__restrict__ nitems) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= Bcap) return;
  if (bd.plan && u == 0) *nitems = 0;
  const int64_t B = sorted_voxels(bd, Bcap);
  if (u >= B) {
    cflag[u] = 0;
    return;
  }
  const int m = mesh_of_u(bd.md, bd.nmesh, u);
  const uint32_t nz = (uint32_t)bd.md[m].g.n[2];
  const uint32_t col = keys[useg[u]] / nz;
  cflag[u] = (u == bd.md[m].u_base || keys[useg[u - 1]] / nz != col) ? 1u : 0u;
}

__global__ void k_colheads(BatchDev bd, const uint32_t *__restrict__ cflag,
                           const uint32_t *__restrict__ cord, int64_t Bcap,
                           uint32_t *__restrict__ colhead) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t B = sorted_voxels(bd, Bcap);
  if (u >= B) return;
  if (cflag[u]) colhead[cord[u]] = (uint32_t)u;
  if (u == B - 1) colhead[cord[u] + cflag[u]] = (uint32_t)B;
}

// An item starts every CH voxels from its column's first boundary voxel and, with z slabs
// (zslab > 0), also where the column enters a new slab of zslab Level1 layers.
__global__ void k_itemflags(BatchDev bd, const uint32_t *__restrict__ keys,
                            const uint32_t *__restrict__ useg, const uint32_t *__restrict__ cflag,
                            const uint32_t *__restrict__ cord, const uint32_t *__restrict__ colhead,
                            int64_t Bcap, int zslab, uint32_t *__restrict__ iflag) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= Bcap) return;
  if (u >= sorted_voxels(bd, Bcap)) {
    iflag[u] = 0;
    return;
  }
  const MeshDesc &d = bd.md[mesh_of_u(bd.md, bd.nmesh, u)];
  const uint32_t c = cord[u] + cflag[u] - 1u;
  bool start = (u - colhead[c]) % d.ch == 0;
  if (zslab > 0 && !start) {
    const uint32_t nz = (uint32_t)d.g.n[2];
    start = (keys[useg[u]] % nz) / (uint32_t)zslab != (keys[useg[u - 1]] % nz) / (uint32_t)zslab;
  }
  // meshes without a Level2 grid (sorted for their normals only) get no Level2 work items
  iflag[u] = (d.has_l2 && start) ? 1u : 0u;
}

__global__ void k_itemstarts(BatchDev bd, const uint32_t *__restrict__ iflag,
                             const uint32_t *__restrict__ iord, int64_t Bcap,
                             uint32_t *__restrict__ istart, uint32_t *__restrict__ nitems) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t B = sorted_voxels(bd, Bcap);
  if (u >= B) return;
  if (iflag[u]) istart[iord[u]] = (uint32_t)u;
  if (u == B - 1) *nitems = iord[u] + iflag[u];
}

// Items of one mesh ordered by z slab (order within a slab is free): per-slab counts, their
// exclusive prefix (ioff[0..nslab]), then each item placed in its slab's range.
__global__ void k_item_slab_count(const uint32_t *__restrict__ istart,
                                  const uint32_t *__restrict__ nitems, const uint32_t *__restrict__ keys,
                                  const uint32_t *__restrict__ useg, int nz, int zslab,
                                  uint32_t *__restrict__ cnt) {
  const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= (int64_t)*nitems) return;
  atomicAdd(&cnt[(keys[useg[istart[it]]] % (uint32_t)nz) / (uint32_t)zslab], 1u);
}

__global__ void k_item_slab_offsets(uint32_t *__restrict__ cnt, int nslab, uint32_t *__restrict__ ioff) {
  if (threadIdx.x != 0) return;
  uint32_t a = 0;
  for (int k = 0; k < nslab; ++k) {
    ioff[k] = a;
    a += cnt[k];
    cnt[k] = ioff[k];  // becomes the slab's placement cursor
  }
  ioff[nslab] = a;
}

__global__ void k_item_slab_place(const uint32_t *__restrict__ istart,
                                  const uint32_t *__restrict__ nitems, const uint32_t *__restrict__ keys,
                                  const uint32_t *__restrict__ useg, int nz, int zslab,
                                  uint32_t *__restrict__ cur, uint32_t *__restrict__ ilist) {
  const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= (int64_t)*nitems) return;
  const uint32_t sl = (keys[useg[istart[it]]] % (uint32_t)nz) / (uint32_t)zslab;
  ilist[atomicAdd(&cur[sl], 1u)] = (uint32_t)it;
}

// 4 bits -> 4 bytes holding 0 or 1 (bit j to byte j; the shifted copies land on distinct bits).
__device__ __forceinline__ uint32_t byte_flags4(uint32_t x) { return (x * 0x00204081u) & 0x01010101u; }

// Output bytes of one boundary voxel when n2z is 8 or 16 and a z layer holds a multiple of 16
// sub-columns: each lane builds 16 consecutive bytes (16 sub-columns of one layer) from the mask
// words, where layer r of a sub-column is bit r of its n2z-bit field, and writes them with one
// 16-byte store (a warp covers 512 contiguous bytes per instruction).  With `codes`, the same 16
// cells go out as one word of 2-bit codes (cell k of the 16 at bits 2k: 0 outside, 1 inside,
// 2 boundary) for the host to expand, a quarter of the bytes over the CPU-GPU link.
template <int NZ>
__device__ __forceinline__ void write_block_vec(uint8_t *out, uint32_t *codes,
                                                const uint32_t *satj, const uint32_t *parj,
                                                const uint32_t *ftacc, int ncol2, unsigned lane,
                                                unsigned long long &nbd, unsigned long long &nin) {
  const int chunks = NZ * ncol2 / 16;
  for (int c = (int)lane; c < chunks; c += 32) {
    const int byte0 = c * 16;
    const int r = byte0 / ncol2, pq0 = byte0 - r * ncol2;
    const uint32_t f16 = (ftacc[pq0 >> 5] >> (pq0 & 31)) & 0xffffu;
    uint32_t o[4], code = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // sub-columns pq0 + 4k .. pq0 + 4k + 3
      uint32_t sf, pf;
      if (NZ == 8) {  // four sub-columns per word
        const int w = (pq0 >> 2) + k;
        sf = (satj[w] >> r) & 0x01010101u;
        pf = (parj[w] >> r) & 0x01010101u;
      } else {  // two sub-columns per word: layer bits at 0 and 16 of each
        const int w = (pq0 >> 1) + 2 * k;
        const uint32_t a = satj[w] >> r, b = satj[w + 1] >> r;
        sf = (a & 1u) | ((a >> 8) & 0x100u) | ((b & 1u) << 16) | ((b << 8) & 0x1000000u);
        const uint32_t c2 = parj[w] >> r, d2 = parj[w + 1] >> r;
        pf = (c2 & 1u) | ((c2 >> 8) & 0x100u) | ((d2 & 1u) << 16) | ((d2 << 8) & 0x1000000u);
      }
      pf ^= byte_flags4((f16 >> (4 * k)) & 0xfu);
      const uint32_t inf = pf & ~sf;
      nbd += (unsigned)__popc(sf);
      nin += (unsigned)__popc(inf);
      o[k] = sf * 254u + inf * 127u;  // flags are 0/1 per byte and disjoint: no carries
      if (codes) {
        // bytes holding 0..2 -> four 2-bit fields
        const uint32_t c4 = sf * 2u + inf;
        code |= ((c4 & 3u) | ((c4 >> 6) & 0xcu) | ((c4 >> 12) & 0x30u) | ((c4 >> 18) & 0xc0u)) << (8 * k);
      }
    }
    // streaming stores: the output is not read again, so it should not displace the working set
    if (codes) __stcs(codes + c, code);
    else __stcs(reinterpret_cast<uint4 *>(out + byte0), make_uint4(o[0], o[1], o[2], o[3]));
  }
}

// n2z bits of a Level2 column starting at bit `off` of a mask.
__device__ __forceinline__ uint32_t column_bits(const uint32_t *m, int off, int n2z) {
  const int sh = off & 31;
  uint32_t b = m[off >> 5] >> sh;
  if (sh + n2z > 32) b |= m[(off >> 5) + 1] << (32 - sh);
  return b;
}

// ---- stencil fill, column prefix ------------------------------------------------------------------
// A triangle whose topmost record in a Level1 column lies below voxel v is not recorded in any
// voxel from v up, so within the column's x/y extent it lies below v's bottom face (up to the
// SAT's rounding, far less than the half Level2 cell to v's first clip height): every covered
// sample keeps it in every slice of v and above.  A Level2 chunk therefore starts from the XOR of
// the sample coverage of the column's triangles whose topmost record lies below its first voxel,
// and draws only the triangles recorded from that voxel up (otherwise every chunk of a tall
// column would draw all the triangles below it again).  Two passes, since the XOR is order-free:
//   k_stencil_segment  one warp per work item: the coverage XOR of the triangles whose topmost
//                      record lies in the item's own voxels (items that end their column skip it),
//                      stored at the item's first voxel;
//   k_stencil_scan     one warp per column with more than one item: those masks turned in place
//                      into exclusive XOR prefixes, the mask each item starts from.
// (One warp per column walking all of its records was latency-bound on the few long columns:
// 186 us on torus262k at 22% warps active.)
constexpr int kPrefixWarps = 4;
constexpr int kPrefixMaskWords = 128;  // 4 * 32 * 32 samples / 32

__global__ void __launch_bounds__(kPrefixWarps * 32) k_stencil_segment(
    BatchDev bd, const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
    const uint32_t *__restrict__ useg, const uint32_t *__restrict__ cflag,
    const uint32_t *__restrict__ cord, const uint32_t *__restrict__ colhead,
    const uint32_t *__restrict__ istart, const uint32_t *__restrict__ nitems, int64_t B) {
  __shared__ uint32_t s_mask[kPrefixWarps][kPrefixMaskWords];
  __shared__ StTri s_t[kPrefixWarps][32];
  __shared__ uint32_t s_pre[kPrefixWarps][32];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const int64_t it = (int64_t)blockIdx.x * kPrefixWarps + warp;
  const int64_t NI = (int64_t)*nitems;
  if (it >= NI) return;
  const uint32_t ua = istart[it];
  const uint32_t ue = it + 1 < NI ? istart[it + 1] : (uint32_t)B;  // the item's voxels [ua, ue)
  if (ue >= colhead[cord[ua] + cflag[ua]]) return;  // the column's last item: no item reads it
  const MeshDesc &d = bd.md[mesh_of_u(bd.md, bd.nmesh, ua)];
  if (!d.has_l2) return;
  const GridDev &g = d.g;
  const int n2x = g.n2[0], n2y = g.n2[1], nz = g.n[2], nx = g.n[0];
  const int SW = 2 * n2x, SH = 2 * n2y;
  const int FWS = (4 * n2x * n2y + 31) >> 5;
  const uint32_t col = keys[useg[ua]] / (uint32_t)nz;
  const int ci = (int)(col % (uint32_t)nx), cj = (int)(col / (uint32_t)nx);
  const float lx = fa(fm((float)ci, g.g[0]), g.bmin[0]), hx = fa(lx, g.g[0]);
  const float ly = fa(fm((float)cj, g.g[1]), g.bmin[1]), hy = fa(ly, g.g[1]);
  uint32_t *mask = s_mask[warp];
  for (int w = lane; w < FWS; w += 32) mask[w] = 0;
  __syncwarp();
  const float4 *__restrict__ ptri = d.ptri;
  const uint32_t e0 = useg[ua], e1 = useg[ue];
  for (uint32_t b0 = e0; b0 < e1; b0 += 32) {
    const uint32_t e = b0 + lane;
    const uint32_t vv = e < e1 ? vals[e] : 0u;
    uint32_t cnt = 0;
    if (vv & 0x80000000u) {  // the triangle's topmost record in the column
      const uint32_t t = vv & 0x7fffffffu;
      const float4 a0 = __ldg(ptri + 3 * (size_t)t), a1 = __ldg(ptri + 3 * (size_t)t + 1),
                   a2 = __ldg(ptri + 3 * (size_t)t + 2);
      const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
      StTri st;
      if (st_setup(V, lx, hx, ly, hy, SW, SH, st)) {
        s_t[warp][lane] = st;
        cnt = (uint32_t)((st.sx1 - st.sx0 + 1) * (st.sy1 - st.sy0 + 1));
      }
    }
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t x = __shfl_up_sync(FULL, inc, o);
      if (lane >= (unsigned)o) inc += x;
    }
    s_pre[warp][lane] = inc - cnt;
    const uint32_t tot = __shfl_sync(FULL, inc, 31);
    __syncwarp();
    for (uint32_t w = lane; w < tot; w += 32) {
      const int tl = batch_search(s_pre[warp], w);
      const StTri &st = s_t[warp][tl];
      const uint32_t loc = w - s_pre[warp][tl];
      const uint32_t nsx = (uint32_t)(st.sx1 - st.sx0 + 1);
      const uint32_t row = loc / nsx;
      const int sx = st.sx0 + (int)(loc - row * nsx), sy = st.sy0 + (int)row;
      float zs;
      if (st_cover(st, sx, sy, zs)) {
        const int sidx = sy * SW + sx;
        atomicXor(&mask[sidx >> 5], 1u << (sidx & 31));
      }
    }
    __syncwarp();
  }
  uint32_t *out = bd.stp + (size_t)ua * bd.stp_words;
  for (int w = lane; w < FWS; w += 32) out[w] = mask[w];
}

__global__ void __launch_bounds__(kPrefixWarps * 32) k_stencil_scan(
    BatchDev bd, const uint32_t *__restrict__ cflag, const uint32_t *__restrict__ cord,
    const uint32_t *__restrict__ colhead, const uint32_t *__restrict__ iflag, int64_t B) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const int64_t c = (int64_t)blockIdx.x * kPrefixWarps + warp;
  const int64_t ncols = (int64_t)cord[B - 1] + cflag[B - 1];
  if (c >= ncols) return;
  const uint32_t u0 = colhead[c], u1 = colhead[c + 1];
  const MeshDesc &d = bd.md[mesh_of_u(bd.md, bd.nmesh, u0)];
  if (!d.has_l2) return;
  // a one-item column has nothing to scan
  bool more = false;
  for (uint32_t u = u0 + 1 + lane; u < u1 && !more; u += 32) more = iflag[u] != 0u;
  if (!__any_sync(FULL, more)) return;
  const int FWS = (4 * d.g.n2[0] * d.g.n2[1] + 31) >> 5;  // <= kPrefixMaskWords
  uint32_t acc[kPrefixMaskWords / 32] = {};
  // the column's item starts 32 voxels at a time (one flag load per lane), then each in order
  for (uint32_t base = u0; base < u1; base += 32) {
    const uint32_t uu = base + lane;
    uint32_t starts = __ballot_sync(FULL, uu < u1 && (uu == u0 || iflag[uu] != 0u));
    while (starts) {
      const uint32_t u = base + (uint32_t)(__ffs(starts) - 1);
      starts &= starts - 1u;
      uint32_t *m = bd.stp + (size_t)u * bd.stp_words;
#pragma unroll
      for (int k = 0; k < kPrefixMaskWords / 32; ++k) {
        const int w = (int)lane + 32 * k;
        if (w < FWS) {
          const uint32_t seg = m[w];  // (the column's last item wrote none: its value goes unused)
          m[w] = acc[k];
          acc[k] ^= seg;
        }
      }
    }
  }
}

// ---- Level2 ------------------------------------------------------------------------------------
// ST: the stencil fill (ClassifyInOut2xLevel2) instead of the ray fill.  QUEUE: the (triangle,
// sub-column) items passing the z-invariant axes are queued and their slab work done 32 records
// at a time (pays off when a pair has many items: triangles large against the Level2 cells);
// otherwise each item lane does its own slab work.  FQ (ray fill): the (triangle, sub-column)
// items passing u/v are queued the same way before their per-voxel work.
template <bool ST, bool QUEUE, bool FQ>
// Six blocks per SM for the queued organisation (80 registers); five with the queued fill (96
// registers, no spills: torus262k 0.535 -> 0.526 ms, a 16k sphere at 4^3 0.136 -> 0.130 ms, while
// five blocks made star1310k, which keeps the inline fill, 3.6% slower); seven for the per-lane
// organisation (72), measured 1.5-3% faster there (the 4096-mesh batch, a 4^3 Level2 grid).
__global__ void __launch_bounds__(kWarps * 32, QUEUE ? (FQ ? 5 : 6) : 7) k_level2c(
    BatchDev bd, const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
    const uint32_t *__restrict__ useg, const uint32_t *__restrict__ cflag,
    const uint32_t *__restrict__ cord, const uint32_t *__restrict__ colhead,
    const uint32_t *__restrict__ istart, const uint32_t *__restrict__ nitems, int per_warp,
    int slab, int zslab, const uint32_t *__restrict__ ilist, const uint32_t *__restrict__ ioff) {
  extern __shared__ uint32_t sm[];
  // one-graph calls launch both SAT organisations; the device plan picks one
  if (bd.plan && bd.plan->qsel != (QUEUE ? 1u : 0u)) return;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t *base = sm + (size_t)warp * per_warp;
  // all items, or (z slabs) this launch's slab of the slab-ordered item list
  const int64_t i0 = ilist ? (int64_t)ioff[slab] : 0;
  const int64_t NI = ilist ? (int64_t)ioff[slab + 1] - i0 : (int64_t)*nitems;
  for (;;) {
  // ---- pull the next chunk item from the queue (one ticket per warp)
  uint32_t tk = 0;
  if (lane == 0) tk = atomicAdd(&bd.queue[1 + slab], 1u);
  const int64_t it = (int64_t)__shfl_sync(FULL, tk, 0);
  if (it >= NI) return;
  const uint32_t ua = ilist ? istart[ilist[i0 + it]] : istart[it];
  const MeshDesc &d = bd.md[mesh_of_u(bd.md, bd.nmesh, ua)];
  const GridDev &g = d.g;
  const float4 *__restrict__ ptri = d.ptri;
  const float4 *__restrict__ fbox = d.fbox;
  const int CH = d.ch;
  const int n2x = g.n2[0], n2y = g.n2[1], n2z = g.n2[2];
  const int cells = n2x * n2y * n2z;
  const int W = (cells + 31) >> 5;
  const int ncol2 = n2x * n2y;
  const int FW = (ncol2 + 31) >> 5;
  uint32_t *sat = base;
  uint32_t *par = sat + CH * W;
  uint32_t *ft = par + CH * W;
  int *kz = (int *)(ft + CH * FW);
  uint32_t *ftacc = (uint32_t *)(kz + CH);
  WarpScratch &ws = *reinterpret_cast<WarpScratch *>(ftacc + FW);
  // stencil fill: per voxel, (2 n2x * 2 n2y) sample columns of n2z slice toggle bits; per voxel
  // one bit per sample toggling every slice of that voxel and of the voxels above it
  uint32_t *stg = reinterpret_cast<uint32_t *>(&ws + 1);
  const int SWd = 4 * W;
  const int FWS = (4 * ncol2 + 31) >> 5;
  uint32_t *sft = stg + CH * SWd, *sftacc = sft + CH * FWS;

  const uint32_t ucol_end = colhead[cord[ua] + cflag[ua]];  // first voxel of the next column
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const uint32_t col = keys[useg[ua]] / (uint32_t)nz;
  int m = (int)min((uint32_t)CH, ucol_end - ua);
  if (zslab > 0) {
    // this launch takes one slab of zslab Level1 layers; an item ends at the slab's edge and at
    // the next CH-aligned item start of its column
    const uint32_t chead = colhead[cord[ua] + cflag[ua] - 1u];
    bool ok = false;
    if ((int)lane < m) {
      const int zl = (int)(keys[useg[ua + lane]] - col * (uint32_t)nz);
      ok = zl / zslab == slab && (lane == 0 || (ua + lane - chead) % (uint32_t)CH != 0);
    }
    m = __ffs(~__ballot_sync(FULL, ok)) - 1;  // leading run of voxels of this item
    if (m < 0) m = 32;
  }
  // clear the masks of the chunk's m voxels only (the arrays are sized for CH voxels)
  for (int w = lane; w < m * W; w += 32) { sat[w] = 0; par[w] = 0; }
  for (int w = lane; w < m * FW; w += 32) ft[w] = 0;
  if (ST) {
    for (int w = lane; w < m * SWd; w += 32) stg[w] = 0;
    for (int w = lane; w < m * FWS; w += 32) sft[w] = 0;
    // the coverage parity of the column's triangles recorded only below the chunk (none below a
    // column's first voxel; the prefix pass writes the masks of the later chunk starts)
    const bool first = colhead[cord[ua] + cflag[ua] - 1u] == ua;
    for (int w = lane; w < FWS; w += 32) sftacc[w] = first ? 0u : bd.stp[(size_t)ua * bd.stp_words + w];
  }
  const int ci = (int)(col % (uint32_t)nx), cj = (int)(col / (uint32_t)nx);
  if ((int)lane < m) kz[lane] = (int)(keys[useg[ua + lane]] - col * (uint32_t)nz);
  __syncwarp();

  const float *sx = g.c2s[0] + (size_t)ci * n2x, *sy = g.c2s[1] + (size_t)cj * n2y;
  const float *ox = g.o2[0] + (size_t)ci * n2x, *oy = g.o2[1] + (size_t)cj * n2y;
  const float sx0 = __ldg(sx), sx1 = __ldg(sx + n2x - 1), sy0 = __ldg(sy), sy1 = __ldg(sy + n2y - 1);

  // ---------------- SAT of each voxel's own triangles: the chunk's (voxel, triangle) pairs are
  // contiguous in the sorted lists and are taken 32 at a time across voxel boundaries.
  if ((int)lane < m) ws.seg[lane] = useg[ua + lane];
  if (lane == 0) ws.seg[m] = useg[ua + m];
  __syncwarp();
  {
    const uint32_t S0 = ws.seg[0], S1 = ws.seg[m];
    for (uint32_t b0 = S0; b0 < S1; b0 += 32) {
      const uint32_t e = b0 + lane;
      uint32_t cnt = 0;
      if (e < S1) {
        int jv = 0;  // last voxel whose segment starts at or before e
#pragma unroll
        for (int st = 16; st > 0; st >>= 1)
          if (jv + st <= m - 1 && ws.seg[jv + st] <= e) jv += st;
        const float *sz = g.c2s[2] + (size_t)kz[jv] * n2z;
        const float sz0 = __ldg(sz), sz1 = __ldg(sz + n2z - 1);
        const uint32_t t = vals[e] & 0x7fffffffu;
        const float4 a0 = __ldg(ptri + 3 * (size_t)t), a1 = __ldg(ptri + 3 * (size_t)t + 1),
                     a2 = __ldg(ptri + 3 * (size_t)t + 2);
        const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
        int p0, p1, q0, q1, r0, r1;
        l2_cell_range(fminf(V[0], fminf(V[3], V[6])), fmaxf(V[0], fmaxf(V[3], V[6])), sx0, g.e2[0],
                 g.inv_g2[0], n2x, p0, p1);
        l2_cell_range(fminf(V[1], fminf(V[4], V[7])), fmaxf(V[1], fmaxf(V[4], V[7])), sy0, g.e2[1],
                 g.inv_g2[1], n2y, q0, q1);
        l2_cell_range(fminf(V[2], fminf(V[5], V[8])), fmaxf(V[2], fmaxf(V[5], V[8])), sz0, g.e2[2],
                 g.inv_g2[2], n2z, r0, r1);
        if (p0 <= p1 && q0 <= q1 && r0 <= r1) {
          const PlaneSlab ps = plane_slab(V, sx0, sx1, sy0, sy1, sz0, sz1, g.e2);
#pragma unroll
          for (int q = 0; q < 9; ++q) ws.v[lane][q] = V[q];
          ws.x[lane][0] = ps.nx; ws.x[lane][1] = ps.ny; ws.x[lane][2] = ps.nz; ws.x[lane][3] = ps.H;
          const int np = p1 - p0 + 1;
          // per-triangle factors of the (triangle, sub-column) items below
          ws.x[lane][4] = __frcp_rn((float)np);
          ws.x[lane][5] = fabsf(ps.nz) > 0.f ? __frcp_rn(ps.nz) : 0.f;
          ws.x[lane][6] = ps.H + 8.f * EPS24 * fabsf(ps.nz) * (fabsf(V[2]) + fabsf(sz0) + fabsf(sz1));
          ws.rng[lane] = (uint32_t)p0 | ((uint32_t)np << 6) | ((uint32_t)q0 << 12) |
                         ((uint32_t)r0 << 18) | ((uint32_t)r1 << 24);
          ws.jm[lane] = jv;
          cnt = (uint32_t)(np * (q1 - q0 + 1));
        }
      }
      const uint32_t inc = warp_incl_scan(cnt);
      ws.pre[lane] = inc - cnt;
      const uint32_t tot = __shfl_sync(FULL, inc, 31);
      __syncwarp();
      if constexpr (QUEUE) {
      // (triangle, sub-column) items, 32 at a time (B1): the z-invariant SAT part; the items that
      // pass are queued as records.  Every 32 records (B2): the plane slab selects the cells left
      // for the full test, so that those lanes all work; then the (triangle, cell) tests run 32
      // at a time whatever the per-column cell counts.  Each record lane lists its cells in a
      // window of 64 slots (its lane and the cell's z), so a test lane reads its work from one
      // slot.
      uint32_t nrec = 0;
      auto run_records = [&](uint32_t nr) {
        uint32_t zm = 0, rec = 0;
        if (lane < nr) {
          rec = ws.brec[lane];
          const int tl = (int)(rec & 31u), p = (int)((rec >> 5) & 63u), q = (int)((rec >> 11) & 63u);
          const uint32_t rg = ws.rng[tl];
          const int r0 = (int)((rg >> 18) & 63u), r1 = (int)((rg >> 24) & 63u);
          const int jv = ws.jm[tl];
          const uint32_t *satj = sat + jv * W;
          const float *sz = g.c2s[2] + (size_t)kz[jv] * n2z;
          const float sz0 = __ldg(sz);
          // cells of this column already marked by another triangle need no test (OR only)
          const int off = (q * n2x + p) * n2z, sh = off & 31;
          uint32_t done = satj[off >> 5] >> sh;
          if (sh + n2z > 32) done |= satj[(off >> 5) + 1] << (32 - sh);
          const float V0 = ws.v[tl][0], V1 = ws.v[tl][1], V2 = ws.v[tl][2];
          const float cx = __ldg(sx + p), cy = __ldg(sy + q);
          const float nxs = ws.x[tl][0], nys = ws.x[tl][1], nzs = ws.x[tl][2], H = ws.x[tl][3];
          const float sxy = fa(fm(nxs, fs(V0, cx)), fm(nys, fs(V1, cy)));
          // The per-cell slab test |sxy + nz (V0z - cz)| <= H can only pass for cz within
          // H/|nz| of V0z + sxy/nz; the interval is widened by the float error of that test
          // (a few ulps of its terms, over |nz|) and one cell, and the exact per-cell test
          // still runs.
          int ra = r0, rb = r1;
          const float rnz = ws.x[tl][5];
          if (rnz != 0.f) {
            const float zc = V2 + sxy * rnz;
            const float ext = (ws.x[tl][6] + 8.f * EPS24 * fabsf(sxy)) * fabsf(rnz);
            const float igz = g.inv_g2[2];
            const float fa0 = (zc - ext - sz0) * igz - 1.f, fb0 = (zc + ext - sz0) * igz + 1.f;
            if (fa0 > -2.f) ra = max(ra, (int)floorf(fminf(fa0, (float)n2z + 2.f)));
            if (fb0 < (float)n2z + 2.f) rb = min(rb, (int)ceilf(fmaxf(fb0, -2.f)));
          }
          // The slab value is monotone in cz (each operation on cz is a monotone rounding:
          // V0z - cz, then times nz, then plus sxy), so the cells passing |value| <= H are
          // one interval of [ra, rb]; its ends are found by testing inwards from both ends.
          while (ra <= rb && !(fabsf(fa(sxy, fm(nzs, fs(V2, __ldg(sz + ra))))) <= H)) ++ra;
          while (rb > ra && !(fabsf(fa(sxy, fm(nzs, fs(V2, __ldg(sz + rb))))) <= H)) --rb;
          if (ra <= rb)
            zm = ((rb - ra + 1 >= 32) ? 0xffffffffu : ((1u << (rb - ra + 1)) - 1u)) << ra & ~done;
        }
        __syncwarp();  // records read: the queue may be refilled
        const uint32_t zc = (uint32_t)__popc(zm);
        const uint32_t zinc = warp_incl_scan(zc);
        ws.zrec[lane] = rec;
        const uint32_t ztot = __shfl_sync(FULL, zinc, 31);
        for (uint32_t w0 = 0; w0 < ztot; w0 += 64) {
          // each record lane lists its cells of this window: (record lane, cell r) per slot
          {
            uint32_t mm = zm, pos = zinc - zc;
            while (mm && pos < w0) { mm &= mm - 1u; ++pos; }
            while (mm && pos < w0 + 64u) {
              ws.zown[pos - w0] = lane | ((uint32_t)(__ffs(mm) - 1) << 5);
              mm &= mm - 1u;
              ++pos;
            }
          }
          __syncwarp();
          const uint32_t wn = min(64u, ztot - w0);
          for (uint32_t z = lane; z < wn; z += 32) {
            const uint32_t own = ws.zown[z];
            const uint32_t rc = ws.zrec[own & 31u];
            const int r = (int)(own >> 5);
            const int tl = (int)(rc & 31u), p = (int)((rc >> 5) & 63u), q = (int)((rc >> 11) & 63u);
            const int jv = ws.jm[tl];
            const float *sz = g.c2s[2] + (size_t)kz[jv] * n2z;
            float V[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) V[c] = ws.v[tl][c];
            SatCol sc;
            sat_col_values(V, __ldg(sx + p), __ldg(sy + q), sc);
            if (sat_z(sc, V, __ldg(sz + r), g.e2)) {
              const int bi = (q * n2x + p) * n2z + r;
              atomicOr(&sat[jv * W + (bi >> 5)], 1u << (bi & 31));
            }
          }
          __syncwarp();
        }
      };
      // one call site for the record work (the last rounds only drain the queue)
      for (uint32_t wb = 0; wb < tot || nrec > 0; wb += 32) {
        const uint32_t w = wb + lane;
        bool pass = false;
        uint32_t rec = 0;
        if (w < tot) {
          const int tl = batch_search(ws.pre, w);
          const uint32_t loc = w - ws.pre[tl];
          const uint32_t rg = ws.rng[tl];
          const int np = (int)((rg >> 6) & 63u);
          // loc / np by a float reciprocal: exact here (loc < 1024, np <= 32, so the quotient of
          // loc + 1/2 stays at least 1/64 away from an integer, far above the rounding)
          const int qq = __float2int_rz(((float)loc + 0.5f) * ws.x[tl][4]);
          const int p = (int)(rg & 63u) + (int)loc - qq * np;
          const int q = (int)((rg >> 12) & 63u) + qq;
          // No check for sub-columns whose cells are all marked already: it skipped ~2% of the
          // items and cost more than it saved (the Level2 kernel: star1310k 3.96 -> 3.84 ms,
          // torus262k 0.558 -> 0.540 ms); the record round still leaves marked cells out.
          {
            float V[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) V[c] = ws.v[tl][c];
            SatCol sc;
            if (sat_col(V, __ldg(sx + p), __ldg(sy + q), g.e2, sc)) {
              pass = true;
              rec = (uint32_t)tl | ((uint32_t)p << 5) | ((uint32_t)q << 11);
            }
          }
        }
        const uint32_t bal = __ballot_sync(FULL, pass);
        if (pass) ws.brec[nrec + __popc(bal & ((1u << lane) - 1u))] = rec;
        nrec += (uint32_t)__popc(bal);
        __syncwarp();
        if (nrec >= 32 || (wb + 32 >= tot && nrec > 0)) {
          const uint32_t nr = min(nrec, 32u);
          run_records(nr);
          // move the records beyond the first nr to the front
          const uint32_t rest = (lane + nr < nrec) ? ws.brec[nr + lane] : 0u;
          __syncwarp();
          if (lane + nr < nrec) ws.brec[lane] = rest;
          nrec -= nr;
          __syncwarp();
        }
      }
      } else {
      // (triangle, sub-column) items, 32 at a time: z-invariant SAT part and the plane slab
      // select the cells left for the full test; then those (triangle, cell) tests run 32 at a
      // time so that the lanes stay busy whatever the per-column cell counts.  Each item lane
      // lists its cells in a window of 64 slots (its lane and the cell's z), so a test lane
      // reads its work from one slot.
      for (uint32_t wb = 0; wb < tot; wb += 32) {
        const uint32_t w = wb + lane;
        uint32_t zm = 0, rec = 0;
        if (w < tot) {
          const int tl = batch_search(ws.pre, w);
          const uint32_t loc = w - ws.pre[tl];
          const uint32_t rg = ws.rng[tl];
          const int np = (int)((rg >> 6) & 63u);
          // loc / np by a float reciprocal: exact here (loc < 1024, np <= 32, so the quotient of
          // loc + 1/2 stays at least 1/64 away from an integer, far above the rounding)
          const int qq = __float2int_rz(((float)loc + 0.5f) * ws.x[tl][4]);
          const int p = (int)(rg & 63u) + (int)loc - qq * np;
          const int q = (int)((rg >> 12) & 63u) + qq;
          const int r0 = (int)((rg >> 18) & 63u), r1 = (int)((rg >> 24) & 63u);
          const int jv = ws.jm[tl];
          const uint32_t *satj = sat + jv * W;
          const float *sz = g.c2s[2] + (size_t)kz[jv] * n2z;
          const float sz0 = __ldg(sz), sz1 = __ldg(sz + n2z - 1);
          // cells of this column already marked by another triangle need no test (OR only); a
          // gate for columns marked entirely cost more than it saved, as in the queued form
          const int off = (q * n2x + p) * n2z, sh = off & 31;
          uint32_t done = satj[off >> 5] >> sh;
          if (sh + n2z > 32) done |= satj[(off >> 5) + 1] << (32 - sh);
          {
            float V[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) V[c] = ws.v[tl][c];
            const float cx = __ldg(sx + p), cy = __ldg(sy + q);
            SatCol sc;
            if (sat_col(V, cx, cy, g.e2, sc)) {
              const float nxs = ws.x[tl][0], nys = ws.x[tl][1], nzs = ws.x[tl][2], H = ws.x[tl][3];
              const float sxy = fa(fm(nxs, fs(V[0], cx)), fm(nys, fs(V[1], cy)));
              // The per-cell slab test |sxy + nz (V0z - cz)| <= H can only pass for cz within
              // H/|nz| of V0z + sxy/nz; the interval is widened by the float error of that test
              // (a few ulps of its terms, over |nz|) and one cell, and the exact per-cell test
              // still runs.
              int ra = r0, rb = r1;
              const float rnz = ws.x[tl][5];
              if (rnz != 0.f) {
                const float zc = V[2] + sxy * rnz;
                const float ext = (ws.x[tl][6] + 8.f * EPS24 * fabsf(sxy)) * fabsf(rnz);
                const float igz = g.inv_g2[2];
                const float fa0 = (zc - ext - sz0) * igz - 1.f, fb0 = (zc + ext - sz0) * igz + 1.f;
                if (fa0 > -2.f) ra = max(ra, (int)floorf(fminf(fa0, (float)n2z + 2.f)));
                if (fb0 < (float)n2z + 2.f) rb = min(rb, (int)ceilf(fmaxf(fb0, -2.f)));
              }
              // The slab value is monotone in cz (each operation on cz is a monotone rounding:
              // V0z - cz, then times nz, then plus sxy), so the cells passing |value| <= H are
              // one interval of [ra, rb]; its ends are found by testing inwards from both ends.
              while (ra <= rb && !(fabsf(fa(sxy, fm(nzs, fs(V[2], __ldg(sz + ra))))) <= H)) ++ra;
              while (rb > ra && !(fabsf(fa(sxy, fm(nzs, fs(V[2], __ldg(sz + rb))))) <= H)) --rb;
              if (ra <= rb)
                zm = ((rb - ra + 1 >= 32) ? 0xffffffffu : ((1u << (rb - ra + 1)) - 1u)) << ra & ~done;
              rec = (uint32_t)tl | ((uint32_t)p << 5) | ((uint32_t)q << 11);
            }
          }
        }
        const uint32_t zc = (uint32_t)__popc(zm);
        const uint32_t zinc = warp_incl_scan(zc);
        ws.zrec[lane] = rec;
        const uint32_t ztot = __shfl_sync(FULL, zinc, 31);
        for (uint32_t w0 = 0; w0 < ztot; w0 += 64) {
          // each record lane lists its cells of this window: (record lane, cell r) per slot
          {
            uint32_t mm = zm, pos = zinc - zc;
            while (mm && pos < w0) { mm &= mm - 1u; ++pos; }
            while (mm && pos < w0 + 64u) {
              ws.zown[pos - w0] = lane | ((uint32_t)(__ffs(mm) - 1) << 5);
              mm &= mm - 1u;
              ++pos;
            }
          }
          __syncwarp();
          const uint32_t wn = min(64u, ztot - w0);
          for (uint32_t z = lane; z < wn; z += 32) {
            const uint32_t own = ws.zown[z];
            const uint32_t rc = ws.zrec[own & 31u];
            const int r = (int)(own >> 5);
            const int tl = (int)(rc & 31u), p = (int)((rc >> 5) & 63u), q = (int)((rc >> 11) & 63u);
            const int jv = ws.jm[tl];
            const float *sz = g.c2s[2] + (size_t)kz[jv] * n2z;
            float V[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) V[c] = ws.v[tl][c];
            SatCol sc;
            sat_col_values(V, __ldg(sx + p), __ldg(sy + q), sc);
            if (sat_z(sc, V, __ldg(sz + r), g.e2)) {
              const int bi = (q * n2x + p) * n2z + r;
              atomicOr(&sat[jv * W + (bi >> 5)], 1u << (bi & 31));
            }
          }
          __syncwarp();
        }
      }
      }
    }
  }

  uint64_t nun = 0;
  if (ST) {
    // ---------------- stencil fill: the triangles recorded anywhere in the Level1 column (the
    // voxel strip of CreateVoxelStripDisplayLists, src/Object.cpp:605-633: each once, at its
    // topmost record) are drawn into 2 n2x x 2 n2y samples over the Level1 voxel's x/y extent
    // (glOrtho over [i*gridSizeX + bBoxMin, + gridSizeX], :1241-1266).  Slice s of voxel k clips
    // at the Level2 ray-origin height o2z[k][s] (minZ + (s + 0.5)*gridSizeZ2, :1297), so a
    // covered sample at height zs counts in every slice from the first with o2z >= zs: one
    // toggle bit there, expanded by a prefix XOR below.
    // triangles recorded from the chunk's first voxel up (those below are in the prefix)
    const uint32_t g0 = useg[ua], g1 = useg[ucol_end];
    const int SW = 2 * n2x, SH = 2 * n2y;
    const float lx = fa(fm((float)ci, g.g[0]), g.bmin[0]), hx = fa(lx, g.g[0]);
    const float ly = fa(fm((float)cj, g.g[1]), g.bmin[1]), hy = fa(ly, g.g[1]);
    const float *ozt = g.o2[2];
    // with increasing clip heights, the chunk's highest one is its top voxel's last slice
    const float top_clip = __ldg(ozt + (size_t)kz[m - 1] * n2z + n2z - 1);
    for (uint32_t b0 = g0; b0 < g1; b0 += 32) {
      const uint32_t e = b0 + lane;
      const uint32_t vv = e < g1 ? vals[e] : 0u;
      uint32_t cnt = 0;
      if (vv & 0x80000000u) {
        const uint32_t t = vv & 0x7fffffffu;
        const float4 a0 = __ldg(ptri + 3 * (size_t)t), a1 = __ldg(ptri + 3 * (size_t)t + 1),
                     a2 = __ldg(ptri + 3 * (size_t)t + 2);
        const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
        // The interpolated height of a covered sample is a convex combination of the vertex
        // heights up to 7 eps max|z| of rounding, so a triangle whose lowest vertex lies more
        // than 16 eps max|z| above the chunk's highest clip height counts in none of its slices.
        const float zmn = fminf(V[2], fminf(V[5], V[8]));
        const float zmag = fmaxf(fabsf(V[2]), fmaxf(fabsf(V[5]), fabsf(V[8])));
        const bool above = g.oz_monotone && zmn - 16.f * EPS24 * zmag > top_clip;
        StTri st;
        if (!above && st_setup(V, lx, hx, ly, hy, SW, SH, st)) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            ws.v[lane][2 * c] = __int_as_float(st.X[c]);
            ws.v[lane][2 * c + 1] = __int_as_float(st.Y[c]);
            ws.v[lane][6 + c] = st.z[c];
          }
          ws.x[lane][0] = st.rA;
          const int nsx = st.sx1 - st.sx0 + 1;
          ws.rng[lane] = (uint32_t)st.sx0 | ((uint32_t)nsx << 7) | ((uint32_t)st.sy0 << 14);
          cnt = (uint32_t)(nsx * (st.sy1 - st.sy0 + 1));
        }
      }
      const uint32_t inc = warp_incl_scan(cnt);
      ws.pre[lane] = inc - cnt;
      const uint32_t tot = __shfl_sync(FULL, inc, 31);
      __syncwarp();
      for (uint32_t w = lane; w < tot; w += 32) {
        const int tl = batch_search(ws.pre, w);
        const uint32_t loc = w - ws.pre[tl];
        const uint32_t rg = ws.rng[tl];
        const uint32_t nsx = (rg >> 7) & 127u;
        const uint32_t row = loc / nsx;
        StTri st;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          st.X[c] = __float_as_int(ws.v[tl][2 * c]);
          st.Y[c] = __float_as_int(ws.v[tl][2 * c + 1]);
          st.z[c] = ws.v[tl][6 + c];
        }
        st.rA = ws.x[tl][0];
        const int sx = (int)(rg & 127u) + (int)(loc - row * nsx), sy = (int)((rg >> 14) & 127u) + (int)row;
        float zs;
        if (!st_cover(st, sx, sy, zs)) continue;
        const int sidx = sy * SW + sx, sbit = sidx * n2z;
        if (g.oz_monotone) {
          // clip heights increase through the chunk: the lowest voxel whose top clip keeps zs
          // gets its toggle at the first such slice, and every voxel above it keeps zs in all
          // slices (one bit in its sample-toggle row, accumulated upwards)
          int jv = 0;
          while (jv < m && !(__ldg(ozt + (size_t)kz[jv] * n2z + n2z - 1) >= zs)) ++jv;
          if (jv < m) {
            const int b = sbit + st_first_slice(ozt + (size_t)kz[jv] * n2z, n2z, zs);
            atomicXor(&stg[jv * SWd + (b >> 5)], 1u << (b & 31));
            if (jv + 1 < m) atomicXor(&sft[(jv + 1) * FWS + (sidx >> 5)], 1u << (sidx & 31));
          }
        } else {
          for (int jv = m - 1; jv >= 0; --jv) {
            const int s0 = st_first_slice(ozt + (size_t)kz[jv] * n2z, n2z, zs);
            if (s0 < n2z) {
              const int b = sbit + s0;
              atomicXor(&stg[jv * SWd + (b >> 5)], 1u << (b & 31));
            }
          }
        }
      }
      __syncwarp();
    }
    // a cell is inside when at least 3 of its 4 samples are odd (ClassifyInOut2xLevel2,
    // :1383-1401): parity per slice = prefix XOR of the sample column's toggles
    const uint32_t zmask = n2z >= 32 ? 0xffffffffu : ((1u << n2z) - 1u);
    for (int jv = 0; jv < m; ++jv) {
      // samples toggled in every slice of this voxel: the XOR of the rows of it and below
      for (int w = lane; w < FWS; w += 32) sftacc[w] ^= sft[jv * FWS + w];
      __syncwarp();
      const uint32_t *sj = stg + jv * SWd;
      for (int pq = lane; pq < ncol2; pq += 32) {
        const int q = pq / n2x, p = pq - q * n2x;
        uint32_t x[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int sidx = (2 * q + (a >> 1)) * SW + 2 * p + (a & 1);
          uint32_t y = column_bits(sj, sidx * n2z, n2z);
          y ^= y << 1; y ^= y << 2; y ^= y << 4; y ^= y << 8; y ^= y << 16;
          if ((sftacc[sidx >> 5] >> (sidx & 31)) & 1u) y = ~y;
          x[a] = y;
        }
        const uint32_t in = ((x[0] & x[1] & (x[2] | x[3])) | (x[2] & x[3] & (x[0] | x[1]))) & zmask;
        if (in) or_column(par + jv * W, pq, n2z, in);
      }
    }
    __syncwarp();
  } else {
  // ---------------- fill: u/v once per (triangle, sub-column) for the whole chunk
  const uint32_t f0 = useg[ua], f1 = useg[ucol_end];
  const float *ozt = g.o2[2];
  const float oz_lo = __ldg(ozt + (size_t)kz[0] * n2z);
  const float oz_hi = __ldg(ozt + (size_t)kz[m - 1] * n2z + n2z - 1);
  for (uint32_t b0 = f0; b0 < f1; b0 += 32) {
    const uint32_t e = b0 + lane;
    const uint32_t vv = e < f1 ? vals[e] : 0u;
    uint32_t cnt = 0;
    if (vv & 0x80000000u) {
      const uint32_t t = vv & 0x7fffffffu;
      const int zt = (int)(keys[e] - col * (uint32_t)nz);
      int jm = 0;
      while (jm < m && kz[jm] <= zt) ++jm;
      nun += (uint64_t)jm;
      const float4 fb = __ldg(fbox + t);
      if (jm > 0 && fb.x <= fb.z) {
        // sub-columns whose origin lies in the box: first origin >= lo, last origin <= hi
        const int p0 = tab_first_ge(ox, n2x, fb.x, g.inv_g2[0]);
        const int p1 = tab_last_le(ox, n2x, fb.z, g.inv_g2[0]);
        const int q0 = tab_first_ge(oy, n2y, fb.y, g.inv_g2[1]);
        const int q1 = tab_last_le(oy, n2y, fb.w, g.inv_g2[1]);
        if (p0 <= p1 && q0 <= q1) {
          const float4 a0 = __ldg(ptri + 3 * (size_t)t), a1 = __ldg(ptri + 3 * (size_t)t + 1),
                       a2 = __ldg(ptri + 3 * (size_t)t + 2);
          const float V[9] = {a0.x, a0.y, a0.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z};
          RayTri rt;
          ray_tri_pre(V, a2.w, rt);
          ws.v[lane][0] = rt.v1x; ws.v[lane][1] = rt.v1y; ws.v[lane][2] = rt.v1z;
          ws.v[lane][3] = rt.e1x; ws.v[lane][4] = rt.e1y; ws.v[lane][5] = rt.e1z;
          ws.v[lane][6] = rt.e2x; ws.v[lane][7] = rt.e2y; ws.v[lane][8] = rt.e2z;
          ws.x[lane][0] = rt.inv_det;
          // Certification bound E2 (below), or 0 where there is none: an unbounded box marks an
          // ill-conditioned x/y projection.  |t - t*| <= 8.2 eps M1 |1/det| for every origin of
          // the chunk (t* exact, affine and decreasing in the origin height), with M1 taken at
          // the largest |Tx|, |Ty| over the triangle's sub-columns (Tx = ox - v1x rounds
          // monotonically in ox, so the extremes sit at the range ends) and the largest |Tz|
          // over the chunk's origins; 16 eps gives the float evaluation room.
          float E2 = 0.f;
          if (g.oz_monotone && !isinf(fb.x) && !isinf(fb.z)) {
            const float Zm = fmaxf(fabsf(oz_lo - rt.v1z), fabsf(oz_hi - rt.v1z)) * 1.0001f;
            const float atx = fmaxf(fabsf(fs(__ldg(ox + p0), rt.v1x)), fabsf(fs(__ldg(ox + p1), rt.v1x)));
            const float aty = fmaxf(fabsf(fs(__ldg(oy + q0), rt.v1y)), fabsf(fs(__ldg(oy + q1), rt.v1y)));
            const float M1 = fabsf(rt.e2x) * (aty * fabsf(rt.e1z) + Zm * fabsf(rt.e1y)) +
                             fabsf(rt.e2y) * (Zm * fabsf(rt.e1x) + atx * fabsf(rt.e1z)) +
                             fabsf(rt.e2z) * (atx * fabsf(rt.e1y) + aty * fabsf(rt.e1x));
            E2 = 2.f * 16.f * EPS24 * M1 * fabsf(rt.inv_det) * 1.0001f;
          }
          ws.x[lane][1] = E2;
          const int np = p1 - p0 + 1;
          ws.x[lane][2] = __frcp_rn((float)np);
          ws.rng[lane] = (uint32_t)p0 | ((uint32_t)np << 6) | ((uint32_t)q0 << 12);
          ws.jm[lane] = jm;
          cnt = (uint32_t)(np * (q1 - q0 + 1));
        }
      }
    }
    const uint32_t inc = warp_incl_scan(cnt);
    ws.pre[lane] = inc - cnt;
    const uint32_t tot = __shfl_sync(FULL, inc, 31);
    __syncwarp();
    // The toggles of one (triangle slot, sub-column pq) item that passed u/v, in the voxels of the
    // chunk at or below the triangle's topmost voxel, top down.
    auto item_voxels = [&](const RayTri &rt, const RayCol &rc, int tl, int pq) {
      const float E2 = ws.x[tl][1];
      const bool well = E2 > 0.f;
      for (int jv = ws.jm[tl] - 1; jv >= 0; --jv) {
        const float *oz = ozt + (size_t)kz[jv] * n2z;
        uint32_t bits = 0;
        if (well) {
          const float otop = __ldg(oz + n2z - 1);
          const float ttop = ray_tval(rt, rc, otop);
          if (ttop > g.thr + E2) {
            // this voxel and every lower voxel of the chunk are hit at every origin
            atomicXor(&ft[jv * FW + (pq >> 5)], 1u << (pq & 31));
            break;
          }
          // Along +z, t* (exact) grows by exactly the drop of the origin below otop:
          // t*(oz) = t*(otop) + (otop - oz), and the float t at every origin and at otop lies
          // within E2/2 of t*.  So with d = otop - oz, the float t exceeds thr when
          // d > thr - ttop + E2 and does not when d <= thr - ttop - E2; the thresholds carry the
          // rounding of d and of themselves (K bounds every magnitude involved).  Origins
          // between the two run the exact test.
          const float dmax = otop - __ldg(oz);
          const float K = fabsf(ttop) + dmax + g.thr;
          const float slack = E2 * 1.0001f + 8.f * EPS24 * K + 1e-30f;
          const float dhit = (g.thr - ttop) + slack, dmiss = (g.thr - ttop) - slack;
          // d = otop - oz rounds monotonically and falls as r grows, so the certain hits are the
          // origins r < rh and the exact tests the band rh <= r < rm
          const int rh = count_drop_above(oz, n2z, otop, dhit, g.inv_g2[2]);
          const int rm = count_drop_above(oz, n2z, otop, dmiss, g.inv_g2[2]);
          bits = rh >= 32 ? 0xffffffffu : ((1u << rh) - 1u);
          for (int r = rh; r < rm; ++r)
            if (ray_t(rt, rc, __ldg(oz + r), g.thr)) bits |= 1u << r;
        } else {
          for (int r = 0; r < n2z; ++r)
            if (ray_t(rt, rc, __ldg(oz + r), g.thr)) bits |= 1u << r;
        }
        if (bits) xor_column(par + jv * W, pq, n2z, bits);
      }
    };
    // (triangle slot, p, q) of item w of this batch
    auto item_of = [&](uint32_t w, int &tl, int &p, int &q) {
      tl = batch_search(ws.pre, w);
      const uint32_t loc = w - ws.pre[tl];
      const uint32_t rg = ws.rng[tl];
      const int np = (int)((rg >> 6) & 63u);
      const int qq = __float2int_rz(((float)loc + 0.5f) * ws.x[tl][2]);
      p = (int)(rg & 63u) + (int)loc - qq * np;
      q = (int)((rg >> 12) & 63u) + qq;
    };
    if constexpr (!FQ) {
      // each item lane goes on to its own voxels
      for (uint32_t w = lane; w < tot; w += 32) {
        int tl, p, q;
        item_of(w, tl, p, q);
        RayTri rt;
        rt.v1x = ws.v[tl][0]; rt.v1y = ws.v[tl][1]; rt.v1z = ws.v[tl][2];
        rt.e1x = ws.v[tl][3]; rt.e1y = ws.v[tl][4]; rt.e1z = ws.v[tl][5];
        rt.e2x = ws.v[tl][6]; rt.e2y = ws.v[tl][7]; rt.e2z = ws.v[tl][8];
        rt.inv_det = ws.x[tl][0];
        rt.ok = true;
        RayCol rc;
        if (!ray_col(rt, __ldg(ox + p), __ldg(oy + q), rc)) continue;
        item_voxels(rt, rc, tl, q * n2x + p);
      }
    } else {
      // the items passing u/v are queued as (triangle slot, sub-column) records with their Tx, Ty
      // and their voxels done 32 records at a time, so that every lane of that loop works (most
      // items fail u/v: 34% pass on torus262k)
      uint32_t nfr = 0;
      for (uint32_t wb = 0; wb < tot || nfr > 0; wb += 32) {
        const uint32_t w = wb + lane;
        bool pass = false;
        uint32_t frec = 0;
        RayCol rc0;
        if (w < tot) {
          int tl, p, q;
          item_of(w, tl, p, q);
          RayTri rt;  // the fields of the u/v test
          rt.v1x = ws.v[tl][0]; rt.v1y = ws.v[tl][1];
          rt.e1x = ws.v[tl][3]; rt.e1y = ws.v[tl][4];
          rt.e2x = ws.v[tl][6]; rt.e2y = ws.v[tl][7];
          rt.inv_det = ws.x[tl][0];
          if (ray_col(rt, __ldg(ox + p), __ldg(oy + q), rc0)) {
            pass = true;
            frec = (uint32_t)tl | ((uint32_t)(q * n2x + p) << 5);
          }
        }
        const uint32_t fbal = __ballot_sync(FULL, pass);
        if (pass) {
          const uint32_t k = nfr + __popc(fbal & ((1u << lane) - 1u));
          ws.brec[k] = frec;
          ws.zown[k] = __float_as_uint(rc0.Tx);
          ws.fty[k] = rc0.Ty;
        }
        nfr += (uint32_t)__popc(fbal);
        __syncwarp();
        // every 32 records, and at the end of the batch (the records name its triangle slots)
        if (nfr < 32 && !(wb + 32 >= tot && nfr > 0)) continue;
        const uint32_t nr = min(nfr, 32u);
        if (lane < nr) {
          const uint32_t fr = ws.brec[lane];
          const int tl = (int)(fr & 31u);
          RayTri rt;
          rt.v1x = ws.v[tl][0]; rt.v1y = ws.v[tl][1]; rt.v1z = ws.v[tl][2];
          rt.e1x = ws.v[tl][3]; rt.e1y = ws.v[tl][4]; rt.e1z = ws.v[tl][5];
          rt.e2x = ws.v[tl][6]; rt.e2y = ws.v[tl][7]; rt.e2z = ws.v[tl][8];
          rt.inv_det = ws.x[tl][0];
          rt.ok = true;
          RayCol rc;
          rc.Tx = __uint_as_float(ws.zown[lane]);
          rc.Ty = ws.fty[lane];
          item_voxels(rt, rc, tl, (int)(fr >> 5));
        }
        __syncwarp();
        // move the records beyond the first nr to the front
        uint32_t m0 = 0, m1 = 0;
        float m2 = 0.f;
        if (lane + nr < nfr) { m0 = ws.brec[nr + lane]; m1 = ws.zown[nr + lane]; m2 = ws.fty[nr + lane]; }
        __syncwarp();
        if (lane + nr < nfr) { ws.brec[lane] = m0; ws.zown[lane] = m1; ws.fty[lane] = m2; }
        nfr -= nr;
        __syncwarp();
      }
    }
    __syncwarp();
  }

  }

  // ---------------- output, top voxel first so the full-hit toggles accumulate downwards.
  // One lane per sub-column: its n2z SAT and parity bits are read once and written as n2z
  // bytes at stride n2x*n2y (consecutive lanes write consecutive bytes of each z layer).
  for (int w = lane; w < FW; w += 32) ftacc[w] = 0;
  __syncwarp();
  unsigned long long nin = 0, nbd = 0;
  const uint32_t zmask_all = n2z >= 32 ? 0xffffffffu : ((1u << n2z) - 1u);
  // 16-byte stores where the layout allows them (also the fast pattern into pinned host memory);
  // measured faster with the queued organisation (torus262k: -6%) and slower with the per-lane
  // one on the mixed batch (+3%), so only the former uses them
  // packed codes for the host: the voxels of this launch's slab below BatchDev::pk_end (the host
  // enables it only where the 16-byte layout below applies)
  const uint32_t pkend = d.l2codes ? bd.pk_end[slab] : 0u;
  const bool vec = (QUEUE || pkend) && (n2z == 8 || n2z == 16) && (ncol2 & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(d.l2) & 15) == 0;
  for (int jv = m - 1; jv >= 0; --jv) {
    for (int w = lane; w < FW; w += 32) ftacc[w] ^= ft[jv * FW + w];
    __syncwarp();
    const int64_t vlin = ((int64_t)kz[jv] * ny + cj) * nx + ci;
    uint8_t *out = d.l2 + (size_t)d.prefix[vlin] * cells;
    const uint32_t vidx = (uint32_t)d.prefix[vlin];
    uint32_t *codes = vidx < pkend ? d.l2codes + (size_t)vidx * (cells >> 4) : nullptr;
    const uint32_t *satj = sat + jv * W, *parj = par + jv * W;
    if (vec) {
      if (n2z == 8) write_block_vec<8>(out, codes, satj, parj, ftacc, ncol2, lane, nbd, nin);
      else write_block_vec<16>(out, codes, satj, parj, ftacc, ncol2, lane, nbd, nin);
      __syncwarp();
      continue;
    }
    for (int pq = lane; pq < ncol2; pq += 32) {
      const int off = pq * n2z, sh = off & 31;
      uint32_t sb = satj[off >> 5] >> sh, pb = parj[off >> 5] >> sh;
      if (sh + n2z > 32) {
        sb |= satj[(off >> 5) + 1] << (32 - sh);
        pb |= parj[(off >> 5) + 1] << (32 - sh);
      }
      sb &= zmask_all;
      if ((ftacc[pq >> 5] >> (pq & 31)) & 1u) pb = ~pb;
      const uint32_t ib = pb & ~sb & zmask_all;
      nbd += (unsigned)__popc(sb);
      nin += (unsigned)__popc(ib);
      uint8_t *o = out + pq;
      for (int r = 0; r < n2z; ++r)
        __stcs(reinterpret_cast<char *>(o + (size_t)r * ncol2),
               (char)(((sb >> r) & 1u) ? 254 : (((ib >> r) & 1u) ? 127 : 0)));
    }
    __syncwarp();
  }
  nin = warp_sum(nin);
  nbd = warp_sum(nbd);
  nun = warp_sum(nun);
  if (lane == 0) {
    if (nin) atomicAdd(&d.stats->l2_inside, nin);
    if (nbd) atomicAdd(&d.stats->l2_boundary, nbd);
    if (nun) atomicAdd(&d.stats->ray2, (unsigned long long)nun * (unsigned long long)cells);
  }
  __syncwarp();
  }  // next item
}

}  // namespace

int level2_chunk(const GridDev &g, int cap) {
  const int cells = g.n2[0] * g.n2[1] * g.n2[2];
  const int W = (cells + 31) >> 5;
  return std::max(1, std::min(std::min(32, std::max(cap, 1)), kMaskWords / W));
}

// Shared-memory words one warp needs for a mesh with this grid.
int level2_warp_words(const GridDev &g, int cap, bool stencil) {
  const int cells = g.n2[0] * g.n2[1] * g.n2[2];
  const int W = (cells + 31) >> 5;
  const int FW = (g.n2[0] * g.n2[1] + 31) >> 5;
  const int CH = level2_chunk(g, cap);
  const int FWS = (4 * g.n2[0] * g.n2[1] + 31) >> 5;
  return 2 * CH * W + CH * FW + CH + FW + (int)(sizeof(WarpScratch) / 4) +
         (stencil ? 4 * CH * W + CH * FWS + FWS : 0);
}

// Measured on one GB300: the queued records win (3-10%) where the triangles span several Level2
// cells in x and y (xycells / pairs >= 4: torus262k at 8^3, a 16k sphere at 4^3); the per-lane
// slab work wins (10-16%) where they span about one (the same torus at 2^3 and 4^3), and on
// mixed batches.
bool level2_queue_pays(const MeshStats *stats, const bool *has_l2, int n) {
  double dense = 0.0, all = 0.0;
  for (int m = 0; m < n; ++m) {
    if (!has_l2[m]) continue;
    const double p = (double)stats[m].pairs;
    all += p;
    if ((double)stats[m].xycells >= 64.0 * p) dense += p;  // xycells carries a factor 16
  }
  // mixed launches do better with the per-lane organisation (the 4096-mesh mix: +3%)
  return dense > 0.9 * all;
}

size_t level2_smem_bytes(int warp_words) { return (size_t)warp_words * 4 * kWarps; }

int64_t level2_temp_words(int64_t B) { return 7 * B + 8 + 2 * (kSlabsMax + 4) + scan_temp_words(B); }

// Builds the chunk items from the sorted pair lists and runs the persistent Level2 kernel.
void launch_level2(const BatchDev &bd, const uint32_t *keys, const uint32_t *vals,
                   const uint32_t *useg, int64_t B, uint32_t *tmp, int warp_words, int num_sms,
                   cudaStream_t s, const std::function<void()> &before_kernel, int zslab,
                   int nslab, const std::function<void(int, cudaStream_t)> &after_slab, int slab_nz,
                   const SlabStreams *aux, bool queue, bool fillq) {
  if (B <= 0) return;
  uint32_t *cflag = tmp, *cord = cflag + B, *colhead = cord + B, *iflag = colhead + B + 1,
           *iord = iflag + B, *istart = iord + B, *nitems = istart + B + 1,
           *slabcnt = nitems + 4, *ioff = slabcnt + (kSlabsMax + 4), *ilist = ioff + (kSlabsMax + 4),
           *stmp = ilist + B;
  if (nslab <= 1) zslab = 0;
  const unsigned nb = (unsigned)((B + 255) / 256);
  // (one-graph calls: B is the capacity, the kernels read the device count)
  k_colflags<<<nb, 256, 0, s>>>(bd, keys, useg, B, cflag, nitems);
  scan_u32(cflag, cord, B, nullptr, stmp, s);
  k_colheads<<<nb, 256, 0, s>>>(bd, cflag, cord, B, colhead);
  k_itemflags<<<nb, 256, 0, s>>>(bd, keys, useg, cflag, cord, colhead, B, zslab, iflag);
  scan_u32(iflag, iord, B, nullptr, stmp, s);
  k_itemstarts<<<nb, 256, 0, s>>>(bd, iflag, iord, B, istart, nitems);
  count_launch(4);
  if (bd.fill == GPV_FILL_STENCIL && bd.stp) {
    const unsigned nbp = (unsigned)((B + kPrefixWarps - 1) / kPrefixWarps);  // items, columns <= B
    k_stencil_segment<<<nbp, kPrefixWarps * 32, 0, s>>>(bd, keys, vals, useg, cflag, cord, colhead,
                                                         istart, nitems, B);
    k_stencil_scan<<<nbp, kPrefixWarps * 32, 0, s>>>(bd, cflag, cord, colhead, iflag, B);
    count_launch(2);
  }
  const size_t smem = level2_smem_bytes(warp_words);
  const bool st = bd.fill == GPV_FILL_STENCIL;
  using Kern = decltype(&k_level2c<false, false, false>);
  static bool attr_set[6] = {false, false, false, false, false, false};
  // the kernel of one SAT organisation, and its persistent grid
  auto pick = [&](bool q, int64_t &grid) {
    Kern k = st ? (q ? k_level2c<true, true, false> : k_level2c<true, false, false>)
           : fillq ? (q ? k_level2c<false, true, true> : k_level2c<false, false, true>)
                   : (q ? k_level2c<false, true, false> : k_level2c<false, false, false>);
    const int kv = (st ? 4 : fillq ? 2 : 0) + (q ? 1 : 0);
    if (!attr_set[kv]) {
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      attr_set[kv] = true;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kWarps * 32, smem);
    per_sm = std::max(per_sm, 1);
    // (one-graph calls: B is a capacity, the queue ends the work)
    grid = bd.plan ? (int64_t)num_sms * per_sm
                   : std::min<int64_t>((B + kWarps - 1) / kWarps, (int64_t)num_sms * per_sm);
    return k;
  };
  int64_t grid = 0, grid2 = 0;
  const Kern kern = pick(queue, grid);
  // one-graph calls: the other organisation too; the device plan leaves one of them empty
  const Kern kern2 = bd.plan ? pick(!queue, grid2) : nullptr;
  const int nz = slab_nz;
  if (zslab > 0) {
    // single mesh: order the items by slab so that each launch takes only its own
    cudaMemsetAsync(slabcnt, 0, (kSlabsMax + 4) * sizeof(uint32_t), s);
    k_item_slab_count<<<nb, 256, 0, s>>>(istart, nitems, keys, useg, nz, zslab, slabcnt);
    k_item_slab_offsets<<<1, 32, 0, s>>>(slabcnt, nslab, ioff);
    k_item_slab_place<<<nb, 256, 0, s>>>(istart, nitems, keys, useg, nz, zslab, slabcnt, ilist);
    count_launch(3);
  }
  if (before_kernel) before_kernel();
  // one launch, or one per z slab over that slab's items; slab launches alternate between two
  // streams (when given) so that one slab's tail overlaps the next slab's start
  const int launches = zslab > 0 ? nslab : 1;
  const bool two = zslab > 0 && launches > 1 && aux;
  cudaMemsetAsync(bd.queue + 1, 0, (size_t)launches * sizeof(uint32_t), s);
  if (two) {
    cudaEventRecord(aux->fork, s);
    cudaStreamWaitEvent(aux->st[0], aux->fork, 0);
    cudaStreamWaitEvent(aux->st[1], aux->fork, 0);
  }
  for (int sl = 0; sl < launches; ++sl) {
    cudaStream_t ls = two ? aux->st[sl & 1] : s;
    kern<<<(unsigned)grid, kWarps * 32, smem, ls>>>(bd, keys, vals, useg, cflag, cord, colhead, istart,
                                                    nitems, warp_words, sl, zslab,
                                                    zslab > 0 ? ilist : nullptr, ioff);
    count_launch();
    if (kern2) {
      kern2<<<(unsigned)grid2, kWarps * 32, smem, ls>>>(bd, keys, vals, useg, cflag, cord, colhead,
                                                        istart, nitems, warp_words, sl, zslab,
                                                        zslab > 0 ? ilist : nullptr, ioff);
      count_launch();
    }
    if (after_slab) after_slab(sl, ls);
  }
  if (two) {
    cudaEventRecord(aux->join[0], aux->st[0]);
    cudaEventRecord(aux->join[1], aux->st[1]);
    cudaStreamWaitEvent(s, aux->join[0], 0);
    cudaStreamWaitEvent(s, aux->join[1], 0);
  }
}

}  // namespace gpv
