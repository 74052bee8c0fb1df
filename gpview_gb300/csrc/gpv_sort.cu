// gpv_sort.cu -- hand-written device scan and LSD radix sort used to build the per-voxel
// triangle lists (the reference builds them on the host, src/Object.cpp:2146-2180, and
// compacts boundary voxels there too, :3271-3279).
//
// scan_u32:  reduce-then-scan, no inter-block waiting: tile sums, then a down-sweep in which every
//            block adds up the sums of the tiles before it (up to 1024 tiles; beyond that a
//            separate single-block scan of the tile sums runs in between).
// sort_pairs: stable LSD radix sort of (u32 key, u32 value), 8-bit digits; per pass a tile
//             histogram, a scan of the digit-major histogram, and a stable scatter whose
//             in-tile ranks come from __match_any_sync peer masks.
#include <algorithm>
#include <atomic>

#include "gpv_internal.h"

namespace gpv {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= (unsigned)d) v += o;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; the block total goes to `total`.
template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t &total) {
  __shared__ uint32_t s_w[NT / 32];
  __shared__ uint32_t s_total;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t inc = warp_incl_scan(v);
  if (lane == 31) s_w[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < NT / 32 ? s_w[lane] : 0u;
    const uint32_t wi = warp_incl_scan(w);
    if (lane < NT / 32) s_w[lane] = wi - w;
    if (lane == 31) s_total = wi;
  }
  __syncthreads();
  const uint32_t r = s_w[warp] + inc - v;
  total = s_total;
  __syncthreads();
  return r;
}

__global__ void k_scan_reduce(const uint32_t *__restrict__ in, int64_t n,
                              uint32_t *__restrict__ part) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint32_t tot;
  block_excl_scan<kScanThreads>(s, tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Single block: exclusive scan of the partials in place; total to *total.
__global__ void k_scan_partials(uint32_t *__restrict__ part, int64_t nb,
                                uint32_t *__restrict__ total) {
  uint32_t carry = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
    int64_t i = b0 + threadIdx.x;
    uint32_t v = i < nb ? part[i] : 0u;
    uint32_t tot;
    uint32_t ex = block_excl_scan<1024>(v, tot);
    if (i < nb) part[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_down(const uint32_t *__restrict__ in, int64_t n,
                            const uint32_t *__restrict__ part, uint32_t *__restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  // blocked arrangement: thread owns kScanItems consecutive items
  uint32_t v[kScanItems];
  uint32_t s = 0;
  const int64_t tb = base + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = tb + k;
    v[k] = i < n ? in[i] : 0u;
    s += v[k];
  }
  uint32_t tot;
  uint32_t ex = block_excl_scan<kScanThreads>(s, tot) + part[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = tb + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
}

// Down-sweep that also finds its own tile offset: the sum of the partials of the tiles before it
// (for up to kFusedTiles tiles, where that sum is cheap), so the partials need no separate scan.
constexpr int64_t kFusedTiles = 1024;

__global__ void k_scan_down_fused(const uint32_t *__restrict__ in, int64_t n,
                                  const uint32_t *__restrict__ part, uint32_t *__restrict__ out,
                                  uint32_t *__restrict__ total) {
  __shared__ uint32_t s_base;
  uint32_t acc = 0;
  for (int64_t k = threadIdx.x; k < blockIdx.x; k += kScanThreads) acc += part[k];
  uint32_t sum;
  block_excl_scan<kScanThreads>(acc, sum);
  if (threadIdx.x == 0) s_base = sum;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t v[kScanItems];
  uint32_t s = 0;
  const int64_t tb = base + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = tb + k;
    v[k] = i < n ? in[i] : 0u;
    s += v[k];
  }
  uint32_t tot;
  uint32_t ex = block_excl_scan<kScanThreads>(s, tot) + s_base;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = tb + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total = s_base + tot;
}

// ---- radix sort ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;

__global__ void k_radix_hist(const uint32_t *__restrict__ keys, int64_t n, int shift,
                             uint32_t *__restrict__ hist, int64_t nb) {
  __shared__ uint32_t s_h[256];
  s_h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortRounds; ++r) {
    int64_t i = base + (int64_t)r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&s_h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nb + blockIdx.x] = s_h[threadIdx.x];
}

__global__ void k_radix_scatter(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                                int64_t n, int shift, const uint32_t *__restrict__ hoff, int64_t nb,
                                uint32_t *__restrict__ kout, uint32_t *__restrict__ vout) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_run[256];
  __shared__ uint16_t s_w[kSortThreads / 32][256];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  s_off[threadIdx.x] = hoff[(int64_t)threadIdx.x * nb + blockIdx.x];
  s_run[threadIdx.x] = 0;
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortRounds; ++r) {
    if (base + (int64_t)r * kSortThreads >= n) break;  // block-uniform
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) s_w[w][threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = base + (int64_t)r * kSortThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t key = 0, val = 0, digit = 256u;
    if (valid) {
      key = keys[i];
      val = vals[i];
      digit = (key >> shift) & 255u;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const unsigned rank = __popc(peers & lt_mask);
    if (valid && rank == 0) s_w[warp][digit] = (uint16_t)__popc(peers);
    __syncthreads();
    uint32_t acc = 0;
    {
      const unsigned d = threadIdx.x;
#pragma unroll
      for (int w = 0; w < kSortThreads / 32; ++w) {
        uint32_t c = s_w[w][d];
        s_w[w][d] = (uint16_t)acc;
        acc += c;
      }
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_off[digit] + s_run[digit] + s_w[warp][digit] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    s_run[threadIdx.x] += acc;
    __syncthreads();
  }
}

// ---- segmented variant: one block per SortTile (mesh m, tile j of that mesh) -----------------
// hist layout per mesh m: [256 digits][ntiles_m tiles] starting at 256 * tile_base[m], so one
// exclusive scan over the whole array yields dense, mesh-major output positions.
__device__ __forceinline__ int64_t seg_in_base(const MeshDesc &d, bool emit) {
  return emit ? d.emit_base : d.pair_base;
}

// by_val: the digit comes from the value's triangle id (bit 31, the topmost flag, excluded)
// instead of the key; value passes run before the key passes to order each voxel's triangles.
__device__ __forceinline__ uint32_t seg_digit(uint32_t key, uint32_t val, bool by_val, int shift) {
  return ((by_val ? (val & 0x7fffffffu) : key) >> shift) & 255u;
}

__global__ void k_radix_hist_seg(const MeshDesc *__restrict__ md, const SortTile *__restrict__ tiles,
                                 const int64_t *__restrict__ tb, const uint32_t *__restrict__ keys,
                                 const uint32_t *__restrict__ vals, bool by_val, bool emit,
                                 int shift, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_h[256];
  s_h[threadIdx.x] = 0;
  __syncthreads();
  const SortTile st = tiles[blockIdx.x];
  const int64_t in0 = seg_in_base(md[st.mesh], emit) + (int64_t)st.j * kSortTile;
  for (int r = 0; r < kSortRounds; ++r) {
    const int i = r * kSortThreads + threadIdx.x;
    if (i < st.count)
      atomicAdd(&s_h[by_val ? seg_digit(0u, vals[in0 + i], true, shift)
                            : seg_digit(keys[in0 + i], 0u, false, shift)], 1u);
  }
  __syncthreads();
  const int64_t nt_m = tb[st.mesh + 1] - tb[st.mesh];
  hist[256 * tb[st.mesh] + (int64_t)threadIdx.x * nt_m + st.j] = s_h[threadIdx.x];
}

__global__ void k_radix_scatter_seg(const MeshDesc *__restrict__ md,
                                    const SortTile *__restrict__ tiles,
                                    const int64_t *__restrict__ tb, const uint32_t *__restrict__ keys,
                                    const uint32_t *__restrict__ vals, bool by_val, bool emit,
                                    int shift, const uint32_t *__restrict__ hoff,
                                    uint32_t *__restrict__ kout,
                                    uint32_t *__restrict__ vout) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_run[256];
  __shared__ uint16_t s_w[kSortThreads / 32][256];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const SortTile st = tiles[blockIdx.x];
  const int64_t nt_m = tb[st.mesh + 1] - tb[st.mesh];
  s_off[threadIdx.x] = hoff[256 * tb[st.mesh] + (int64_t)threadIdx.x * nt_m + st.j];
  s_run[threadIdx.x] = 0;
  const int64_t in0 = seg_in_base(md[st.mesh], emit) + (int64_t)st.j * kSortTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortRounds; ++r) {
    if (r * kSortThreads >= st.count) break;  // block-uniform
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) s_w[w][threadIdx.x] = 0;
    __syncthreads();
    const int i = r * kSortThreads + threadIdx.x;
    const bool valid = i < st.count;
    uint32_t key = 0, val = 0, digit = 256u;
    if (valid) {
      key = keys[in0 + i];
      val = vals[in0 + i];
      digit = seg_digit(key, val, by_val, shift);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const unsigned rank = __popc(peers & lt_mask);
    if (valid && rank == 0) s_w[warp][digit] = (uint16_t)__popc(peers);
    __syncthreads();
    uint32_t acc = 0;
    {
      const unsigned d = threadIdx.x;
#pragma unroll
      for (int w = 0; w < kSortThreads / 32; ++w) {
        uint32_t c = s_w[w][d];
        s_w[w][d] = (uint16_t)acc;
        acc += c;
      }
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_off[digit] + s_run[digit] + s_w[warp][digit] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    s_run[threadIdx.x] += acc;
    __syncthreads();
  }
}

}  // namespace

namespace {
std::atomic<uint64_t> g_launches{0};
}
uint64_t launch_count() { return g_launches.load(); }
void count_launch(uint64_t n) { g_launches.fetch_add(n); }

int64_t scan_temp_words(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

void scan_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *d_total, uint32_t *temp,
              cudaStream_t s) {
  if (n <= 0) {
    if (d_total) cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s);
    return;
  }
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, temp);
  if (nb <= kFusedTiles) {
    k_scan_down_fused<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, temp, out, d_total);
    count_launch(2);
    return;
  }
  k_scan_partials<<<1, 1024, 0, s>>>(temp, nb, d_total);
  k_scan_down<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, temp, out);
  count_launch(3);
}

int64_t sort_temp_words(int64_t n) {
  const int64_t nb = (n + kSortTile - 1) / kSortTile;
  return 2 * 256 * nb + scan_temp_words(256 * nb);
}

// Sorts (keys, vals) by the low key_bits bits.  Ping-pongs with (kalt, valt); returns true when
// the sorted data ended in (kalt, valt).
bool sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *kalt, uint32_t *valt, int64_t n,
                int key_bits, uint32_t *temp, cudaStream_t s) {
  if (n <= 1) return false;
  const int64_t nb = (n + kSortTile - 1) / kSortTile;
  uint32_t *hist = temp;
  uint32_t *hoff = temp + 256 * nb;
  uint32_t *stmp = temp + 2 * 256 * nb;
  bool alt = false;
  for (int shift = 0; shift < key_bits; shift += 8) {
    const uint32_t *ki = alt ? kalt : keys;
    const uint32_t *vi = alt ? valt : vals;
    uint32_t *ko = alt ? keys : kalt;
    uint32_t *vo = alt ? vals : valt;
    k_radix_hist<<<(unsigned)nb, kSortThreads, 0, s>>>(ki, n, shift, hist, nb);
    scan_u32(hist, hoff, 256 * nb, nullptr, stmp, s);
    k_radix_scatter<<<(unsigned)nb, kSortThreads, 0, s>>>(ki, vi, n, shift, hoff, nb, ko, vo);
    count_launch(2);
    alt = !alt;
  }
  return alt;
}

}  // namespace gpv

namespace gpv {

int64_t sort_seg_temp_words(int64_t ntiles) {
  return 2 * 256 * ntiles + scan_temp_words(256 * ntiles) + 4;
}

// ---- counting sort by voxel (lists without triangle order) -----------------------------------
// Rank of a pair's voxel among the marked voxels of all meshes in key order; nseg past the end
// when the marks do not hold the key (a broken invariant: the pair is then skipped).
__device__ __forceinline__ uint32_t cs_rank(const BatchDev &bd, const MeshDesc &d,
                                            const uint32_t *__restrict__ kpre, uint32_t key,
                                            int64_t nseg) {
  const int64_t w = d.word_base + (key >> 5);
  const uint32_t word = bd.kmask[w], bit = 1u << (key & 31u);
  if (!(word & bit)) return (uint32_t)nseg;
  return kpre[w] - kpre[0] + __popc(word & (bit - 1u));
}

// The block's pair tile: from the host's list, or (one-graph calls, tiles == nullptr) from the
// device plan: the mesh by its sort-tile base, the count from its pairs.  False: no tile (the
// grid was launched for the capacity, or the plan did not fit).
__device__ __forceinline__ bool cs_tile(const BatchDev &bd, const SortTile *tiles, SortTile &st) {
  if (tiles) {
    st = tiles[blockIdx.x];
    return true;
  }
  if (!bd.plan->ok || blockIdx.x >= bd.plan->ntiles) return false;
  const int m = find_mesh<&MeshDesc::stile_base>(bd.md, bd.nmesh, (int64_t)blockIdx.x);
  const int64_t j = (int64_t)blockIdx.x - bd.md[m].stile_base;
  st.mesh = m;
  st.j = (int32_t)j;
  st.count = (int32_t)min((int64_t)kSortTile, (int64_t)bd.md[m].stats->pairs - j * kSortTile);
  return true;
}

__global__ void __launch_bounds__(kSortThreads) k_cs_count(BatchDev bd,
                                                           const SortTile *__restrict__ tiles,
                                                           const uint32_t *__restrict__ keys,
                                                           const uint32_t *__restrict__ kpre,
                                                           int64_t nseg, uint32_t *__restrict__ cnt) {
  SortTile st;
  if (!cs_tile(bd, tiles, st)) return;
  if (bd.plan) nseg = bd.plan->ub;
  const MeshDesc &d = bd.md[st.mesh];
  const int64_t in0 = d.emit_base + (int64_t)st.j * kSortTile;
  for (int i = threadIdx.x; i < st.count; i += kSortThreads) {
    const uint32_t g = cs_rank(bd, d, kpre, keys[in0 + i], nseg);
    if (g < nseg) atomicAdd(cnt + g, 1u);
  }
}

// Places each pair at its voxel's segment start + (pairs of the voxel still unplaced - 1), so the
// counts return to zero; counts the voxels whose last pair this block placed.
__global__ void __launch_bounds__(kSortThreads) k_cs_scatter(
    BatchDev bd, const SortTile *__restrict__ tiles, const uint32_t *__restrict__ keys,
    const uint32_t *__restrict__ vals, const uint32_t *__restrict__ kpre, int64_t nseg, int64_t P,
    uint32_t *__restrict__ cnt, const uint32_t *__restrict__ useg, uint32_t *__restrict__ kout,
    uint32_t *__restrict__ vout, uint32_t *__restrict__ done) {
  __shared__ uint32_t s_done;
  SortTile st;
  if (!cs_tile(bd, tiles, st)) return;
  if (bd.plan) {
    nseg = bd.plan->ub;
    P = (int64_t)bd.plan->P2;
  }
  if (threadIdx.x == 0) s_done = 0;
  __syncthreads();
  const MeshDesc &d = bd.md[st.mesh];
  const int64_t in0 = d.emit_base + (int64_t)st.j * kSortTile;
  uint32_t fin = 0;
  for (int i = threadIdx.x; i < st.count; i += kSortThreads) {
    const uint32_t key = keys[in0 + i];
    const uint32_t g = cs_rank(bd, d, kpre, key, nseg);
    if (g >= nseg) continue;
    const uint32_t left = atomicSub(cnt + g, 1u);
    const int64_t pos = (int64_t)useg[g] + left - 1;
    if (left == 0 || pos >= P) continue;
    kout[pos] = key;
    vout[pos] = vals[in0 + i];
    fin += left == 1u;
  }
  fin = __reduce_add_sync(0xffffffffu, fin);
  if ((threadIdx.x & 31u) == 0 && fin) atomicAdd(&s_done, fin);
  __syncthreads();
  if (threadIdx.x == 0 && s_done) atomicAdd(done, s_done);
}

bool sort_pairs_seg(const BatchDev &bd, const SortTile *tiles, const int64_t *tile_base_dev,
                    int64_t ntiles, uint32_t *keys, uint32_t *vals, uint32_t *kalt, uint32_t *valt,
                    int64_t Ptotal, int key_bits, int val_bits, uint32_t *temp, cudaStream_t s) {
  static_assert(kSortTileItems == kSortTile, "tile size mismatch");
  if (Ptotal <= 0 || ntiles <= 0) return false;
  uint32_t *hist = temp;
  uint32_t *hoff = temp + 256 * ntiles;
  uint32_t *stmp = temp + 2 * 256 * ntiles;
  // Pass 0 always runs (it also moves the pairs from the emission segments to the dense
  // layout), so the result lands in (kalt, valt) after an odd number of passes.  Value passes
  // (triangle id digits) come first, so the stable key passes leave each key's triangles in
  // ascending order.
  const int vpasses = val_bits > 0 ? (val_bits + 7) / 8 : 0;
  const int kpasses = std::max(vpasses > 0 ? 0 : 1, (key_bits + 7) / 8);
  bool alt = false;
  for (int ps = 0; ps < vpasses + kpasses; ++ps) {
    const bool by_val = ps < vpasses;
    const int shift = 8 * (by_val ? ps : ps - vpasses);
    const bool emit = ps == 0;
    const uint32_t *ki = alt ? kalt : keys;
    const uint32_t *vi = alt ? valt : vals;
    uint32_t *ko = alt ? keys : kalt;
    uint32_t *vo = alt ? vals : valt;
    k_radix_hist_seg<<<(unsigned)ntiles, kSortThreads, 0, s>>>(bd.md, tiles, tile_base_dev, ki, vi,
                                                                by_val, emit, shift, hist);
    scan_u32(hist, hoff, 256 * ntiles, nullptr, stmp, s);
    k_radix_scatter_seg<<<(unsigned)ntiles, kSortThreads, 0, s>>>(
        bd.md, tiles, tile_base_dev, ki, vi, by_val, emit, shift, hoff, ko, vo);
    count_launch(2);
    alt = !alt;
  }
  return alt;
}

void count_sort_pairs(const BatchDev &bd, const SortTile *tiles, int64_t ntiles,
                      const uint32_t *keys, const uint32_t *vals, const uint32_t *kpre,
                      int64_t nseg, int64_t P, uint32_t *cnt, uint32_t *useg, uint32_t *kout,
                      uint32_t *vout, uint32_t *done, uint32_t *temp, cudaStream_t s) {
  if (P <= 0 || ntiles <= 0 || nseg <= 0) return;
  k_cs_count<<<(unsigned)ntiles, kSortThreads, 0, s>>>(bd, tiles, keys, kpre, nseg, cnt);
  // one-graph calls: nseg is the capacity and the counts past the device's segment count are
  // zero (cleared, never counted), so the scan of nseg + 1 counts puts the total at useg[ub]
  if (bd.plan) scan_u32(cnt, useg, nseg + 1, nullptr, temp, s);
  else scan_u32(cnt, useg, nseg, useg + nseg, temp, s);
  k_cs_scatter<<<(unsigned)ntiles, kSortThreads, 0, s>>>(bd, tiles, keys, vals, kpre, nseg, P, cnt,
                                                          useg, kout, vout, done);
  count_launch(2);
}

}  // namespace gpv
