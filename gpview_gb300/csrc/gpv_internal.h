// gpv_internal.h -- declarations shared by the library's translation units (not installed).
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/gpview.h"
#include "gpv_common.cuh"

namespace gpv {

// ---- launch accounting: every kernel launch of the library bumps this counter ----------------
uint64_t launch_count();
void count_launch(uint64_t n = 1);

// ---- scan / sort (gpv_sort.cu) ---------------------------------------------------------------
int64_t scan_temp_words(int64_t n);
void scan_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *d_total, uint32_t *temp,
              cudaStream_t s);
int64_t sort_temp_words(int64_t n);
bool sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *kalt, uint32_t *valt, int64_t n,
                int key_bits, uint32_t *temp, cudaStream_t s);

// ---- host-side grid derivation (gpv_grid.cpp) ------------------------------------------------
struct GridHost {
  gpv_grid_spec spec;
  int n[3], n2[3];
  float g[3], e1[3], g2[3], e2[3];
  std::vector<float> c1[3], c2s[3], o2[3];
  std::vector<float> sp1;  // stencil fill: Level1 slice clip heights
  int64_t N1 = 0, cells = 0;
  int nxw = 0, nzw = 0, key_bits = 0;
  bool level2 = false;
  bool oz_monotone = false;
  float thr = 0.f;
};
// Derives sizes and coordinate tables exactly as the reference does (double then float).
// Level1 half extents may be given explicitly (the CUDAClassifyTessellation shim receives them).
int grid_derive(const gpv_grid_spec &spec, GridHost &out, const float *ext1_override = nullptr);
float eps_threshold();  // largest float below 1e-6

// ---- batched kernels (gpv_kernels.cu, gpv_level2.cu, gpv_sort.cu) -----------------------------
// Every kernel works on a batch of meshes described by a device array of MeshDesc; a work item
// (triangle, tile, row, pair tile, Level2 chunk) finds its mesh by binary search over the
// per-mesh prefix of that work kind.  The plain path is a batch of one.
struct MeshDesc {
  GridDev g;
  const float *tris;     // input float[T*9]
  float4 *ptri;          // packed triangles, 3 float4 per triangle (w: fill ranges, 1/det)
  int4 *rng;             // packed Level1 SAT candidate box per triangle
  float4 *fbox;          // conservative x/y box for the ray tests per triangle
  uint32_t *bplane;      // boundary bit plane (padded rows), slice of the batch plane
  uint32_t *iplane;      // inside (parity) bit plane, slice
  uint32_t *toggles;     // column-major parity toggles
  uint32_t *keys, *vals; // pair emission segment (capacity pair_cap)
  MeshStats *stats;
  uint8_t *l1;           // outputs
  int32_t *prefix;
  int32_t *bindex;
  uint8_t *l2;
  int64_t T, pair_cap;
  int64_t tri_base;      // prefix over meshes of triangles
  int64_t tile_base;     // ... of Level1 tiles
  int64_t fwarp_base;    // ... of fill-finish warps (ny * nxw * nzw)
  int64_t row_base;      // ... of Level1 rows (nz * ny)
  int64_t xc_base;       // ... of 128-voxel expansion chunks (ceil(N1 / 128))
  int64_t word_base;     // ... of bit-plane words (nz * ny * nxw)
  int64_t emit_base;     // ... of pair capacities (emission segments)
  int64_t pair_base;     // ... of pairs (dense layout after the sort)
  int64_t u_base;        // ... of boundary voxels
  int64_t stile_base;    // ... of pair-sort tiles (one-graph calls: set on the device by k_plan)
  int32_t ch;            // Level2 chunk length
  int32_t has_l2;        // the mesh has a Level2 grid
  float4 *fnorm;         // normals on: normalised face normal per triangle
  void *l1n, *l2n;       // normals on: Level1 / Level2 normal outputs (bytes or floats)
  uint32_t *stg;         // stencil fill: Level1 sample-column toggles, (2nx * 2ny) x nzw words
  // host outputs through packed codes (one mesh): the Level2 states as 2-bit codes (0 outside,
  // 1 inside, 2 boundary), 16 cells per word in output byte order, written here (device-mapped
  // page-locked staging) by the z slabs whose bit is set in BatchDev::packed_slabs; the host
  // expands them into the caller's bytes while later slabs compute
  uint32_t *l2codes;
};

// Sizes of the second half of a one-graph call (the whole voxelization recorded as one CUDA
// graph), computed on the device by k_plan from the first half's counts.  The second half's
// kernels are launched for capacities known when the graph is recorded and read these sizes;
// with ok = 0 (a size above its capacity, or a mesh status raised) they do nothing and the host
// re-runs the call with the exact sizes.
struct DevPlan {
  uint32_t ok;
  uint32_t qsel;     // Level2 SAT organisation: 1 queued records, 0 per lane
  uint32_t ub;       // boundary voxels of the meshes with a Level2 grid (the sorted segments)
  uint32_t ntiles;   // pair-sort tiles of those meshes
  unsigned long long P2;       // pairs of those meshes
  unsigned long long Btot;     // boundary voxels of all meshes
  unsigned long long l2bytes;  // Level2 output bytes
};

// BatchDev::fill value for Level1 SAT units only (no parity fill): the reference-named Level1
// shim, whose ClassifyTessellation marks boundary voxels and records their triangles.
constexpr int kFillNone = -1;

// z slabs of one Level2 launch sequence, at most (gpv_voxelize_to_host).  16 measured slower
// than 8 for the packed host transfer (star1310k host to host 6.58 against 6.43 ms): each slab
// launch adds its ramp and tail
constexpr int kSlabsMax = 8;

struct BatchDev {
  const MeshDesc *md;
  int nmesh;
  int tile;              // Level1 triangles per tile (32, 64, 128, 256)
  int64_t total_tris, total_tiles, total_fwarps, total_rows, total_words;
  int64_t total_xchunks;  // 128-voxel expansion chunks of all meshes
  uint32_t *queue;       // work-queue tickets, zeroed before each persistent launch
  int normals;           // GPV_NORMALS_* of this batch
  int fill;              // GPV_FILL_* of this batch
  uint32_t *stp;         // stencil fill: per boundary voxel, the sample-coverage parity of the
  int stp_words;         //   column's triangles recorded only below it (stp_words words each)
  // Level1 marks the voxel of every pair it emits for a mesh with a Level2 grid here: one
  // column-major bit plane per mesh (bit = pair key) at the mesh's word_base; nullptr: no marks
  uint32_t *kmask = nullptr;
  // Level1's bounded wait for its staged tile: polls before giving up (0: the built-in limit);
  // fail_wait != 0 gives up at once (GPV_DEBUG_FAIL_WAIT, failure-detection tests)
  uint32_t wait_limit = 0;
  int fail_wait = 0;
  // packed Level2 host output: in z slab k of the Level2 launch, the boundary voxels whose output
  // index is below pk_end[k] write MeshDesc::l2codes instead of bytes (the slab's first share)
  uint32_t pk_end[kSlabsMax] = {};
  // one-graph calls: the device-computed sizes of the second half (nullptr: sizes from the host)
  const DevPlan *plan = nullptr;
};

// Mesh owning work index idx: last m with md[m].*F <= idx (meshes with no work of this kind
// share their successor's base and are skipped).
template <int64_t MeshDesc::*F>
__device__ __forceinline__ int find_mesh(const MeshDesc *md, int nmesh, int64_t idx) {
  int lo = 0, hi = nmesh - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (md[mid].*F <= idx) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Small copies and clears around a phase, done by one kernel instead of copy-engine and memset
// nodes, so a recorded phase is kernels only.  Every address must be device-accessible: device
// memory, or page-locked host memory (cudaMallocHost), which unified addressing maps at the same
// address.  The operations of one list run concurrently: none may read what another writes.
// Sizes that are not a multiple of 4 bytes go to cudaMemcpyAsync / cudaMemsetAsync instead.
struct StageOp {
  const uint32_t *src;  // nullptr: clear dst
  uint32_t *dst;
  int64_t words;
};
struct StageOps {
  static constexpr int kMax = 8;
  StageOp op[kMax];
  int n;
};
class StageList {
 public:
  StageList(int num_sms, cudaStream_t s) : sms_(num_sms), s_(s) { ops_.n = 0; }
  void copy(void *dst, const void *src, size_t bytes) { add(dst, src, bytes); }
  void clear(void *dst, size_t bytes) { add(dst, nullptr, bytes); }
  void launch();  // runs the queued operations (one kernel) and empties the list

 private:
  void add(void *dst, const void *src, size_t bytes);
  StageOps ops_;
  int sms_;
  cudaStream_t s_;
};

void launch_prep(const BatchDev &bd, cudaStream_t s);
// Boundary rank at each z-slab start of a single mesh (nslab + 1 values into out).
void launch_slab_offsets(const uint32_t *wpre, const uint32_t *wtot, int64_t words_per_layer,
                         int nz, int zslab, int nslab, uint32_t *out, cudaStream_t s);
// One-graph calls: from the first half's per-mesh counts, the per-mesh bases of the second half
// (u_base, pair_base, stile_base, and the bindex and l2 slices of the given result arenas) and
// the DevPlan, checked against the capacities the second half was recorded with.  level2_mode is
// GPV_LEVEL2_*; the automatic choice is the host's level2_queue_pays, evaluated on the device.
struct PlanCaps { int64_t B, U, l2bytes, tiles, P; };  // boundary, sorted, Level2 bytes, tiles, pairs
void launch_plan(const BatchDev &bd, MeshDesc *d_md, int32_t *bindex, uint8_t *l2,
                 const PlanCaps &caps, int level2_mode, DevPlan *plan, cudaStream_t s);
// Device-side per-mesh pair segments (emit_base, pair_cap, keys, vals) from prep's sat1 counts.
void launch_pair_bases(const BatchDev &bd, MeshDesc *d_md, uint32_t *keys, uint32_t *vals,
                       int64_t cap, cudaStream_t s);
void launch_level1(const BatchDev &bd, int num_sms, cudaStream_t s);
void launch_fill_finish(const BatchDev &bd, cudaStream_t s);
// Stencil fill, Level1 (gpv_stencil.cu): per-sample-column slice toggles of every triangle into
// MeshDesc::stg (zeroed by the caller); launch_fill_finish then reduces them.
void launch_stencil1(const BatchDev &bd, cudaStream_t s);
void launch_popc(const uint32_t *plane, int64_t nwords, uint32_t *cnt, cudaStream_t s);
void launch_boundary_counts(const BatchDev &bd, const uint32_t *wpre, const uint32_t *wtotal,
                            cudaStream_t s);
void launch_expand(const BatchDev &bd, const uint32_t *wpre, cudaStream_t s);
void launch_heads(const uint32_t *keys, int64_t P, uint32_t *flags, const BatchDev &bd,
                  cudaStream_t s);
void launch_useg(const uint32_t *flags, const uint32_t *uidx, int64_t P, uint32_t *useg,
                 cudaStream_t s);

// segmented radix sort: per mesh the pairs [in_base, in_base + P_m) end dense at pair_base
struct SortTile { int32_t mesh, j, count, pad; };
int64_t sort_seg_temp_words(int64_t ntiles);
// Returns true when the sorted data ended in (kalt, valt).  tiles[] (device) lists the tiles of
// every mesh; hist_base[m] = 256 * (tiles before mesh m) (device).
// Counting sort of the emitted pairs by voxel, for lists whose triangle order does not matter
// (no normals): the rank of a pair's voxel among the marked voxels in key order comes from
// bd.kmask and its exclusive word prefix kpre (global over all meshes: kpre[0] is subtracted), so
// one count, one scan and one scatter give the dense (kout, vout) lists and the segment starts
// useg[0..nseg] directly.  done receives the number of voxels whose last pair was placed (nseg
// when the marks and the pairs agree); cnt (nseg words) must be zero and is left zero.
// One-graph calls (tiles == nullptr, bd.plan set): the tiles and sizes come from the device
// plan; ntiles and nseg are capacities, and cnt holds nseg + 1 zero words.
void count_sort_pairs(const BatchDev &bd, const SortTile *tiles, int64_t ntiles,
                      const uint32_t *keys, const uint32_t *vals, const uint32_t *kpre,
                      int64_t nseg, int64_t P, uint32_t *cnt, uint32_t *useg, uint32_t *kout,
                      uint32_t *vout, uint32_t *done, uint32_t *temp, cudaStream_t s);
bool sort_pairs_seg(const BatchDev &bd, const SortTile *tiles, const int64_t *tile_base_dev,
                    int64_t ntiles, uint32_t *keys, uint32_t *vals, uint32_t *kalt, uint32_t *valt,
                    int64_t Ptotal, int key_bits, int val_bits, uint32_t *temp, cudaStream_t s);
constexpr int kSortTileItems = 2048;

int level2_chunk(const GridDev &g, int cap = 32);
int level2_warp_words(const GridDev &g, int cap = 32, bool stencil = false);
int64_t level2_temp_words(int64_t Btot);
// before_kernel (optional) runs on the host between the work-item launches and the Level2
// kernel's launch, e.g. to record an event that times the kernel alone.
// With zslab > 0 and nslab > 1 the Level2 kernel runs once per slab of zslab Level1 layers (one
// mesh with slab_nz Level1 layers): the outputs of slab k are contiguous and complete after the
// work after_slab(k, stream) sees on `stream`, so a copy of them can start while the next slab
// computes.  With aux, slab launches alternate between aux's two streams (joined back into s).
struct SlabStreams {  // two streams and their events for overlapping slab launches
  cudaStream_t st[2];
  cudaEvent_t fork, join[2];
};
void launch_level2(const BatchDev &bd, const uint32_t *keys, const uint32_t *vals,
                   const uint32_t *useg, int64_t Btot, uint32_t *tmp, int warp_words, int num_sms,
                   cudaStream_t s, const std::function<void()> &before_kernel = {}, int zslab = 0,
                   int nslab = 1, const std::function<void(int, cudaStream_t)> &after_slab = {},
                   int slab_nz = 0, const SlabStreams *aux = nullptr, bool queue = true,
                   bool fillq = false);
// Level2 SAT organisation for a batch (see k_level2c): queued records when most of the pair work
// belongs to meshes whose pairs carry many (triangle, sub-column) items.
bool level2_queue_pays(const MeshStats *stats, const bool *has_l2, int n);
// Level2 ray-fill organisation: the u/v-passing items queued before their per-voxel work when
// every Level2 grid of the launch has at most kFillQueueCells cells.
constexpr int kFillQueueCells = 512;

// ---- normals (gpv_normals.cu) ----------------------------------------------------------------
void launch_face_normals(const BatchDev &bd, cudaStream_t s);
// Level1 normals of the U boundary voxels of the sorted meshes, then (any_l2) Level2 normals.
void launch_normals(const BatchDev &bd, const uint32_t *keys, const uint32_t *vals,
                    const uint32_t *useg, int64_t U, bool any_l2, int num_sms, cudaStream_t s);

// ---- voxel box hierarchy (gpv_hierarchy.cu) ----------------------------------------------------
int hierarchy_levels(int64_t N1);  // 0 unless N1 is a power of two >= 2
void launch_hierarchy(const GridDev &g, const uint32_t *iplane, gpv_box *out, cudaStream_t s);

GridDev make_griddev(const GridHost &gh, const float *dtables);
int64_t table_floats(const GridHost &gh);
void pack_tables(const GridHost &gh, float *host);

}  // namespace gpv
