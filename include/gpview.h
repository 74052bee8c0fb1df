/*
 * gpview.h -- C ABI of the GB300-native two-level voxelizer (libgpview.so).
 *
 * Two groups of entry points:
 *
 *  1. Reference-named shims.  Same names, signatures and "1 on success" return as the CUDA
 *     wrappers GPView's Object class binds (includes/CUDAUtilities.h:63-64, :87-89).  All pointers
 *     are DEVICE pointers owned by the caller; launches go to the legacy default stream, as in
 *     the reference.  A reference-shaped caller relinks against this library unchanged.
 *
 *  2. The native API (gpv_*).  Plain pointers and sizes, an int status (0 = GPV_OK, negative =
 *     error), an explicit cudaStream_t, a context that owns a stream-ordered device pool.  The
 *     voxelization contract is the reference's CPU path: every Level1/Level2 state equals what
 *     ClassifyInOutCPU + ClassifyTessellation + ClassifyInOutLevel2CPU + ClassifyTessellationLevel2
 *     (src/Object.cpp) produce on the same triangles and grid, bit for bit.
 *
 * One context per host thread.  Device-side failures are reported through status words read
 * back by the host, never by a trap.
 */
#ifndef GPVIEW_H
#define GPVIEW_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h> /* cudaStream_t */
#include <vector_types.h>     /* float3, int3: the reference shim signatures use them by value */

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define GPV_OK 0
#define GPV_ERR_INVALID (-1)  /* bad argument or grid */
#define GPV_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define GPV_ERR_OOM (-3)      /* device or host allocation refused */
#define GPV_ERR_IO (-4)       /* file could not be opened / written */
#define GPV_ERR_PARSE (-5)    /* malformed .obj / .off */
#define GPV_ERR_DEVICE (-6)   /* a kernel raised its error status word (bounded wait expired) */
#define GPV_ERR_BUDGET (-7)   /* request exceeds the serving memory budget */
#define GPV_ERR_PENDING (-8)  /* serving: result not ready yet */
#define GPV_ERR_NOTFOUND (-9) /* serving: unknown ticket */

typedef struct gpv_ctx gpv_ctx;

/* Grid of one voxelization.  bbox_min/bbox_max play the role of Object::bBoxMin/bBoxMax
 * (includes/Object.h:95-96): Level1 cell sizes are float((max-min)/(n*1.0)) and every centre
 * and ray origin follows the reference's formulas (src/Object.cpp:3108-3130, :743-745,
 * :1132-1160, :2329-2331, :2389-2391).  ndiv2 = {0,0,0} disables Level2. */
typedef struct {
    float bbox_min[3];
    float bbox_max[3];
    int32_t ndiv[3];
    int32_t ndiv2[3];
} gpv_grid_spec;

/* Algorithmic work of one voxelization, counted from the reference's own algorithm:
 *   sat1 = sum over triangles of the Level1 candidate box size   (src/Object.cpp:2309-2325)
 *   sat2 = sum over boundary voxels of |tris(b)| * n2^3          (src/Object.cpp:2374-2398)
 *   ray1 = sum over triangles of (columns whose centre lies in the triangle's x/y box) * nz
 *   ray2 = sum over boundary voxels of |column union(b)| * n2^3  (src/Object.cpp:1162-1193)
 * ray1 counts the candidate pairs a column-binned fill must test; the reference's brute force
 * (every voxel against every triangle) is not counted. */
typedef struct {
    int64_t sat1, sat2, ray1, ray2;
} gpv_work;

/* Result of one voxelization.  Device arrays are owned by the context until
 * gpv_result_release().  State bytes are the reference's .raw encoding uint8(state*127):
 * 0 = outside, 127 = inside, 254 = boundary (src/Object.cpp:3031). */
typedef struct {
    gpv_grid_spec spec;
    float grid_size[3];
    float grid_size2[3];
    int64_t num_level1;          /* nx*ny*nz */
    int64_t num_boundary;        /* Level1 boundary voxels (B) */
    int64_t num_level1_inside;   /* Level1 voxels with state 1 */
    int64_t num_level2_inside;   /* Level2 cells with state 1 */
    int64_t num_level2_boundary; /* Level2 cells with state 2 */
    int64_t num_pairs;           /* (Level1 voxel, triangle) records */
    gpv_work work;
    uint8_t *level1_inout;       /* device, num_level1 bytes, x fastest */
    int32_t *level1_prefix;      /* device, num_level1 int32: boundaryPrefixSum */
    int32_t *boundary_index;     /* device, num_boundary int32: boundaryIndex */
    uint8_t *level2_inout;       /* device, num_boundary * n2x*n2y*n2z bytes */
    uint64_t handle;             /* internal */
    /* Normals (gpv_set_normals; NULL when off).  Three values per Level1 voxel (x fastest) and
     * per Level2 cell (boundary order, cell order as level2_inout): bytes in the .raw encoding
     * uint8(n * float(256/3) + 127) (src/Object.cpp:2940-2941, :3033-3035) or floats. */
    void *level1_normal;         /* device, 3 * num_level1 values */
    void *level2_normal;         /* device, 3 * num_boundary * n2x*n2y*n2z values */
    int32_t normal_mode;         /* GPV_NORMALS_* the result was made with */
    int32_t hierarchy_levels;    /* gpv_set_hierarchy: levels of `hierarchy`, else 0 */
    struct gpv_box *hierarchy;   /* device, num_level1 - 1 boxes, or NULL */
} gpv_result;

/* One node of the voxel box hierarchy (BBoxData fields used by Object::BuildHierarchy,
 * includes/Utilities.h:57-77): centre, half size, solid flag, the two children's indices and its
 * own index.  Level-1 children index the Level1 voxels (x fastest); later levels index nodes. */
typedef struct gpv_box {
    float mid[3];
    float half[3];
    int32_t solid, child1, child2, index;
} gpv_box;

/* A triangle soup on the host, as Object::CreateFlatTriangleData builds it
 * (src/Object.cpp:3496-3527): float[num_triangles*9], vertex-major, file face order.
 * bbox_min/bbox_max are the loader's bounds padded by 0.001*|max-min| (src/Object.cpp:572-583). */
typedef struct {
    float *tris;
    int64_t num_triangles;
    float bbox_min[3];
    float bbox_max[3];
    float max_model_size;
} gpv_mesh;

/* ---- context ------------------------------------------------------------------------------ */
int gpv_init(int device, gpv_ctx **out);
void gpv_destroy(gpv_ctx *ctx);
const char *gpv_last_error(gpv_ctx *ctx);
/* Tunables (autotuner output): triangles per Level1 tile (32..256, power of two; 0, the default,
 * picks per call the largest tile that still gives every SM three tiles) and the largest number
 * of boundary voxels of one Level1 column that one Level2 work item takes (1..32, default 16). */
int gpv_set_tile(gpv_ctx *ctx, int tris_per_tile);
int gpv_set_level2_chunk(gpv_ctx *ctx, int max_voxels);
/* Organisation of the Level2 kernel's SAT stage (results are identical; only speed differs):
 * GPV_LEVEL2_AUTO (default) picks per launch from the item density the prep kernel measures;
 * GPV_LEVEL2_QUEUED queues the (triangle, sub-column) items that pass the z-invariant axes and
 * finishes them 32 at a time; GPV_LEVEL2_INLINE lets each item's lane finish its own item. */
#define GPV_LEVEL2_AUTO 0
#define GPV_LEVEL2_QUEUED 1
#define GPV_LEVEL2_INLINE 2
int gpv_set_level2_mode(gpv_ctx *ctx, int mode);
/* Voxel normals (default off), the reference's Level1 and Level2 normal passes
 * (src/Object.cpp:3219-3253, :2402-2424, :2715-2719): GPV_NORMALS_OFF, GPV_NORMALS_BYTES (the
 * .raw encoding) or GPV_NORMALS_FLOAT.  With normals on, each voxel's triangles are also ordered
 * by id (the reference CPU path's list order), which the float sums follow. */
#define GPV_NORMALS_OFF 0
#define GPV_NORMALS_BYTES 1
#define GPV_NORMALS_FLOAT 2
int gpv_set_normals(gpv_ctx *ctx, int mode);
/* Voxel box hierarchy (Object::BuildHierarchy, src/Object.cpp:2750-2867; default off): a binary
 * tree over the Level1 voxels, whose leaves are the voxel boxes with solid = the inside fill's
 * parity.  Built for grids whose voxel count is a power of two; others get none. */
int gpv_set_hierarchy(gpv_ctx *ctx, int on);
int gpv_result_copy_hierarchy_to_host(gpv_ctx *ctx, const gpv_result *res, gpv_box *out,
                                      cudaStream_t stream);
/* Inside fill of both levels (default GPV_FILL_RAY):
 *   GPV_FILL_RAY      +z ray parity from each voxel centre / Level2 ray origin, the CPU path
 *                     ClassifyInOutCPU + ClassifyInOutLevel2CPU (src/Object.cpp:716-779,
 *                     :1111-1207), bit for bit.
 *   GPV_FILL_STENCIL  the rasterised stencil-parity fill ClassifyInOut2x + ClassifyInOut2xLevel2
 *                     (src/Object.cpp:1446-1649, :1210-1444), which the reference runs through
 *                     OpenGL, as CUDA kernels: per z slice, 2x2 samples per voxel (pixel centres
 *                     of an orthographic viewport over the bounding box, or over the Level1
 *                     voxel's x/y extent for Level2), each counting the triangles that cover it
 *                     with their surface at or below the slice's clip plane; a voxel is inside
 *                     when at least 3 of its 4 counts are odd.  Level1 draws every triangle,
 *                     Level2 the triangles recorded in the voxel's Level1 column.  Coverage uses
 *                     vertices snapped to 1/256 pixel, exact integer edge functions and a
 *                     top-left tie rule; the surface height is interpolated in float.  A GPU
 *                     rasteriser's own sub-pixel and clipping arithmetic can differ, so bit
 *                     equality holds against this restatement, not against a GL driver.
 * The work counts ray1 and ray2 are 0 with the stencil fill. */
#define GPV_FILL_RAY 0
#define GPV_FILL_STENCIL 1
int gpv_set_fill(gpv_ctx *ctx, int mode);
/* Record the launch sequences of each voxelization as CUDA graphs; the executable graphs are
 * cached in the context and updated in place.
 *   GPV_GRAPHS_ONE (default, also any other non-zero value): a call with the same meshes (counts)
 *     and grids as the context's previous call on this path (device triangles, no normals, the
 *     ray fill, no hierarchy) is recorded as ONE graph: its result arrays and second-half launches
 *     are sized by that call's counts, and a planning kernel computes every per-mesh base on the
 *     device, so no host synchronisation splits the call.  A size that does not fit re-runs the
 *     call with the exact sizes.  Other calls run as two graphs;
 *   GPV_GRAPHS_TWO: always two graphs (first half, host synchronisation and planning, second half);
 *   0: launched directly. */
#define GPV_GRAPHS_ONE 1
#define GPV_GRAPHS_TWO 2
int gpv_set_graphs(gpv_ctx *ctx, int mode);
/* Autotuner: times every (tile, Level2 chunk) pair of {32,64,128,256} x {4,8,16,32} on the given
 * sample batch (CUDA events on `stream`), keeps the fastest in the context and reports it. */
int gpv_autotune(gpv_ctx *ctx, int32_t n, const float *const *d_tris, const int64_t *num_triangles,
                 const gpv_grid_spec *specs, cudaStream_t stream, int32_t *tile,
                 int32_t *level2_chunk, float *ms_per_batch);
/* Per-stage CUDA-event timing on the launching stream (off by default).  Stages:
 * 0 prep, 1 Level1 SAT+fill, 2 fill finish + boundary scan, 3 Level1 expansion,
 * 4 pair sort + lists, 5 Level2 (work items + kernel), 6 the Level2 kernel alone, 7 per-mesh pair
 * bases, 8 between the two phases (counts copied out, host planning, second launch, uploads in).
 * gpv_stage_times returns the number of timed calls and the accumulated milliseconds per stage
 * (up to 9 slots; unused slots stay 0).  The events are recorded inside the phases' CUDA graphs
 * and cost ~0.01-0.05 ms per call, so time the calls themselves with timing off. */
int gpv_set_timing(gpv_ctx *ctx, int on);
int gpv_stage_times(gpv_ctx *ctx, double *ms, int n);
/* Host-side milliseconds per call segment, accumulated while timing is on: 0 setup up to the
 * first recorded launch sequence, 1 from there to the first synchronisation returning, 2 planning
 * between the synchronisations, 3 the second launch sequence to the last synchronisation
 * returning, 4 result assembly.  Returns the number of timed calls. */
int gpv_host_times(gpv_ctx *ctx, double *ms, int n);
/* Number of kernels this library has launched in this process. */
uint64_t gpv_kernel_launches(void);
/* Failure-detection hooks (no counterpart in the reference).  They make the failure paths run
 * on demand, without faulting or hanging the GPU:
 *   GPV_DEBUG_WAIT_LIMIT    polls of the Level1 kernel's bounded wait for a staged tile before it
 *                           gives up (0: the built-in limit);
 *   GPV_DEBUG_FAIL_WAIT     non-zero: that wait gives up at once.  The kernel raises its status
 *                           word, lets the copies in flight land and returns; the call returns
 *                           GPV_ERR_DEVICE and the context stays usable;
 *   GPV_DEBUG_PAIR_CAPACITY the next call starts with this (voxel, triangle) record capacity
 *                           (one-shot): an overflow re-runs the call with the exact capacity;
 *   GPV_DEBUG_FAIL_ALLOCS   the next this-many device allocations of the context are refused
 *                           (the call returns GPV_ERR_OOM);
 *   GPV_DEBUG_ONE_GRAPH_CAPACITY the next one-graph call's boundary-voxel capacity (one-shot): a
 *                           smaller one than the call needs re-runs it with the exact sizes.
 * gpv_get_debug reads GPV_DEBUG_REPLANS (calls re-run after a record-buffer overflow),
 * GPV_DEBUG_ONE_GRAPH_CALLS (calls completed as one graph) and GPV_DEBUG_ONE_GRAPH_REPLANS
 * (one-graph calls re-run because a size did not fit). */
#define GPV_DEBUG_WAIT_LIMIT 1
#define GPV_DEBUG_FAIL_WAIT 2
#define GPV_DEBUG_PAIR_CAPACITY 3
#define GPV_DEBUG_FAIL_ALLOCS 4
#define GPV_DEBUG_REPLANS 5
#define GPV_DEBUG_ONE_GRAPH_CAPACITY 6
#define GPV_DEBUG_ONE_GRAPH_CALLS 7
#define GPV_DEBUG_ONE_GRAPH_REPLANS 8
int gpv_set_debug(gpv_ctx *ctx, int what, int64_t value);
int64_t gpv_get_debug(gpv_ctx *ctx, int what);

/* ---- grids --------------------------------------------------------------------------------- */
/* Explicit grid: n^3 cells over the mesh box grown by one cell on every side. */
int gpv_grid_padded(const float mesh_min[3], const float mesh_max[3], const int32_t ndiv[3],
                    const int32_t ndiv2[3], gpv_grid_spec *out);
/* Reference sizing from GLParameters::voxelCount / voxelCount2 (src/Object.cpp:3094-3107). */
int gpv_grid_reference(const float bbox_min[3], const float bbox_max[3], float max_model_size,
                       int32_t voxel_count, int32_t voxel_count2, gpv_grid_spec *out);

/* ---- voxelization ---------------------------------------------------------------------------- */
/* Plain path: one mesh, device triangles (16-byte aligned), results stay on the device. */
int gpv_voxelize(gpv_ctx *ctx, const float *d_tris, int64_t num_triangles,
                 const gpv_grid_spec *spec, gpv_result *out, cudaStream_t stream);
/* Same, from host triangles: page-locked, 16-byte aligned triangles are read in place by the
 * first kernel (which packs them into device memory); others are copied in on the stream. */
int gpv_voxelize_host(gpv_ctx *ctx, const float *h_tris, int64_t num_triangles,
                      const gpv_grid_spec *spec, gpv_result *out, cudaStream_t stream);
/* Host triangles in, host outputs out, with the transfers overlapped with the computation.  The
 * Level1 arrays are copied on a copy stream of the context as soon as they exist.  The Level2
 * blocks:
 *   slabs == 0 and h_level2_inout page-locked (cudaMallocHost / cudaHostRegister): the Level2
 *     kernel writes them into h_level2_inout itself while it computes (no device copy, no D2H);
 *     the result's level2_inout is then that buffer's device address and is not freed;
 *   otherwise: z-slab by z-slab -- the Level2 launch is split into `slabs` slabs of Level1
 *     layers (<= 8; 0 picks one slab per 12 MB of Level2 output; slab launches alternate
 *     between two streams so their tails overlap) and each slab is copied while later slabs
 *     compute.
 * Any host pointer may be NULL; page-locked buffers give the full transfer rate.  The result is
 * also returned (device arrays valid until gpv_result_release).  If h_l2_bytes < num_boundary *
 * n2^3 nothing is written to h_l2 and GPV_ERR_BUDGET is returned with the result complete
 * (release it; num_boundary gives the size needed). */
/* Packed Level2 transfer of gpv_voxelize_to_host (default: on, threads by the machine, every
 * slab with a share of 45 percent, outputs of 64 MiB and more).  When the Level2 kernel writes page-locked host memory
 * directly (slabs == 0), the link carries one byte per Level2 cell.  With this on, the z slabs
 * in slab_mask (bit k: slab k of 8) send 2-bit codes into page-locked staging instead, a quarter
 * of the bytes, for the first share_percent percent of their boundary voxels (output order; the
 * rest keep the direct byte writes).  `threads` host threads (the calling thread among them; -1:
 * up to 16 by the machine; 0 or 1: off) turn each finished slab's codes into the same bytes in
 * h_level2_inout, while later slabs compute.  It applies to Level2 grids with n2z of 8 or 16 and
 * a multiple of 16 sub-columns per layer, to 16-byte aligned Level2 buffers and to outputs of at
 * least min_level2_bytes.  The link carries the direct bytes and the codes while the host
 * threads expand, so the two share the output.  share_percent 0..100 (0: off). */
int gpv_set_host_expand(gpv_ctx *ctx, int threads, uint32_t slab_mask, int32_t share_percent,
                        int64_t min_level2_bytes);
int gpv_voxelize_to_host(gpv_ctx *ctx, const float *h_tris, int64_t num_triangles,
                         const gpv_grid_spec *spec, uint8_t *h_level1_inout,
                         int32_t *h_level1_prefix, int32_t *h_boundary_index, uint8_t *h_level2_inout,
                         int64_t h_level2_bytes, int32_t slabs, gpv_result *out,
                         cudaStream_t stream);
/* Copy a result's arrays to host buffers (any may be NULL) and wait for the stream. */
int gpv_result_copy_to_host(gpv_ctx *ctx, const gpv_result *res, uint8_t *level1_inout,
                            int32_t *level1_prefix, int32_t *boundary_index,
                            uint8_t *level2_inout, cudaStream_t stream);
/* Copy a result's normals (3 bytes or 3 floats per voxel / cell, per normal_mode) to host
 * buffers (either may be NULL) and wait for the stream. */
int gpv_result_copy_normals_to_host(gpv_ctx *ctx, const gpv_result *res, void *level1_normal,
                                    void *level2_normal, cudaStream_t stream);
/* Frees a result's device arrays (stream-ordered, on the stream the result was made on: release
 * results before destroying that stream, and from the thread that uses the context -- a stream
 * being recorded into a graph by another thread must not receive the frees). */
int gpv_result_release(gpv_ctx *ctx, gpv_result *res);

/* Batched path: n meshes in one launch sequence (persistent work-queue kernels).
 * d_tris[i] are device pointers (16-byte aligned); results are filled like gpv_voxelize. */
int gpv_voxelize_batch(gpv_ctx *ctx, int32_t n, const float *const *d_tris,
                       const int64_t *num_triangles, const gpv_grid_spec *specs,
                       gpv_result *results, cudaStream_t stream);

/* Level1 voxelization that allocates nothing (no counterpart in the reference).  For callers
 * that cannot call cudaMalloc -- code running inside another allocator's or memory pool's hooks
 * (calling back into an allocator from there recurses or deadlocks), host paths that must not
 * take the device synchronisation cudaMalloc/cudaFree can cause, plugin hosts that forbid a
 * library its own device memory.  The caller passes device triangles (16-byte aligned) and three
 * device outputs: level1_inout (nx*ny*nz bytes), level1_prefix (nx*ny*nz int32) and
 * boundary_index (room for nx*ny*nz int32); the boundary count is returned in *num_boundary and
 * the call waits for `stream`.  Results equal gpv_voxelize's Level1 outputs; the Level2 divisions
 * of the spec are checked as gpv_voxelize checks them and otherwise ignored.  All intermediates
 * live in one file-scope device array of 32 MiB that every GPU loading the library holds until
 * exit; inputs whose intermediates do not fit (about 400k triangles at most, fewer on large
 * grids) are rejected with GPV_ERR_INVALID and a reason in gpv_noalloc_last_error() (per host
 * thread).  Every call looks up the array's device address (cudaGetSymbolAddress) with the
 * caller's device current.  A call copies its tables from host memory and waits for `stream`,
 * so it is refused (GPV_ERR_INVALID) on a stream that is capturing.  Calls share the array and clear
 * what must start at zero themselves; calls whose GPU work overlaps race on it and must be
 * serialised. */
int gpv_voxelize_level1_noalloc(const float *d_tris, int64_t num_triangles,
                                const gpv_grid_spec *spec, uint8_t *d_level1_inout,
                                int32_t *d_level1_prefix, int32_t *d_boundary_index,
                                int64_t *num_boundary, cudaStream_t stream);
const char *gpv_noalloc_last_error(void);

/* ---- serving: continuous batching (no counterpart in the reference) -------------------------
 * Requests carry host triangles (caller memory, valid until the request completes; pinned memory
 * gives the fastest copies) and a grid.  `workers` threads, each with its own context and stream,
 * admit every waiting request that fits `budget_bytes` of device memory by a predicted footprint
 * (FIFO), and voxelize each admitted set with one batched launch sequence; requests arriving
 * meanwhile join the next set.  Results stay on the device (and count against the budget) until
 * gpv_server_release.  Submit returns GPV_ERR_BUDGET for a request that can never fit. */
typedef struct gpv_server gpv_server;
int gpv_server_create(int device, int64_t budget_bytes, int32_t workers, int32_t max_batch,
                      gpv_server **out);
int gpv_server_set_tunables(gpv_server *srv, int32_t tile, int32_t level2_chunk);
int gpv_server_submit(gpv_server *srv, const float *h_tris, int64_t num_triangles,
                      const gpv_grid_spec *spec, uint64_t *ticket);
/* Waits up to timeout_ms (0: no wait, <0: forever).  GPV_ERR_PENDING while running; on
 * completion the result's status, its device arrays, the submit-to-done latency and the time the
 * request waited before its batch started. */
int gpv_server_poll(gpv_server *srv, uint64_t ticket, int32_t timeout_ms, gpv_result *out,
                    double *latency_ms, double *queue_ms);
int gpv_server_release(gpv_server *srv, uint64_t ticket);
/* Resident meshes: gpv_server_add_mesh uploads a mesh once into the server's device pool (its
 * bytes count against the budget until removed) and returns its id; gpv_server_submit_mesh
 * requests a voxelization of it by id (no host-to-device copy per request);
 * gpv_server_remove_mesh frees it (GPV_ERR_PENDING while requests still read it). */
int gpv_server_add_mesh(gpv_server *srv, const float *h_tris, int64_t num_triangles,
                        uint64_t *mesh_id);
int gpv_server_submit_mesh(gpv_server *srv, uint64_t mesh_id, const gpv_grid_spec *spec,
                           uint64_t *ticket);
int gpv_server_remove_mesh(gpv_server *srv, uint64_t mesh_id);
int gpv_server_stats(gpv_server *srv, int64_t *in_use_bytes, int64_t *pending, uint64_t *batches,
                     uint64_t *served);
void gpv_server_destroy(gpv_server *srv);

/* ---- meshes and files (host) ---------------------------------------------------------------- */
int gpv_load_obj(const char *path, gpv_mesh *out); /* Object::ReadObject (src/Object.cpp:395) */
int gpv_load_off(const char *path, gpv_mesh *out); /* Object::ReadOFFObject (src/Object.cpp:171) */
void gpv_mesh_free(gpv_mesh *mesh);
/* Object::SaveVoxelization's files from host arrays (src/Object.cpp:2934-3075):
 * <prefix>VoxelConfig.txt, Level1InOut.raw, Level1BoundaryPrefixSum.raw, Level2InOut.raw. */
int gpv_write_raw(const char *prefix, const gpv_result *res, const uint8_t *level1_inout,
                  const int32_t *level1_prefix, const uint8_t *level2_inout);
/* The two normal files of Object::SaveVoxelization (src/Object.cpp:3032-3035, :3047-3049,
 * :3058-3064): <prefix>Level1Normal.raw (3 * num_level1 bytes) and, with Level2,
 * <prefix>Level2Normal.raw (3 * num_boundary * n2x*n2y*n2z bytes), from host byte normals. */
int gpv_write_raw_normals(const char *prefix, const gpv_result *res, const uint8_t *level1_normal,
                          const uint8_t *level2_normal);

/* Reading a saved voxelization back (host).  <prefix>VoxelConfig.txt, in the line order
 * Object::SaveVoxelization writes (src/Object.cpp:3009-3022): prefix; bbox min; bbox max; Level1
 * divisions; Level1 grid size; Level1 inside count; Level1 boundary count; and with Level2: Level2
 * divisions; Level2 grid size; Level2 inside count; Level2 boundary count. */
typedef struct {
    float bbox_min[3], bbox_max[3];
    int32_t ndiv[3];
    float grid_size[3];
    int64_t num_level1_inside;
    int64_t num_boundary;        /* Level1 boundary voxels = Level2 blocks */
    int32_t has_level2;
    int32_t ndiv2[3];
    float grid_size2[3];
    int64_t num_level2_inside;
    int64_t num_level2_boundary;
} gpv_voxel_config;
int gpv_read_voxel_config(const char *prefix, gpv_voxel_config *out);
/* Reads the .raw files of a saved voxelization into host buffers sized from the config (any
 * buffer may be NULL to skip its file): Level1InOut (N1 bytes), Level1BoundaryPrefixSum (N1
 * int32), Level2InOut (B*n2^3 bytes), Level1Normal (3*N1 bytes), Level2Normal (3*B*n2^3 bytes).
 * A file shorter than its size is GPV_ERR_IO. */
int gpv_read_raw(const char *prefix, const gpv_voxel_config *cfg, uint8_t *level1_inout,
                 int32_t *level1_prefix, uint8_t *level2_inout, uint8_t *level1_normal,
                 uint8_t *level2_normal);

/* ---- seeded synthetic meshes (host) ---------------------------------------------------------- */
/* Each returns the triangle count; with tris == NULL only the count is returned. */
int64_t gpv_gen_uvsphere(uint64_t seed, int32_t nlon, int32_t nlat, const float center[3],
                         float radius, float jitter_sigma, float *tris);
int64_t gpv_gen_torus(uint64_t seed, int32_t nu, int32_t nv, const float center[3], float R,
                      float r, float noise_amp, float *tris);
int64_t gpv_gen_star(uint64_t seed, int32_t subdiv, const float center[3], float radius,
                     float amp, const float scale[3], float *tris);
int64_t gpv_gen_superellipsoid(uint64_t seed, int32_t nlon, int32_t nlat, const float center[3],
                               const float semi[3], float e1, float e2, const float rot[9],
                               float *tris);

/* ---- reference-named shims: the C entry points of GPView's GPViewCUDA library ------------------
 * (includes/CUDAUtilities.h:72-74, :87-89).  InitializeCUDA and CUDACheckErrors are not among
 * them: the reference declares those with C++ linkage (includes/CUDAUtilities.h:63-64) and
 * defines them in the application (src/CUDAUtilities.cpp:33-55), which keeps them. */
/* cuda/CUDAClassifyTessellation.cu:507-515.  Marks inOut[v]=2 for every voxel whose SAT test
 * passes inside each triangle's candidate box, counts triangles per voxel in voxelTriCount and
 * stores up to triBufferLen ids per voxel in voxelTriIndex[v*triBufferLen..] (never beyond;
 * the count still reports the true number, so the caller's resize-and-retry works).  Centres
 * are the reference CPU's: float((p+0.5)*boxExtents*2 + objBoxMin), evaluated in double. */
int CUDAClassifyTessellation(float *trianglesCUDAData, int numTriangles, float *inOutCUDAData,
                             int *voxelTriCountCUDAData, int *voxelTriIndexCUDAData,
                             float3 objBoxMin, float3 objBoxMax, float3 boxExtents, int3 numDiv,
                             int triBufferLen);
/* cuda/CUDAClassifyTessellation.cu:518-527.  Level2 SAT of each boundary voxel b against the
 * triangles listed for Level1 voxel level2Index[b]; writes 2 into level2InOut and accumulates
 * unit face normals + a count into level2Normal (4 floats per cell), in list order. */
int CUDAClassifyTessellationLevel2(float *trianglesCUDAData, float *level2InOutCUDAData,
                                   float *level2NormalCUDAData, float *level1MidPointCUDAData,
                                   int *level2IndexCUDAData, int *voxelTriCountCUDAData,
                                   int *level1TriFlatIndexCUDAData, int *level1TriFlatCUDAData,
                                   int numBoundary, int3 numDiv2, float3 boxExtentsLevel1,
                                   float3 boxExtentsLevel2);
/* cuda/CUDAClassifyTessellation.cu:531-540.  +z ray parity of every Level2 cell centre against
 * the x/y-column triangle list of its Level1 voxel; odd -> level2InOut = 1. */
int CUDAClassifyInOutLevel2(float *trianglesCUDAData, float *level2InOutCUDAData,
                            float *level1MidPointCUDAData, int *level2IndexCUDAData,
                            int *xyTriCountCUDAData, int *xyTriFlatIndexCUDAData,
                            int *xyTriFlatCUDAData, int numBoundary, int3 numDiv, int3 numDiv2,
                            float3 boxExtentsLevel1, float3 boxExtentsLevel2);
/* cuda/THRUSTUtilities.cu:44-60 (called by src/CUDAUtilities.cpp:121-132 under the default
 * `#define THRUST`, includes/Includes.h:49): the largest of w*h device floats, first index on ties
 * (thrust::max_element), returned to the host; 0 for an empty range. */
float THRUSTDeviceFindMax(float *dataCUDAPointer, int w, int h);
/* cuda/THRUSTUtilities.cu:82-102: the float4 with the largest w; x, y, z and w = 1 into the host
 * *maxVal, its index into the host *maxLoc, its w returned. */
float THRUSTDeviceFindMaxFloat4(float4 *dataCUDAPointer, int numValues, float4 *maxVal, int *maxLoc);
/* cuda/THRUSTUtilities.cu:128-160: the rows of n (row, min, max) triples sorted by row into the
 * host array rowNumbers (rows >= 0 ascending, then negative rows in input order); the device
 * inputs are unchanged and minData / maxData are not written, as in the reference. */
void THRUSTDeviceMinMaxSort(float *minDataCUDAPointer, float *maxDataCUDAPointer,
                            int *rowDataCUDAPointer, int n, float *minData, float *maxData,
                            int *rowNumbers);

#ifdef __cplusplus
}
#endif
#endif /* GPVIEW_H */
