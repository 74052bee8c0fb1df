// gpv_internal.h -- declarations shared by the library's translation units (not installed).
#pragma once
#include <cstdint>
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

// ---- kernels (gpv_kernels.cu) -----------------------------------------------------------------
struct Level1Bufs {
  const float *tris;     // input float[T*9]
  int64_t T;
  float4 *ptri;          // packed triangles, 3 float4 per triangle (w carries fill ranges)
  int4 *rng;             // SAT candidate box (packed) per triangle
  float4 *fbox;          // conservative x/y box for the ray tests per triangle
  uint32_t *bplane;      // boundary bit plane (padded rows)
  uint32_t *iplane;      // inside (parity) bit plane (padded rows)
  uint32_t *toggles;     // column-major parity toggles
  uint32_t *keys, *vals; // pair buffer
  MeshStats *stats;
};

void launch_prep(const GridDev &g, const Level1Bufs &b, cudaStream_t s);
void launch_level1(const GridDev &g, const Level1Bufs &b, int tile, cudaStream_t s);
void launch_fill_finish(const GridDev &g, const Level1Bufs &b, cudaStream_t s);
void launch_popc(const GridDev &g, const uint32_t *bplane, uint32_t *cnt, cudaStream_t s);
void launch_expand(const GridDev &g, const uint32_t *bplane, const uint32_t *iplane,
                   const uint32_t *wpre, uint8_t *l1, int32_t *prefix, int32_t *bindex,
                   MeshStats *st, cudaStream_t s);
void launch_heads(const uint32_t *keys, int64_t P, uint32_t *flags, cudaStream_t s);
void launch_useg(const uint32_t *flags, const uint32_t *uidx, int64_t P, uint32_t *useg,
                 cudaStream_t s);
int level2_chunk(const GridDev &g);
size_t level2_smem(const GridDev &g);
int64_t level2_temp_words(int64_t B);
void launch_level2c(const GridDev &g, const float4 *ptri, const float4 *fbox,
                    const uint32_t *keys, const uint32_t *vals, const uint32_t *useg,
                    const int32_t *prefix, int64_t B, uint32_t *tmp, uint8_t *l2, MeshStats *st,
                    cudaStream_t s);

GridDev make_griddev(const GridHost &gh, const float *dtables);
int64_t table_floats(const GridHost &gh);
void pack_tables(const GridHost &gh, float *host);

}  // namespace gpv
