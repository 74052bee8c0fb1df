/*
 * gpv_oracle.c -- CPU restatement of GPView's two-level voxelization (test infrastructure).
 *
 * THIS FILE IS THE CORRECTNESS ORACLE, NOT PART OF THE PRODUCT.  Only the test suite, the
 * smoke check and the CPU-baseline leg of bench.py load it.  The GPU library never links it.
 *
 * It restates, in plain C with the reference's exact float/double promotions and operation
 * order, the CPU composition of the reference (GPView, idealab-isu):
 *   - predicates:   src/TriBoxIntersection.cpp:64-210 (planeBoxOverlap, TriBoxOverlap)
 *                   src/TriRayIntersection.cpp:78-131 (triangle_ray_intersection)
 *   - grid sizing:  src/Object.cpp:3094-3136 (reference mode) and the explicit-grid mode
 *   - Level1 fill:  src/Object.cpp:716-779   (ClassifyInOutCPU, +z ray parity over all triangles)
 *   - Level1 SAT:   src/Object.cpp:2256-2342 (ClassifyTessellation) + :2681-2748 (TestTriBox,
 *                   AddPointToVoxel)
 *   - compaction:   src/Object.cpp:3258-3284 (boundaryPrefixSum, boundaryIndex)
 *   - Level2 fill:  src/Object.cpp:1111-1207 (ClassifyInOutLevel2CPU)
 *   - Level2 SAT:   src/Object.cpp:2344-2400 (ClassifyTessellationLevel2)
 *
 * Build with -O2 -ffp-contract=off -fno-fast-math (mandatory: an FMA would change results).
 * Arrays the reference leaves uninitialised (Level2 blocks after the first, src/Object.cpp:3284)
 * are zero-initialised here.
 *
 * Level1 fill modes:
 *   ORC_FILL_VOXEL   -- exactly ClassifyInOutCPU: every voxel centre against every triangle.
 *   ORC_FILL_COLUMN  -- the same predicate, reorganised per column: the u/v part of the
 *                       Moller-Trumbore test depends only on the ray's x,y, so it is evaluated
 *                       once per (column, triangle); t is evaluated per voxel centre.  Same
 *                       float operations, same results; O(columns * T).
 *   ORC_FILL_CAND    -- per-column candidate lists: a triangle is tested against a column only
 *                       if the column centre lies inside the triangle's x/y bounding box grown by
 *                       a generous margin (or always, for triangles whose x/y projection is
 *                       ill-conditioned).  Checked equal to ORC_FILL_COLUMN by the tests.
 *   ORC_FILL_STENCIL -- both levels filled by the rasterised stencil parity of ClassifyInOut2x
 *                       (src/Object.cpp:1446-1649) and ClassifyInOut2xLevel2 (:1210-1444), which
 *                       the reference runs through OpenGL.  No graphics stack exists here, so the
 *                       rasterisation is restated (orc_st_* below) and parity for this mode is
 *                       unpinned: it is pinned to the restatement, and the tests check the
 *                       restatement against a literal slice-by-slice form of the two functions.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORC_REF_PREDICATES
/* Built only in oracle/_ref: the reference's own TriBoxOverlap / triangle_ray_intersection,
 * compiled from its sources and exported through ref_shim.cpp. */
int ref_tri_box(const float c[3], const float h[3], const float *tv);
void ref_face_normal(const float *tv, float *out);
void ref_average_normal(const float *sum, float count, float *out);
int ref_tri_ray(const float *V1, const float *V2, const float *V3, const float *O,
                const float *D, float *out);
#endif

#define ORC_FILL_VOXEL 0
#define ORC_FILL_COLUMN 1
#define ORC_FILL_CAND 2
#define ORC_FILL_STENCIL 3

/* ------------------------------------------------------------------------------------------ */
/* Predicates                                                                                  */
/* ------------------------------------------------------------------------------------------ */

/* Plane/box part of the SAT (src/TriBoxIntersection.cpp:64-86). */
static int orc_plane_box(const float nrm[3], const float vert[3], const float maxbox[3], int *full)
{
    float vmin[3], vmax[3];
    for (int q = 0; q < 3; ++q) {
        float v = vert[q];
        if (nrm[q] > 0.0f) {
            vmin[q] = -maxbox[q] - v;
            vmax[q] = maxbox[q] - v;
        } else {
            vmin[q] = maxbox[q] - v;
            vmax[q] = -maxbox[q] - v;
        }
    }
    float dmin = nrm[0] * vmin[0] + nrm[1] * vmin[1] + nrm[2] * vmin[2];
    if (dmin > 0.0f) return 0;
    *full = 1;
    float dmax = nrm[0] * vmax[0] + nrm[1] * vmax[1] + nrm[2] * vmax[2];
    if (dmax >= 0.0f) return 1;
    return 0;
}

/* One edge-cross-axis test: projections pa, pb of two vertices, radius from |edge| and the
 * half sizes.  Separated (return 1) iff min(pa,pb) > rad or max(pa,pb) < -rad. */
static inline int orc_axis_sep(float pa, float pb, float rad)
{
    float mn, mx;
    if (pa < pb) { mn = pa; mx = pb; } else { mn = pb; mx = pa; }
    return (mn > rad || mx < -rad);
}

/* Akenine-Moller triangle/box overlap in the reference's order and roundings
 * (src/TriBoxIntersection.cpp:135-210). tv = 9 floats, vertex-major. */
/* Executed FP32 operation counts of the reference predicates by exit point (add, sub, mul, and
 * the one divide of the ray test; fabs, negation and compares excluded).  SAT
 * (src/TriBoxIntersection.cpp:135-210, :64-86): 18 subtractions for the translated vertices and
 * edges, 9 per edge-cross axis (two 2-product differences and the radius), nothing for the box
 * axes, then the normal (9), vmin/vmax (6) and one dot product (5) before the first plane exit and
 * a second dot product (5) before the last.  Ray (src/TriRayIntersection.cpp:78-131): edges (6),
 * P (9) and det (5); 1/det, T (3) and u (6); Q (9), v (6) and u+v (1); t (6). */
enum {
    ORC_OPS_SAT_SETUP = 18, ORC_OPS_SAT_AXIS = 9, ORC_OPS_SAT_BOX = 99, ORC_OPS_SAT_PLANE = 119,
    ORC_OPS_SAT_FULL = 124
};
enum { ORC_OPS_RAY_DET = 20, ORC_OPS_RAY_U = 30, ORC_OPS_RAY_V = 46, ORC_OPS_RAY_FULL = 52 };

static int orc_tri_box_own(const float c[3], const float h[3], const float *tv, int *ops);
int orc_tri_box(const float c[3], const float h[3], const float *tv)
{
#ifdef ORC_REF_PREDICATES
    return ref_tri_box(c, h, tv);
#else
    int ops;
    return orc_tri_box_own(c, h, tv, &ops);
#endif
}

/* The nine edge-cross axes in the reference's order: (edge, vertex pair, axis). */
static int orc_tri_box_own(const float c[3], const float h[3], const float *tv, int *ops)
{
    float v0[3], v1[3], v2[3], e0[3], e1[3], e2[3];
    for (int a = 0; a < 3; ++a) {
        v0[a] = tv[0 + a] - c[a];
        v1[a] = tv[3 + a] - c[a];
        v2[a] = tv[6 + a] - c[a];
    }
    for (int a = 0; a < 3; ++a) {
        e0[a] = v1[a] - v0[a];
        e1[a] = v2[a] - v1[a];
        e2[a] = v0[a] - v2[a];
    }
    float fx, fy, fz, a_, b_;
#define ORC_SEP(k, pa, pb, rad) \
    if (orc_axis_sep((pa), (pb), (rad))) { *ops = ORC_OPS_SAT_SETUP + ORC_OPS_SAT_AXIS * (k); return 0; }
    /* edge 0 */
    fx = fabsf(e0[0]); fy = fabsf(e0[1]); fz = fabsf(e0[2]);
    a_ = e0[2]; b_ = e0[1]; /* X01 */
    ORC_SEP(1, a_ * v0[1] - b_ * v0[2], a_ * v2[1] - b_ * v2[2], fz * h[1] + fy * h[2])
    a_ = e0[2]; b_ = e0[0]; /* Y02 */
    ORC_SEP(2, -a_ * v0[0] + b_ * v0[2], -a_ * v2[0] + b_ * v2[2], fz * h[0] + fx * h[2])
    a_ = e0[1]; b_ = e0[0]; /* Z12 */
    ORC_SEP(3, a_ * v1[0] - b_ * v1[1], a_ * v2[0] - b_ * v2[1], fy * h[0] + fx * h[1])
    /* edge 1 */
    fx = fabsf(e1[0]); fy = fabsf(e1[1]); fz = fabsf(e1[2]);
    a_ = e1[2]; b_ = e1[1]; /* X01 */
    ORC_SEP(4, a_ * v0[1] - b_ * v0[2], a_ * v2[1] - b_ * v2[2], fz * h[1] + fy * h[2])
    a_ = e1[2]; b_ = e1[0]; /* Y02 */
    ORC_SEP(5, -a_ * v0[0] + b_ * v0[2], -a_ * v2[0] + b_ * v2[2], fz * h[0] + fx * h[2])
    a_ = e1[1]; b_ = e1[0]; /* Z0 */
    ORC_SEP(6, a_ * v0[0] - b_ * v0[1], a_ * v1[0] - b_ * v1[1], fy * h[0] + fx * h[1])
    /* edge 2 */
    fx = fabsf(e2[0]); fy = fabsf(e2[1]); fz = fabsf(e2[2]);
    a_ = e2[2]; b_ = e2[1]; /* X2 */
    ORC_SEP(7, a_ * v0[1] - b_ * v0[2], a_ * v1[1] - b_ * v1[2], fz * h[1] + fy * h[2])
    a_ = e2[2]; b_ = e2[0]; /* Y1 */
    ORC_SEP(8, -a_ * v0[0] + b_ * v0[2], -a_ * v1[0] + b_ * v1[2], fz * h[0] + fx * h[2])
    a_ = e2[1]; b_ = e2[0]; /* Z12 */
    ORC_SEP(9, a_ * v1[0] - b_ * v1[1], a_ * v2[0] - b_ * v2[1], fy * h[0] + fx * h[1])
#undef ORC_SEP
    /* box axes: min/max of the translated vertices */
    *ops = ORC_OPS_SAT_BOX;
    for (int a = 0; a < 3; ++a) {
        float mn = v0[a], mx = v0[a];
        if (v1[a] < mn) mn = v1[a];
        if (v1[a] > mx) mx = v1[a];
        if (v2[a] < mn) mn = v2[a];
        if (v2[a] > mx) mx = v2[a];
        if (mn > h[a] || mx < -h[a]) return 0;
    }
    /* triangle plane */
    float nrm[3];
    nrm[0] = e0[1] * e1[2] - e0[2] * e1[1];
    nrm[1] = e0[2] * e1[0] - e0[0] * e1[2];
    nrm[2] = e0[0] * e1[1] - e0[1] * e1[0];
    int full = 0;
    const int hit = orc_plane_box(nrm, v0, h, &full);
    *ops = full ? ORC_OPS_SAT_FULL : ORC_OPS_SAT_PLANE;
    return hit;
}

/* Moller-Trumbore ray/triangle test with a general direction, as src/TriRayIntersection.cpp:
 * 78-131: edges from V1, P = D x e2, det compared against 1e-6 IN DOUBLE, u/v bounds in
 * float, t > 1e-6 IN DOUBLE.  Returns 1 on a hit and writes t. */
int orc_tri_ray(const float V1[3], const float V2[3], const float V3[3], const float O[3],
                const float D[3], float *out)
{
#ifdef ORC_REF_PREDICATES
    return ref_tri_ray(V1, V2, V3, O, D, out);
#endif
    float e1[3], e2[3], P[3], Q[3], T[3];
    for (int a = 0; a < 3; ++a) { e1[a] = V2[a] - V1[a]; e2[a] = V3[a] - V1[a]; }
    P[0] = D[1] * e2[2] - D[2] * e2[1];
    P[1] = D[2] * e2[0] - D[0] * e2[2];
    P[2] = D[0] * e2[1] - D[1] * e2[0];
    float det = e1[0] * P[0] + e1[1] * P[1] + e1[2] * P[2];
    if ((double)det > -0.000001 && (double)det < 0.000001) return 0;
    float inv_det = 1.f / det;
    for (int a = 0; a < 3; ++a) T[a] = O[a] - V1[a];
    float u = (T[0] * P[0] + T[1] * P[1] + T[2] * P[2]) * inv_det;
    if (u < 0.f || u > 1.f) return 0;
    Q[0] = T[1] * e1[2] - T[2] * e1[1];
    Q[1] = T[2] * e1[0] - T[0] * e1[2];
    Q[2] = T[0] * e1[1] - T[1] * e1[0];
    float v = (D[0] * Q[0] + D[1] * Q[1] + D[2] * Q[2]) * inv_det;
    if (v < 0.f || u + v > 1.f) return 0;
    float t = (e2[0] * Q[0] + e2[1] * Q[1] + e2[2] * Q[2]) * inv_det;
    if ((double)t > 0.000001) {
        if (out) *out = t;
        return 1;
    }
    return 0;
}

/* Column part of the +z test (D = (0,0,1)).  With D = +z the reference's products against the
 * zero components of D only add signed zeros, which never change a comparison, so:
 *   det = e1x*(-e2y) + e1y*e2x,  u = (Tx*(-e2y) + Ty*e2x) * inv_det,  v = (Tx*e1y - Ty*e1x) * inv_det.
 * Returns 1 if the (x,y) column passes the det/u/v tests and fills the state for the t test. */
typedef struct {
    float e1[3], e2[3], inv_det, Tx, Ty, v1z;
    const float *tv; /* ORC_REF_PREDICATES: the whole test runs per origin */
    float ox, oy;
} orc_colhit;

/* *ops receives the reference's executed operation count for one origin of this column: the
 * det/u/v exits depend on the column only (D = +z), so every origin of the column takes the
 * same exit, and origins that reach the t test run the whole test. */
static int orc_ray_column_own(const float *tv, float ox, float oy, orc_colhit *st, int *ops)
{
    float e1x = tv[3] - tv[0], e1y = tv[4] - tv[1], e1z = tv[5] - tv[2];
    float e2x = tv[6] - tv[0], e2y = tv[7] - tv[1], e2z = tv[8] - tv[2];
    float det = e1x * (-e2y) + e1y * e2x;
    *ops = ORC_OPS_RAY_DET;
    if ((double)det > -0.000001 && (double)det < 0.000001) return 0;
    float inv_det = 1.f / det;
    float Tx = ox - tv[0], Ty = oy - tv[1];
    float u = (Tx * (-e2y) + Ty * e2x) * inv_det;
    *ops = ORC_OPS_RAY_U;
    if (u < 0.f || u > 1.f) return 0;
    float v = (Tx * e1y - Ty * e1x) * inv_det;
    *ops = ORC_OPS_RAY_V;
    if (v < 0.f || u + v > 1.f) return 0;
    *ops = ORC_OPS_RAY_FULL;
    st->e1[0] = e1x; st->e1[1] = e1y; st->e1[2] = e1z;
    st->e2[0] = e2x; st->e2[1] = e2y; st->e2[2] = e2z;
    st->inv_det = inv_det; st->Tx = Tx; st->Ty = Ty; st->v1z = tv[2];
    return 1;
}

static int orc_ray_column(const float *tv, float ox, float oy, orc_colhit *st)
{
#ifdef ORC_REF_PREDICATES
    st->tv = tv; st->ox = ox; st->oy = oy;
    return 1;
#else
    int ops;
    return orc_ray_column_own(tv, ox, oy, st, &ops);
#endif
}

/* t part of the +z test for one origin height. */
static inline int orc_ray_t(const orc_colhit *s, float oz)
{
#ifdef ORC_REF_PREDICATES
    {
        const float O[3] = {s->ox, s->oy, oz}, D[3] = {0.f, 0.f, 1.f};
        float tt;
        return ref_tri_ray(s->tv, s->tv + 3, s->tv + 6, O, D, &tt);
    }
#endif
    float Tz = oz - s->v1z;
    float Q0 = s->Ty * s->e1[2] - Tz * s->e1[1];
    float Q1 = Tz * s->e1[0] - s->Tx * s->e1[2];
    float Q2 = s->Tx * s->e1[1] - s->Ty * s->e1[0];
    float t = (s->e2[0] * Q0 + s->e2[1] * Q1 + s->e2[2] * Q2) * s->inv_det;
    return (double)t > 0.000001;
}

/* Full +z test through the column/t split; equal to orc_tri_ray with D=(0,0,1). */
int orc_tri_ray_z(const float *tv, const float O[3])
{
    orc_colhit s;
    if (!orc_ray_column(tv, O[0], O[1], &s)) return 0;
    return orc_ray_t(&s, O[2]);
}

/* ------------------------------------------------------------------------------------------ */
/* Grid                                                                                        */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    float bmin[3], bmax[3]; /* object bounding box (Object::bBoxMin/bBoxMax) */
    int32_t n[3];           /* Level1 divisions */
    int32_t n2[3];          /* Level2 divisions; 0 = no Level2 */
} orc_spec;

typedef struct {
    float g[3], e1[3], g2[3], e2[3];
    float *c1[3];  /* Level1 centres per axis (SAT centres, ray origins, midpoints) */
    float *c2s[3]; /* Level2 SAT centres, [i*n2+p] */
    float *o2[3];  /* Level2 ray origins, [i*n2+p] */
} orc_tables;

/* Grid sizes: src/Object.cpp:3108-3110 (gridSize = float((max-min)/(n*1.0))),
 * :3128-3130 (gridSize2 = float(gridSize/(n2*1.0))), extents = float(gridSize/2.0) (:3167). */
static void orc_tables_build(const orc_spec *s, orc_tables *t)
{
    for (int a = 0; a < 3; ++a) {
        float span = s->bmax[a] - s->bmin[a];
        t->g[a] = (float)(span / (s->n[a] * 1.0));
        t->e1[a] = (float)(t->g[a] / 2.0);
        int n2 = s->n2[a] > 0 ? s->n2[a] : 1;
        t->g2[a] = (float)(t->g[a] / (n2 * 1.0));
        t->e2[a] = (float)(t->g2[a] / 2.0);
        int n = s->n[a];
        t->c1[a] = (float *)malloc(sizeof(float) * (size_t)n);
        t->c2s[a] = (float *)malloc(sizeof(float) * (size_t)n * n2);
        t->o2[a] = (float *)malloc(sizeof(float) * (size_t)n * n2);
        for (int i = 0; i < n; ++i) {
            /* (i + 0.5)*gridSize + bBoxMin, double -> float (src/Object.cpp:3176-3178, :2329, :743) */
            float mid = (float)((i + 0.5) * t->g[a] + s->bmin[a]);
            t->c1[a][i] = mid;
            /* Level1 voxel minimum corner for the Level2 rays: float arithmetic (:1132-1134) */
            float mn = i * t->g[a] + s->bmin[a];
            for (int p = 0; p < n2; ++p) {
                /* (p + 0.5)*gridSize2 + midPoint - boxExtentsLevel1, double -> float (:2389-2391) */
                t->c2s[a][(size_t)i * n2 + p] = (float)((p + 0.5) * t->g2[a] + mid - t->e1[a]);
                /* minPoint + (p + 0.5)*gridSize2, double -> float (:1158-1160) */
                t->o2[a][(size_t)i * n2 + p] = (float)(mn + (p + 0.5) * t->g2[a]);
            }
        }
    }
}

static void orc_tables_free(orc_tables *t)
{
    for (int a = 0; a < 3; ++a) { free(t->c1[a]); free(t->c2s[a]); free(t->o2[a]); }
}

/* Exported so tests can compare the GPU library's host tables against these. */
void orc_grid_tables(const orc_spec *s, float *g, float *e1, float *g2, float *e2, float *c1,
                     float *c2s, float *o2)
{
    orc_tables t;
    orc_tables_build(s, &t);
    size_t off1 = 0, off2 = 0;
    for (int a = 0; a < 3; ++a) {
        int n = s->n[a], n2 = s->n2[a] > 0 ? s->n2[a] : 1;
        g[a] = t.g[a]; e1[a] = t.e1[a]; g2[a] = t.g2[a]; e2[a] = t.e2[a];
        if (c1) memcpy(c1 + off1, t.c1[a], sizeof(float) * n);
        if (c2s) memcpy(c2s + off2, t.c2s[a], sizeof(float) * (size_t)n * n2);
        if (o2) memcpy(o2 + off2, t.o2[a], sizeof(float) * (size_t)n * n2);
        off1 += n; off2 += (size_t)n * n2;
    }
    orc_tables_free(&t);
}

/* Reference-mode sizing (src/Object.cpp:3094-3107): nominal = maxModelSize/voxelCount,
 * n = GetNextDiv4(max(1, int(extent/nominal))). */
void orc_reference_divisions(const float bmin[3], const float bmax[3], float max_model_size,
                             int voxel_count, int32_t n_out[3])
{
    float nominal = (float)(max_model_size / (1.0 * voxel_count));
    for (int a = 0; a < 3; ++a) {
        int n = (int)((bmax[a] - bmin[a]) / nominal);
        if (n == 0) n++;
        n = (n % 4 == 0) ? n : n + (4 - n % 4);
        n_out[a] = n;
    }
}

/* Level1 cell index of a coordinate (src/Object.cpp:2280-2306): float divide and multiply,
 * truncation, and the decrement when the vertex sits exactly on the box maximum. */
static inline int orc_cell(float v, float bmin, float bmax, int n)
{
    float q = (v - bmin) / (bmax - bmin) * n;
    /* clamp before converting: vertices outside the box are undefined in the reference */
    if (q < -1.0f) q = -1.0f;
    if (q > n + 1.0f) q = n + 1.0f;
    int c = (int)q;
    if (c == n && v == bmax) c--;
    return c;
}

/* ------------------------------------------------------------------------------------------ */
/* Voxelization run                                                                             */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    orc_spec s;
    orc_tables t;
    const float *tris;
    int64_t T;
    int64_t N1, B;
    uint8_t *state1;     /* 0 outside, 1 inside, 2 boundary */
    uint8_t *parity;     /* the inside fill alone (before the boundary marks), 0/1 */
    int32_t *prefix;     /* boundaryPrefixSum */
    int32_t *bindex;     /* boundaryIndex */
    int64_t *vstart;     /* per-voxel triangle list CSR (size N1+1) */
    int32_t *vtris;      /* triangle ids in objTriangleID order within each voxel */
    int64_t sat1_tests;  /* sum over triangles of the candidate box size */
    int64_t ray1_cand;   /* (column,triangle) pairs in the triangles' exact x/y boxes, times nz */
    int fill;            /* ORC_FILL_* */
} orc_run;

/* ---- Stencil fill --------------------------------------------------------------------------
 * One rendering of the reference draws triangles into an orthographic viewport of W x H pixels
 * over [lx, hx] x [ly, hy] with the clip plane (0, 0, -1, c) (keeps z <= c), GL_INCR on the
 * stencil of every fragment.  Restated: window coordinates ((v - lo) / (hi - lo)) * W in float,
 * snapped to 1/256 pixel (clamped to +-2^21 pixels); a pixel centre (s + 1/2) is covered when
 * the three integer edge functions of the counter-clockwise snapped triangle are positive, or
 * zero on a left edge (dy < 0) or a bottom edge (dy == 0, dx > 0); the height there is
 * sum_i (w_i * (1/A)) * z_i in float; the fragment survives the clip when height <= c. */
static int orc_first_ge(const float *tab, int n, float x);

typedef struct {
    int32_t X[3], Y[3];
    float z[3];
    float rA;
    int sx0, sx1, sy0, sy1;
} orc_sttri;

static int32_t orc_st_snap(float v, float lo, float hi, int npx)
{
    float w = ((v - lo) / (hi - lo)) * (float)npx;
    if (!(w > -2097152.0f)) w = -2097152.0f;
    else if (w > 2097152.0f) w = 2097152.0f;
    return (int32_t)llrintf(w * 256.0f);
}

static int32_t orc_floor256(int32_t x) { return x >= 0 ? x / 256 : -((-x + 255) / 256); }

static int orc_st_setup(const float *tv, float lx, float hx, float ly, float hy, int W, int H,
                        orc_sttri *t)
{
    for (int i = 0; i < 3; ++i) {
        t->X[i] = orc_st_snap(tv[3 * i], lx, hx, W);
        t->Y[i] = orc_st_snap(tv[3 * i + 1], ly, hy, H);
        t->z[i] = tv[3 * i + 2];
    }
    int64_t A = (int64_t)(t->X[1] - t->X[0]) * (t->Y[2] - t->Y[0]) -
                (int64_t)(t->Y[1] - t->Y[0]) * (t->X[2] - t->X[0]);
    if (A == 0) return 0; /* zero area: no fragments */
    if (A < 0) {
        int32_t a = t->X[1]; t->X[1] = t->X[2]; t->X[2] = a;
        a = t->Y[1]; t->Y[1] = t->Y[2]; t->Y[2] = a;
        float f = t->z[1]; t->z[1] = t->z[2]; t->z[2] = f;
        A = -A;
    }
    t->rA = 1.0f / (float)A;
    int32_t xmn = t->X[0], xmx = t->X[0], ymn = t->Y[0], ymx = t->Y[0];
    for (int i = 1; i < 3; ++i) {
        if (t->X[i] < xmn) xmn = t->X[i];
        if (t->X[i] > xmx) xmx = t->X[i];
        if (t->Y[i] < ymn) ymn = t->Y[i];
        if (t->Y[i] > ymx) ymx = t->Y[i];
    }
    t->sx0 = -orc_floor256(128 - xmn);
    t->sx1 = orc_floor256(xmx - 128);
    t->sy0 = -orc_floor256(128 - ymn);
    t->sy1 = orc_floor256(ymx - 128);
    if (t->sx0 < 0) t->sx0 = 0;
    if (t->sy0 < 0) t->sy0 = 0;
    if (t->sx1 > W - 1) t->sx1 = W - 1;
    if (t->sy1 > H - 1) t->sy1 = H - 1;
    return t->sx0 <= t->sx1 && t->sy0 <= t->sy1;
}

static int orc_st_edge(int64_t w, int32_t dx, int32_t dy)
{
    return w > 0 || (w == 0 && (dy < 0 || (dy == 0 && dx > 0)));
}

static int orc_st_cover(const orc_sttri *t, int sx, int sy, float *zs)
{
    int64_t px = (int64_t)sx * 256 + 128, py = (int64_t)sy * 256 + 128;
    int64_t w[3];
    for (int e = 0; e < 3; ++e) {
        int a = (e + 1) % 3, b = (e + 2) % 3; /* edge opposite vertex e, counter-clockwise */
        int32_t dx = t->X[b] - t->X[a], dy = t->Y[b] - t->Y[a];
        w[e] = (int64_t)dx * (py - t->Y[a]) - (int64_t)dy * (px - t->X[a]);
        if (!orc_st_edge(w[e], dx, dy)) return 0;
    }
    *zs = ((float)w[0] * t->rA) * t->z[0] + ((float)w[1] * t->rA) * t->z[1];
    *zs = *zs + ((float)w[2] * t->rA) * t->z[2];
    return 1;
}

static int orc_tri_finite(const float *tv)
{
    for (int k = 0; k < 9; ++k)
        if (!isfinite(tv[k])) return 0;
    return 1;
}

/* ClassifyInOut2x: per slice k the stencil counts of the 2nx x 2ny samples over the bounding
 * box, clip height (k + 0.5)*gridSizeZ + bBoxMin[2] (double, stored as float); a voxel is inside
 * when more than 2 of its 4 counts are odd.  A fragment at height zs counts in slices k >= k0
 * (the first clip height >= zs), so the counts are accumulated per (sample, slice) parity. */
static void orc_fill_stencil1(orc_run *r)
{
    const int nx = r->s.n[0], ny = r->s.n[1], nz = r->s.n[2];
    const int W = 2 * nx, H = 2 * ny;
    float *clip = (float *)malloc(sizeof(float) * (size_t)nz);
    for (int k = 0; k < nz; ++k) clip[k] = (float)((k + 0.5) * (double)r->t.g[2] + (double)r->s.bmin[2]);
    uint8_t *par = (uint8_t *)calloc((size_t)W * H * nz, 1);
    for (int64_t t = 0; t < r->T; ++t) {
        const float *tv = r->tris + 9 * t;
        orc_sttri st;
        if (!orc_tri_finite(tv)) continue;
        if (!orc_st_setup(tv, r->s.bmin[0], r->s.bmax[0], r->s.bmin[1], r->s.bmax[1], W, H, &st)) continue;
        for (int sy = st.sy0; sy <= st.sy1; ++sy)
            for (int sx = st.sx0; sx <= st.sx1; ++sx) {
                float zs;
                if (!orc_st_cover(&st, sx, sy, &zs)) continue;
                uint8_t *c = par + ((size_t)sy * W + sx) * nz;
                for (int k = orc_first_ge(clip, nz, zs); k < nz; ++k) c[k] ^= 1;
            }
    }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int cnt = 0;
                for (int l = 0; l < 2; ++l)
                    for (int m = 0; m < 2; ++m) cnt += par[((size_t)(2 * j + l) * W + 2 * i + m) * nz + k];
                r->state1[((int64_t)k * ny + j) * nx + i] = cnt > 2 ? 1 : 0;
            }
    free(par);
    free(clip);
}

static int orc_threads(int req)
{
#ifdef _OPENMP
    return req > 0 ? req : omp_get_max_threads();
#else
    (void)req;
    return 1;
#endif
}

/* Conservative x/y candidate test used by ORC_FILL_CAND.  The margin is a generous multiple of
 * the float rounding bound of the u/v tests; triangles whose projection is ill-conditioned
 * (det rounding bound comparable to det) are tested against every column. */
typedef struct { float lo[2], hi[2]; int all, none; } orc_xybox;

static void orc_xy_box(const float *tv, float gx, float gy, orc_xybox *b)
{
    float e1x = tv[3] - tv[0], e1y = tv[4] - tv[1];
    float e2x = tv[6] - tv[0], e2y = tv[7] - tv[1];
    /* the float determinant of the test itself: when it fails the 1e-6 test no column passes */
    float detf = e1x * (-e2y) + e1y * e2x;
    double det = detf;
    double sd = fabs((double)e1x * e2y) + fabs((double)e1y * e2x);
    const double eps = 5.9604644775390625e-08; /* 2^-24 */
    b->all = 0;
    b->none = 0;
    if (det > -0.000001 && det < 0.000001) { b->none = 1; return; }
    if (64.0 * eps * sd >= fabs(det)) { b->all = 1; return; }
    double G = gx > gy ? gx : gy;
    double au = 64.0 * eps * G * (fabs(e2x) + fabs(e2y)) / fabs(det);
    double av = 64.0 * eps * G * (fabs(e1x) + fabs(e1y)) / fabs(det);
    double rel = 64.0 * eps * sd / fabs(det);
    double mu = 4.0 * (rel + au + av) + 1e-5;
    for (int a = 0; a < 2; ++a) {
        float mn = tv[a], mx = tv[a];
        if (tv[3 + a] < mn) mn = tv[3 + a];
        if (tv[3 + a] > mx) mx = tv[3 + a];
        if (tv[6 + a] < mn) mn = tv[6 + a];
        if (tv[6 + a] > mx) mx = tv[6 + a];
        double w = (double)mx - mn;
        double m = 2.0 * mu * w + 1e-4 * (fabs((double)mn) + fabs((double)mx)) + 1e-6;
        b->lo[a] = (float)(mn - m);
        b->hi[a] = (float)(mx + m);
    }
}

/* first index with tab[i] >= x (n if none), last index with tab[i] <= x (-1 if none) */
static int orc_first_ge(const float *tab, int n, float x)
{
    int lo = 0, hi = n;
    while (lo < hi) { int m = (lo + hi) / 2; if (tab[m] >= x) hi = m; else lo = m + 1; }
    return lo;
}
static int orc_last_le(const float *tab, int n, float x)
{
    int lo = 0, hi = n;
    while (lo < hi) { int m = (lo + hi) / 2; if (tab[m] > x) hi = m; else lo = m + 1; }
    return lo - 1;
}

/* Level1 inside fill (ClassifyInOutCPU semantics) into st[] as 1 for odd hit counts. */
static void orc_fill_level1(orc_run *r, int mode, int nth)
{
    const int nx = r->s.n[0], ny = r->s.n[1], nz = r->s.n[2];
    const float *cx = r->t.c1[0], *cy = r->t.c1[1], *cz = r->t.c1[2];
    const int64_t T = r->T;
    if (mode == ORC_FILL_VOXEL) {
        const float D[3] = {0.f, 0.f, 1.f};
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
        for (int64_t col = 0; col < (int64_t)nx * ny; ++col) {
            int i = (int)(col % nx), j = (int)(col / nx);
            for (int k = 0; k < nz; ++k) {
                float O[3] = {cx[i], cy[j], cz[k]};
                int cnt = 0;
                for (int64_t t = 0; t < T; ++t) {
                    const float *tv = r->tris + 9 * t;
                    float tt;
                    if (orc_tri_ray(tv, tv + 3, tv + 6, O, D, &tt)) cnt++;
                }
                if (cnt % 2 == 1) r->state1[(int64_t)k * ny * nx + (int64_t)j * nx + i] = 1;
            }
        }
        return;
    }
    if (mode == ORC_FILL_COLUMN) {
#pragma omp parallel num_threads(nth)
        {
            uint8_t *par = (uint8_t *)calloc((size_t)nz, 1);
#pragma omp for schedule(dynamic, 4)
            for (int64_t col = 0; col < (int64_t)nx * ny; ++col) {
                int i = (int)(col % nx), j = (int)(col / nx);
                memset(par, 0, (size_t)nz);
                for (int64_t t = 0; t < T; ++t) {
                    orc_colhit s;
                    if (!orc_ray_column(r->tris + 9 * t, cx[i], cy[j], &s)) continue;
                    for (int k = 0; k < nz; ++k) par[k] ^= (uint8_t)orc_ray_t(&s, cz[k]);
                }
                for (int k = 0; k < nz; ++k)
                    if (par[k]) r->state1[(int64_t)k * ny * nx + (int64_t)j * nx + i] = 1;
            }
            free(par);
        }
        return;
    }
    /* ORC_FILL_CAND: bin triangles to columns by conservative x/y boxes. */
    int64_t ncol = (int64_t)nx * ny;
    int64_t *cnt = (int64_t *)calloc((size_t)ncol + 1, sizeof(int64_t));
    orc_xybox *bx = (orc_xybox *)malloc(sizeof(orc_xybox) * (size_t)(T > 0 ? T : 1));
    int *rng = (int *)malloc(sizeof(int) * 4 * (size_t)(T > 0 ? T : 1));
    int64_t nall = 0;
    for (int64_t t = 0; t < T; ++t) {
        orc_xy_box(r->tris + 9 * t, r->t.g[0], r->t.g[1], &bx[t]);
        int *q = rng + 4 * t;
        if (bx[t].none) { q[0] = 1; q[1] = 0; q[2] = 1; q[3] = 0; }
        else if (bx[t].all) { q[0] = 0; q[1] = nx - 1; q[2] = 0; q[3] = ny - 1; nall++; }
        else {
            /* columns whose centre lies in [lo,hi] of the monotone centre tables */
            q[0] = orc_first_ge(cx, nx, bx[t].lo[0]);
            q[1] = orc_last_le(cx, nx, bx[t].hi[0]);
            q[2] = orc_first_ge(cy, ny, bx[t].lo[1]);
            q[3] = orc_last_le(cy, ny, bx[t].hi[1]);
        }
        for (int j = q[2]; j <= q[3]; ++j)
            for (int i = q[0]; i <= q[1]; ++i) cnt[(int64_t)j * nx + i + 1]++;
    }
    for (int64_t c = 0; c < ncol; ++c) cnt[c + 1] += cnt[c];
    int64_t tot = cnt[ncol];
    int32_t *lst = (int32_t *)malloc(sizeof(int32_t) * (size_t)(tot > 0 ? tot : 1));
    int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)ncol);
    memcpy(pos, cnt, sizeof(int64_t) * (size_t)ncol);
    for (int64_t t = 0; t < T; ++t) {
        int *q = rng + 4 * t;
        for (int j = q[2]; j <= q[3]; ++j)
            for (int i = q[0]; i <= q[1]; ++i) lst[pos[(int64_t)j * nx + i]++] = (int32_t)t;
    }
#pragma omp parallel num_threads(nth)
    {
        uint8_t *par = (uint8_t *)calloc((size_t)nz, 1);
#pragma omp for schedule(dynamic, 4)
        for (int64_t col = 0; col < ncol; ++col) {
            int i = (int)(col % nx), j = (int)(col / nx);
            memset(par, 0, (size_t)nz);
            for (int64_t e = cnt[col]; e < cnt[col + 1]; ++e) {
                orc_colhit s;
                if (!orc_ray_column(r->tris + 9 * (int64_t)lst[e], cx[i], cy[j], &s)) continue;
                for (int k = 0; k < nz; ++k) par[k] ^= (uint8_t)orc_ray_t(&s, cz[k]);
            }
            for (int k = 0; k < nz; ++k)
                if (par[k]) r->state1[(int64_t)k * ny * nx + (int64_t)j * nx + i] = 1;
        }
        free(par);
    }
    free(pos); free(lst); free(rng); free(bx); free(cnt);
}

/* Candidate Level1 box of a triangle (src/Object.cpp:2280-2325).  Lower bounds are clamped at
 * 0: a vertex below bBoxMin would index before the grid in the reference (undefined there). */
static void orc_tri_range(const orc_run *r, const float *tv, int lo[3], int hi[3])
{
    for (int a = 0; a < 3; ++a) {
        int c0 = orc_cell(tv[a], r->s.bmin[a], r->s.bmax[a], r->s.n[a]);
        int c1 = orc_cell(tv[3 + a], r->s.bmin[a], r->s.bmax[a], r->s.n[a]);
        int c2 = orc_cell(tv[6 + a], r->s.bmin[a], r->s.bmax[a], r->s.n[a]);
        int mn = c0 < c1 ? c0 : c1; mn = mn < c2 ? mn : c2;
        int mx = c0 > c1 ? c0 : c1; mx = mx > c2 ? mx : c2;
        if (mn < 0) mn = 0;
        if (mx > r->s.n[a] - 1) mx = r->s.n[a] - 1;
        lo[a] = mn; hi[a] = mx;
    }
}

/* Level1 SAT + per-voxel triangle lists (ClassifyTessellation + AddPointToVoxel). */
static void orc_sat_level1(orc_run *r, int nth)
{
    const int nx = r->s.n[0], ny = r->s.n[1];
    const int64_t T = r->T;
    /* pass 1: per-triangle pass lists (parallel), pass 2: ordered CSR build. */
    int64_t *tcnt = (int64_t *)calloc((size_t)T + 1, sizeof(int64_t));
    int64_t sat_tests = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : sat_tests) num_threads(nth)
    for (int64_t t = 0; t < T; ++t) {
        int lo[3], hi[3];
        orc_tri_range(r, r->tris + 9 * t, lo, hi);
        int64_t c = 0;
        for (int p = lo[0]; p <= hi[0]; ++p)
            for (int q = lo[1]; q <= hi[1]; ++q)
                for (int k = lo[2]; k <= hi[2]; ++k) {
                    float c3[3] = {r->t.c1[0][p], r->t.c1[1][q], r->t.c1[2][k]};
                    if (orc_tri_box(c3, r->t.e1, r->tris + 9 * t)) c++;
                }
        tcnt[t + 1] = c;
        sat_tests += (int64_t)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    }
    r->sat1_tests = sat_tests;
    for (int64_t t = 0; t < T; ++t) tcnt[t + 1] += tcnt[t];
    int64_t P = tcnt[T];
    int64_t *pv = (int64_t *)malloc(sizeof(int64_t) * (size_t)(P > 0 ? P : 1));
#pragma omp parallel for schedule(dynamic, 256) num_threads(nth)
    for (int64_t t = 0; t < T; ++t) {
        int lo[3], hi[3];
        orc_tri_range(r, r->tris + 9 * t, lo, hi);
        int64_t w = tcnt[t];
        for (int p = lo[0]; p <= hi[0]; ++p)
            for (int q = lo[1]; q <= hi[1]; ++q)
                for (int k = lo[2]; k <= hi[2]; ++k) {
                    float c3[3] = {r->t.c1[0][p], r->t.c1[1][q], r->t.c1[2][k]};
                    if (orc_tri_box(c3, r->t.e1, r->tris + 9 * t))
                        pv[w++] = (int64_t)k * ny * nx + (int64_t)q * nx + p;
                }
    }
    r->vstart = (int64_t *)calloc((size_t)r->N1 + 1, sizeof(int64_t));
    for (int64_t e = 0; e < P; ++e) r->vstart[pv[e] + 1]++;
    for (int64_t v = 0; v < r->N1; ++v) r->vstart[v + 1] += r->vstart[v];
    r->vtris = (int32_t *)malloc(sizeof(int32_t) * (size_t)(P > 0 ? P : 1));
    int64_t *fillp = (int64_t *)malloc(sizeof(int64_t) * (size_t)r->N1);
    memcpy(fillp, r->vstart, sizeof(int64_t) * (size_t)r->N1);
    for (int64_t t = 0; t < T; ++t)
        for (int64_t e = tcnt[t]; e < tcnt[t + 1]; ++e) {
            int64_t v = pv[e];
            r->vtris[fillp[v]++] = (int32_t)t;
            r->state1[v] = 2;
        }
    free(fillp); free(pv); free(tcnt);
}

orc_run *orc_create(const float *tris, int64_t T, const orc_spec *s, int fill_mode, int nthreads)
{
    int nth = orc_threads(nthreads);
    orc_run *r = (orc_run *)calloc(1, sizeof(orc_run));
    r->s = *s;
    r->tris = tris;
    r->T = T;
    orc_tables_build(s, &r->t);
    r->N1 = (int64_t)s->n[0] * s->n[1] * s->n[2];
    r->state1 = (uint8_t *)calloc((size_t)r->N1, 1);
    r->fill = fill_mode;
    if (fill_mode == ORC_FILL_STENCIL) orc_fill_stencil1(r);
    else orc_fill_level1(r, fill_mode, nth);
    r->parity = (uint8_t *)malloc((size_t)r->N1);
    memcpy(r->parity, r->state1, (size_t)r->N1);
    orc_sat_level1(r, nth);
    /* Compaction (src/Object.cpp:3271-3279): exclusive count of value 2 in linear order. */
    r->prefix = (int32_t *)malloc(sizeof(int32_t) * (size_t)r->N1);
    int64_t B = 0;
    for (int64_t v = 0; v < r->N1; ++v) {
        r->prefix[v] = (int32_t)B;
        if (r->state1[v] == 2) B++;
    }
    r->B = B;
    r->bindex = (int32_t *)malloc(sizeof(int32_t) * (size_t)(B > 0 ? B : 1));
    for (int64_t v = 0, b = 0; v < r->N1; ++v)
        if (r->state1[v] == 2) r->bindex[b++] = (int32_t)v;
    /* Exact-box candidate count for the Level1 ray work unit. */
    int64_t rc = 0;
    const int nx = s->n[0], ny = s->n[1];
    for (int64_t t = 0; t < T; ++t) {
        const float *tv = tris + 9 * t;
        int cnt[2];
        for (int a = 0; a < 2; ++a) {
            float mn = tv[a], mx = tv[a];
            for (int w = 1; w < 3; ++w) {
                if (tv[3 * w + a] < mn) mn = tv[3 * w + a];
                if (tv[3 * w + a] > mx) mx = tv[3 * w + a];
            }
            int n = a == 0 ? nx : ny;
            int c = orc_last_le(r->t.c1[a], n, mx) - orc_first_ge(r->t.c1[a], n, mn) + 1;
            cnt[a] = c > 0 ? c : 0;
        }
        rc += (int64_t)cnt[0] * cnt[1];
    }
    r->ray1_cand = fill_mode == ORC_FILL_STENCIL ? 0 : rc * s->n[2];
    return r;
}

void orc_free(orc_run *r)
{
    if (!r) return;
    orc_tables_free(&r->t);
    free(r->state1); free(r->parity); free(r->prefix); free(r->bindex); free(r->vstart); free(r->vtris);
    free(r);
}

int64_t orc_num_boundary(const orc_run *r) { return r->B; }
int64_t orc_num_pairs(const orc_run *r) { return r->vstart[r->N1]; }
int64_t orc_sat1_tests(const orc_run *r) { return r->sat1_tests; }
int64_t orc_ray1_candidates(const orc_run *r) { return r->ray1_cand; }
void orc_level1_state(const orc_run *r, uint8_t *out) { memcpy(out, r->state1, (size_t)r->N1); }
void orc_prefix(const orc_run *r, int32_t *out) { memcpy(out, r->prefix, sizeof(int32_t) * (size_t)r->N1); }
void orc_boundary_index(const orc_run *r, int32_t *out)
{
    memcpy(out, r->bindex, sizeof(int32_t) * (size_t)r->B);
}
/* Per-voxel triangle list (objTriangles order) of Level1 voxel v; returns its length. */
int64_t orc_voxel_tris(const orc_run *r, int64_t v, int32_t *out, int64_t cap)
{
    int64_t n = r->vstart[v + 1] - r->vstart[v];
    for (int64_t e = 0; e < n && e < cap; ++e) out[e] = r->vtris[r->vstart[v] + e];
    return n;
}

/* ClassifyInOut2xLevel2 for the boundary voxel (i, j, k): 2 n2x x 2 n2y samples over the voxel's
 * x/y extent (minX = i*gridSizeX + bBoxMin[0] in float, maxX = minX + gridSizeX, :1241-1266),
 * slice s clipped at minZ + (s + 0.5)*gridSizeZ2 (double, stored as float: the Level2 ray-origin
 * heights), drawing the triangles recorded in the Level1 column (i, j) -- the strip display list
 * of CreateVoxelStripDisplayLists (:605-633), each triangle once.  blk receives 1 for inside. */
static void orc_fill_stencil2(const orc_run *r, int i, int j, int k, uint8_t *blk)
{
    const int nx = r->s.n[0], ny = r->s.n[1], nz = r->s.n[2];
    const int n2x = r->s.n2[0], n2y = r->s.n2[1], n2z = r->s.n2[2];
    const int W = 2 * n2x, H = 2 * n2y;
    const float lx = i * r->t.g[0] + r->s.bmin[0], hx = lx + r->t.g[0];
    const float ly = j * r->t.g[1] + r->s.bmin[1], hy = ly + r->t.g[1];
    const float *clip = r->t.o2[2] + (size_t)k * n2z;
    uint8_t *par = (uint8_t *)calloc((size_t)W * H * n2z, 1);
    uint8_t *seen = (uint8_t *)calloc((size_t)r->T + 1, 1);
    const int64_t ij = (int64_t)j * nx + i;
    for (int z = 0; z < nz; ++z) {
        const int64_t w = (int64_t)z * nx * ny + ij;
        for (int64_t e = r->vstart[w]; e < r->vstart[w + 1]; ++e) {
            const int32_t t = r->vtris[e];
            if (seen[t]) continue;
            seen[t] = 1;
            orc_sttri st;
            if (!orc_st_setup(r->tris + 9 * (int64_t)t, lx, hx, ly, hy, W, H, &st)) continue;
            for (int sy = st.sy0; sy <= st.sy1; ++sy)
                for (int sx = st.sx0; sx <= st.sx1; ++sx) {
                    float zs;
                    if (!orc_st_cover(&st, sx, sy, &zs)) continue;
                    uint8_t *c = par + ((size_t)sy * W + sx) * n2z;
                    for (int s2 = orc_first_ge(clip, n2z, zs); s2 < n2z; ++s2) c[s2] ^= 1;
                }
        }
    }
    for (int s2 = 0; s2 < n2z; ++s2)
        for (int q = 0; q < n2y; ++q)
            for (int p = 0; p < n2x; ++p) {
                int cnt = 0;
                for (int l = 0; l < 2; ++l)
                    for (int m = 0; m < 2; ++m) cnt += par[((size_t)(2 * q + l) * W + 2 * p + m) * n2z + s2];
                if (cnt > 2) blk[((int64_t)s2 * n2y + q) * n2x + p] = 1;
            }
    free(seen);
    free(par);
}

/* Level2 of one boundary voxel b into blk (n2x*n2y*n2z states 0/1/2): ClassifyInOutLevel2CPU
 * then ClassifyTessellationLevel2.  uni/ucap/mark/par are the calling thread's scratch (mark all
 * zero on entry and exit); the algorithmic Level2 test counts are added to *s2 and *r2. */
static void orc_level2_voxel(const orc_run *r, int64_t b, uint8_t *blk, int32_t **uni_p,
                             int64_t *ucap_p, uint8_t *mark, uint8_t *par, int64_t *s2, int64_t *r2)
{
    const int nx = r->s.n[0], ny = r->s.n[1], nz = r->s.n[2];
    const int n2x = r->s.n2[0], n2y = r->s.n2[1], n2z = r->s.n2[2];
    const int64_t cells = (int64_t)n2x * n2y * n2z;
    int32_t *uni = *uni_p;
    int64_t ucap = *ucap_p;
    memset(blk, 0, (size_t)cells);
    int64_t v = r->bindex[b];
    int k = (int)(v / ((int64_t)nx * ny));
    int64_t ij = v - (int64_t)k * nx * ny;
    int j = (int)(ij / nx), i = (int)(ij % nx);
    /* Union of the triangles of Level1 voxels (i,j,z>=k), each once (:1162-1193). */
    int64_t nu = 0;
    for (int z = k; z < nz; ++z) {
        int64_t w = (int64_t)z * nx * ny + ij;
        for (int64_t e = r->vstart[w]; e < r->vstart[w + 1]; ++e) {
            int32_t t = r->vtris[e];
            if (mark[t]) continue;
            mark[t] = 1;
            if (nu == ucap) {
                ucap = ucap ? 2 * ucap : 256;
                uni = (int32_t *)realloc(uni, sizeof(int32_t) * (size_t)ucap);
            }
            uni[nu++] = t;
        }
    }
    for (int64_t e = 0; e < nu; ++e) mark[uni[e]] = 0;
    *uni_p = uni;
    *ucap_p = ucap;
    if (r->fill == ORC_FILL_STENCIL) {
        orc_fill_stencil2(r, i, j, k, blk);
    } else {
        *r2 += nu * cells;
        const float *ox = r->t.o2[0] + (size_t)i * n2x;
        const float *oy = r->t.o2[1] + (size_t)j * n2y;
        const float *oz = r->t.o2[2] + (size_t)k * n2z;
        for (int q = 0; q < n2y; ++q)
            for (int p = 0; p < n2x; ++p) {
                memset(par, 0, (size_t)n2z);
                for (int64_t e = 0; e < nu; ++e) {
                    orc_colhit s;
                    if (!orc_ray_column(r->tris + 9 * (int64_t)uni[e], ox[p], oy[q], &s)) continue;
                    for (int rr = 0; rr < n2z; ++rr) par[rr] ^= (uint8_t)orc_ray_t(&s, oz[rr]);
                }
                for (int rr = 0; rr < n2z; ++rr)
                    if (par[rr]) blk[((int64_t)rr * n2y + q) * n2x + p] = 1;
            }
    }
    /* Level2 SAT over every sub-cell for every triangle of the voxel (:2374-2398). */
    const float *sx = r->t.c2s[0] + (size_t)i * n2x;
    const float *sy = r->t.c2s[1] + (size_t)j * n2y;
    const float *sz = r->t.c2s[2] + (size_t)k * n2z;
    int64_t nt = r->vstart[v + 1] - r->vstart[v];
    *s2 += nt * cells;
    for (int64_t e = r->vstart[v]; e < r->vstart[v + 1]; ++e) {
        const float *tv = r->tris + 9 * (int64_t)r->vtris[e];
        for (int p = 0; p < n2x; ++p)
            for (int q = 0; q < n2y; ++q)
                for (int rr = 0; rr < n2z; ++rr) {
                    float c3[3] = {sx[p], sy[q], sz[rr]};
                    if (orc_tri_box(c3, r->t.e2, tv)) blk[((int64_t)rr * n2y + q) * n2x + p] = 2;
                }
    }
}

/* Level2 of the boundary voxels list[0..n) (list == NULL: voxels b0 + 0..n) in one parallel
 * region; out receives n blocks of n2x*n2y*n2z states in list order. */
static void orc_level2_many(const orc_run *r, int64_t b0, int64_t n, const int64_t *list,
                            uint8_t *out, int nthreads, int64_t *sat2_tests, int64_t *ray2_tests)
{
    int nth = orc_threads(nthreads);
    const int n2z = r->s.n2[2];
    const int64_t cells = (int64_t)r->s.n2[0] * r->s.n2[1] * n2z;
    int64_t s2 = 0, r2 = 0;
#pragma omp parallel num_threads(nth) reduction(+ : s2, r2)
    {
        int32_t *uni = NULL;
        int64_t ucap = 0;
        uint8_t *mark = (uint8_t *)calloc((size_t)r->T + 1, 1);
        uint8_t *par = (uint8_t *)malloc((size_t)(n2z > 0 ? n2z : 1));
#pragma omp for schedule(dynamic, 1)
        for (int64_t e = 0; e < n; ++e)
            orc_level2_voxel(r, list ? list[e] : b0 + e, out + e * cells, &uni, &ucap, mark, par,
                             &s2, &r2);
        free(uni); free(mark); free(par);
    }
    if (sat2_tests) *sat2_tests = s2;
    if (ray2_tests) *ray2_tests = r2;
}

/* Level2 of boundary voxels [b0, b1): ClassifyInOutLevel2CPU then ClassifyTessellationLevel2.
 * out receives (b1-b0)*n2x*n2y*n2z states (0/1/2) in the reference's block layout.
 * Also accumulates the algorithmic Level2 test counts. */
void orc_level2(const orc_run *r, int64_t b0, int64_t b1, uint8_t *out, int nthreads,
                int64_t *sat2_tests, int64_t *ray2_tests)
{
    orc_level2_many(r, b0, b1 > b0 ? b1 - b0 : 0, NULL, out, nthreads, sat2_tests, ray2_tests);
}

/* Level2 of the listed boundary voxels (any order, e.g. a strided sample), one block each. */
void orc_level2_list(const orc_run *r, int64_t n, const int64_t *list, uint8_t *out,
                     int nthreads, int64_t *sat2_tests, int64_t *ray2_tests)
{
    orc_level2_many(r, 0, n, list, out, nthreads, sat2_tests, ray2_tests);
}

/* ClassifyInOutCPU as the reference writes it (src/Object.cpp:716-779), on a sample of Level1
 * columns, on the calling thread: every voxel centre of column cols[c] = j*nx + i against every
 * triangle with the general-direction ray test (D = +z), parity into out[c*nz + k] (1 = odd).
 * Timing it gives the reference's single-threaded brute-force fill cost per column. */
void orc_voxel_fill_columns(const orc_run *r, int64_t ncols, const int64_t *cols, uint8_t *out)
{
    const int nx = r->s.n[0], nz = r->s.n[2];
    const float D[3] = {0.f, 0.f, 1.f};
    for (int64_t c = 0; c < ncols; ++c) {
        const int i = (int)(cols[c] % nx), j = (int)(cols[c] / nx);
        for (int k = 0; k < nz; ++k) {
            float O[3] = {r->t.c1[0][i], r->t.c1[1][j], r->t.c1[2][k]};
            int cnt = 0;
            for (int64_t t = 0; t < r->T; ++t) {
                const float *tv = r->tris + 9 * t;
                float tt;
                if (orc_tri_ray(tv, tv + 3, tv + 6, O, D, &tt)) cnt++;
            }
            out[c * nz + k] = (uint8_t)(cnt & 1);
        }
    }
}

/* The algorithmic Level2 test counts of orc_level2 over every boundary voxel, without running
 * the predicates: sat2 = sum of |tris(b)| * n2^3, ray2 = sum of |column union(b)| * n2^3, the
 * union being the triangles of Level1 voxels (i,j,z>=k) counted once (src/Object.cpp:1162-1193).
 * Used to state a sampled CPU timing per whole mesh. */
void orc_level2_work(const orc_run *r, int nthreads, int64_t *sat2_tests, int64_t *ray2_tests)
{
    int nth = orc_threads(nthreads);
    const int nx = r->s.n[0], ny = r->s.n[1], nz = r->s.n[2];
    const int64_t cells = (int64_t)r->s.n2[0] * r->s.n2[1] * r->s.n2[2];
    int64_t s2 = 0, r2 = 0;
#pragma omp parallel num_threads(nth) reduction(+ : s2, r2)
    {
        uint8_t *mark = (uint8_t *)calloc((size_t)r->T + 1, 1);
#pragma omp for schedule(dynamic, 64)
        for (int64_t b = 0; b < r->B; ++b) {
            int64_t v = r->bindex[b];
            int k = (int)(v / ((int64_t)nx * ny));
            int64_t ij = v - (int64_t)k * nx * ny;
            int64_t nu = 0;
            for (int z = k; z < nz; ++z) {
                int64_t w = (int64_t)z * nx * ny + ij;
                for (int64_t e = r->vstart[w]; e < r->vstart[w + 1]; ++e)
                    if (!mark[r->vtris[e]]) { mark[r->vtris[e]] = 1; ++nu; }
            }
            for (int z = k; z < nz; ++z) {
                int64_t w = (int64_t)z * nx * ny + ij;
                for (int64_t e = r->vstart[w]; e < r->vstart[w + 1]; ++e) mark[r->vtris[e]] = 0;
            }
            if (r->fill != ORC_FILL_STENCIL) r2 += nu * cells;
            s2 += (r->vstart[v + 1] - r->vstart[v]) * cells;
        }
        free(mark);
    }
    *sat2_tests = s2;
    *ray2_tests = r2;
}

/* Algorithmic FP32 work of the reference predicates over the tests the work counts define,
 * early exits included (operation counts per exit above).  Level1 over the whole mesh, Level2
 * over boundary voxels [b0, b1):
 *   out[0] sat1 ops  (every candidate-box test of every triangle)
 *   out[1] ray1 ops  (every column centre in a triangle's exact x/y box, times nz origins)
 *   out[2] sat2 ops  (every triangle of a boundary voxel against its n2^3 sub-cells)
 *   out[3] ray2 ops  (every triangle of the column union against the n2^3 Level2 origins) */
void orc_count_ops(const orc_run *r, int64_t b0, int64_t b1, int nthreads, int64_t out[4])
{
    int nth = orc_threads(nthreads);
    const int nx = r->s.n[0], ny = r->s.n[1], nz = r->s.n[2];
    const int64_t T = r->T;
    int64_t s1 = 0, r1 = 0, s2 = 0, r2 = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : s1, r1) num_threads(nth)
    for (int64_t t = 0; t < T; ++t) {
        const float *tv = r->tris + 9 * t;
        int lo[3], hi[3], ops;
        orc_tri_range(r, tv, lo, hi);
        for (int p = lo[0]; p <= hi[0]; ++p)
            for (int q = lo[1]; q <= hi[1]; ++q)
                for (int k = lo[2]; k <= hi[2]; ++k) {
                    float c3[3] = {r->t.c1[0][p], r->t.c1[1][q], r->t.c1[2][k]};
                    orc_tri_box_own(c3, r->t.e1, tv, &ops);
                    s1 += ops;
                }
        int clo[2], chi[2];
        for (int a = 0; a < 2; ++a) {
            float mn = tv[a], mx = tv[a];
            for (int w = 1; w < 3; ++w) {
                if (tv[3 * w + a] < mn) mn = tv[3 * w + a];
                if (tv[3 * w + a] > mx) mx = tv[3 * w + a];
            }
            int n = a == 0 ? nx : ny;
            clo[a] = orc_first_ge(r->t.c1[a], n, mn);
            chi[a] = orc_last_le(r->t.c1[a], n, mx);
        }
        for (int j = clo[1]; j <= chi[1]; ++j)
            for (int i = clo[0]; i <= chi[0]; ++i) {
                orc_colhit st;
                orc_ray_column_own(tv, r->t.c1[0][i], r->t.c1[1][j], &st, &ops);
                r1 += (int64_t)ops * nz;
            }
    }
    if (b1 > r->B) b1 = r->B;
    const int n2x = r->s.n2[0], n2y = r->s.n2[1], n2z = r->s.n2[2];
    if (n2x > 0 && b0 < b1) {
#pragma omp parallel num_threads(nth) reduction(+ : s2, r2)
        {
            int32_t *uni = NULL;
            int64_t ucap = 0;
            uint8_t *mark = (uint8_t *)calloc((size_t)r->T + 1, 1);
#pragma omp for schedule(dynamic, 16)
            for (int64_t b = b0; b < b1; ++b) {
                int64_t v = r->bindex[b];
                int k = (int)(v / ((int64_t)nx * ny));
                int64_t ij = v - (int64_t)k * nx * ny;
                int j = (int)(ij / nx), i = (int)(ij % nx);
                int64_t nu = 0;
                for (int z = k; z < nz; ++z) {
                    int64_t w = (int64_t)z * nx * ny + ij;
                    for (int64_t e = r->vstart[w]; e < r->vstart[w + 1]; ++e) {
                        int32_t t = r->vtris[e];
                        if (mark[t]) continue;
                        mark[t] = 1;
                        if (nu == ucap) {
                            ucap = ucap ? 2 * ucap : 256;
                            uni = (int32_t *)realloc(uni, sizeof(int32_t) * (size_t)ucap);
                        }
                        uni[nu++] = t;
                    }
                }
                for (int64_t e = 0; e < nu; ++e) mark[uni[e]] = 0;
                const float *ox = r->t.o2[0] + (size_t)i * n2x;
                const float *oy = r->t.o2[1] + (size_t)j * n2y;
                for (int q = 0; q < n2y; ++q)
                    for (int p = 0; p < n2x; ++p)
                        for (int64_t e = 0; e < nu; ++e) {
                            orc_colhit st;
                            int ops;
                            orc_ray_column_own(r->tris + 9 * (int64_t)uni[e], ox[p], oy[q], &st, &ops);
                            r2 += (int64_t)ops * n2z;
                        }
                const float *sx = r->t.c2s[0] + (size_t)i * n2x;
                const float *sy = r->t.c2s[1] + (size_t)j * n2y;
                const float *sz = r->t.c2s[2] + (size_t)k * n2z;
                for (int64_t e = r->vstart[v]; e < r->vstart[v + 1]; ++e) {
                    const float *tv = r->tris + 9 * (int64_t)r->vtris[e];
                    for (int p = 0; p < n2x; ++p)
                        for (int q = 0; q < n2y; ++q)
                            for (int rr = 0; rr < n2z; ++rr) {
                                float c3[3] = {sx[p], sy[q], sz[rr]};
                                int ops;
                                orc_tri_box_own(c3, r->t.e2, tv, &ops);
                                s2 += ops;
                            }
                }
            }
            free(uni); free(mark);
        }
    }
    out[0] = s1; out[1] = r1; out[2] = s2; out[3] = r2;
}

/* ------------------------------------------------------------------------------------------ */
/* Normals                                                                                     */
/* ------------------------------------------------------------------------------------------ */

/* VectorNormalize (includes/FloatVector.h:333-342): float magnitude, divide when non-zero. */
static void orc_normalize(float a[3])
{
    float mag = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (mag != 0) {
        a[0] /= mag;
        a[1] /= mag;
        a[2] /= mag;
    }
}

/* Face normal of one triangle as the loader and Level1 pass compute it (src/Object.cpp:522-526,
 * :3233-3239): VectorCrossProduct(v1 - v0, v2 - v0) (includes/FloatVector.h:293-296),
 * normalised. */
void orc_face_normal(const float *tv, float out[3])
{
#ifdef ORC_REF_PREDICATES
    ref_face_normal(tv, out);
    return;
#endif
    float a[3], b[3];
    for (int c = 0; c < 3; ++c) { a[c] = tv[3 + c] - tv[c]; b[c] = tv[6 + c] - tv[c]; }
    out[0] = a[1] * b[2] - b[1] * a[2];
    out[1] = a[2] * b[0] - b[2] * a[0];
    out[2] = a[0] * b[1] - b[0] * a[1];
    orc_normalize(out);
}

/* sum / count componentwise, normalised (src/Object.cpp:3247-3248, :2410-2415). */
static void orc_average(const float sum[3], float count, float out[3])
{
#ifdef ORC_REF_PREDICATES
    ref_average_normal(sum, count, out);
    return;
#endif
    out[0] = sum[0] / count; out[1] = sum[1] / count; out[2] = sum[2] / count;
    orc_normalize(out);
}

/* Level1 normals (src/Object.cpp:3219-3253) into out[3*N1]: for every voxel with recorded
 * triangles, the float sum of their face normals in list order (ascending triangle id, the order
 * ClassifyTessellation records them, :2267-2340), divided by the count and normalised; 0 for the
 * other voxels (:3151-3152). */
void orc_level1_normals(const orc_run *r, float *out)
{
    memset(out, 0, sizeof(float) * 3 * (size_t)r->N1);
    for (int64_t v = 0; v < r->N1; ++v) {
        int64_t n = r->vstart[v + 1] - r->vstart[v];
        if (n == 0) continue;
        float sum[3] = {0.f, 0.f, 0.f};
        for (int64_t e = r->vstart[v]; e < r->vstart[v + 1]; ++e) {
            float fn[3];
            orc_face_normal(r->tris + 9 * (int64_t)r->vtris[e], fn);
            sum[0] += fn[0]; sum[1] += fn[1]; sum[2] += fn[2];
        }
        float avg[3];
        orc_average(sum, (float)n, avg);
        out[3 * v + 0] = avg[0]; out[3 * v + 1] = avg[1]; out[3 * v + 2] = avg[2];
    }
}

/* Level2 normals of boundary voxels [b0, b1) into out[3*(b1-b0)*cells], cell order as the Level2
 * states.  Every SAT pass of ClassifyTessellationLevel2 (src/Object.cpp:2374-2398) adds the
 * triangle's face normal and 1 to the cell (AddPointToVoxel, :2715-2719), triangles in list
 * order; the sums are divided by the count and normalised (:2402-2424); cells without a pass
 * stay 0 (:3309-3310). */
void orc_level2_normals(const orc_run *r, int64_t b0, int64_t b1, float *out, int nthreads)
{
    int nth = orc_threads(nthreads);
    const int nx = r->s.n[0], ny = r->s.n[1];
    const int n2x = r->s.n2[0], n2y = r->s.n2[1], n2z = r->s.n2[2];
    const int64_t cells = (int64_t)n2x * n2y * n2z;
    if (b1 > r->B) b1 = r->B;
    if (b0 >= b1 || cells <= 0) return;
#pragma omp parallel num_threads(nth)
    {
        float *acc = (float *)malloc(sizeof(float) * 4 * (size_t)cells);
#pragma omp for schedule(dynamic, 16)
        for (int64_t b = b0; b < b1; ++b) {
            memset(acc, 0, sizeof(float) * 4 * (size_t)cells);
            int64_t v = r->bindex[b];
            int k = (int)(v / ((int64_t)nx * ny));
            int64_t ij = v - (int64_t)k * nx * ny;
            int j = (int)(ij / nx), i = (int)(ij % nx);
            const float *sx = r->t.c2s[0] + (size_t)i * n2x;
            const float *sy = r->t.c2s[1] + (size_t)j * n2y;
            const float *sz = r->t.c2s[2] + (size_t)k * n2z;
            for (int64_t e = r->vstart[v]; e < r->vstart[v + 1]; ++e) {
                const float *tv = r->tris + 9 * (int64_t)r->vtris[e];
                float fn[3];
                orc_face_normal(tv, fn);
                for (int p = 0; p < n2x; ++p)
                    for (int q = 0; q < n2y; ++q)
                        for (int rr = 0; rr < n2z; ++rr) {
                            float c3[3] = {sx[p], sy[q], sz[rr]};
                            if (!orc_tri_box(c3, r->t.e2, tv)) continue;
                            float *a = acc + 4 * (((int64_t)rr * n2y + q) * n2x + p);
                            a[0] += fn[0]; a[1] += fn[1]; a[2] += fn[2]; a[3] += 1;
                        }
            }
            float *o = out + 3 * (b - b0) * cells;
            for (int64_t c = 0; c < cells; ++c) {
                float avg[3] = {0.f, 0.f, 0.f};
                const float *a = acc + 4 * c;
                if (a[3] > 0) orc_average(a, a[3], avg);
                o[3 * c + 0] = avg[0]; o[3 * c + 1] = avg[1]; o[3 * c + 2] = avg[2];
            }
        }
        free(acc);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Voxel box hierarchy                                                                         */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    float mid[3], half[3];
    int32_t solid, child1, child2, index;
} orc_box;

/* CombineBBox (src/Object.cpp:2750-2788): two empty boxes give an empty box; one solid box is
 * copied; two solid boxes give their bounding box as (max+min)/2, (max-min)/2 in float. */
static void orc_combine(const orc_box *a, int32_t ia, const orc_box *b, int32_t ib, orc_box *o)
{
    float mid[3] = {0.f, 0.f, 0.f}, half[3] = {0.f, 0.f, 0.f};
    if (a->solid == 0 && b->solid == 0) {
        o->solid = 0;
    } else if (a->solid == 0) {
        o->solid = 1;
        memcpy(mid, b->mid, sizeof mid); memcpy(half, b->half, sizeof half);
    } else if (b->solid == 0) {
        o->solid = 1;
        memcpy(mid, a->mid, sizeof mid); memcpy(half, a->half, sizeof half);
    } else {
        o->solid = 1;
        for (int c = 0; c < 3; ++c) {
            float amn = a->mid[c] - a->half[c], amx = a->mid[c] + a->half[c];
            float bmn = b->mid[c] - b->half[c], bmx = b->mid[c] + b->half[c];
            /* std::max / std::min: (a < b) ? b : a and (b < a) ? b : a */
            float mx = (amx < bmx) ? bmx : amx, mn = (bmn < amn) ? bmn : amn;
            mid[c] = (mx + mn) / 2.0f;
            half[c] = (mx - mn) / 2.0f;
        }
    }
    memcpy(o->mid, mid, sizeof mid);
    memcpy(o->half, half, sizeof half);
    o->child1 = ia;
    o->child2 = ib;
}

/* Object::BuildHierarchy (src/Object.cpp:2790-2867) over the Level1 voxels: the leaves are the
 * voxel boxes (centre, half size, solid = the inside fill's parity, :3176-3187); level 1 pairs
 * x-neighbours, later levels pair along x, y, z in turn (level % 3) with the reference's fallback
 * when that axis is already one box wide.  out receives N1-1 boxes; level-1 children are the
 * leaf indices (2i, 2i+1).  Returns the number of levels, or -1 unless N1 is a power of two. */
int orc_build_hierarchy(const orc_run *r, orc_box *out)
{
    const int64_t N1 = r->N1;
    if (N1 < 2 || (N1 & (N1 - 1))) return -1;
    int levels = 0;
    for (int64_t x = N1; x > 1; x >>= 1) ++levels;
    const int nx = r->s.n[0], ny = r->s.n[1];
    memset(out, 0, sizeof(orc_box) * (size_t)(N1 - 1));
    int64_t nlev = N1 / 2;
    for (int64_t i = 0; i < nlev; ++i) {
        orc_box leaf[2];
        for (int h = 0; h < 2; ++h) {
            const int64_t v = 2 * i + h;
            const int k = (int)(v / ((int64_t)nx * ny)), j = (int)((v / nx) % ny), q = (int)(v % nx);
            leaf[h].mid[0] = r->t.c1[0][q]; leaf[h].mid[1] = r->t.c1[1][j]; leaf[h].mid[2] = r->t.c1[2][k];
            for (int c = 0; c < 3; ++c) leaf[h].half[c] = r->t.e1[c];
            leaf[h].solid = r->parity[v] % 2;
        }
        orc_combine(&leaf[0], (int32_t)(2 * i), &leaf[1], (int32_t)(2 * i + 1), &out[i]);
        out[i].index = (int32_t)i;
    }
    int dx = r->s.n[0] / 2, dy = r->s.n[1], dz = r->s.n[2];
    int64_t prev = 0, cur = nlev;
    nlev /= 2;
    for (int level = 2; level < levels + 1; ++level) {
        int is = (level % 3 == 1 && dx > 1) ? 2 : 1;
        int js = (level % 3 == 2 && dy > 1) ? 2 : 1;
        int ks = (level % 3 == 0 && dz > 1) ? 2 : 1;
        if (is == 1 && js == 1 && ks == 1) {
            if (dx > 1) is = 2;
            else if (dy > 1) js = 2;
            else if (dz > 1) ks = 2;
        }
        for (int k = 0; k < dz; k += ks)
            for (int j = 0; j < dy; j += js)
                for (int i = 0; i < dx; i += is) {
                    const int64_t i1 = (int64_t)k * dy * dx + (int64_t)j * dx + i;
                    const int64_t i2 = (int64_t)(k / ks) * (dy / js) * (dx / is) + (int64_t)(j / js) * (dx / is) + i / is;
                    const int64_t sk = (int64_t)(ks - 1) * dy * dx + (int64_t)(js - 1) * dx + (is - 1);
                    const orc_box *a = out + prev + i1, *b = out + prev + i1 + sk;
                    orc_combine(a, a->index, b, b->index, out + cur + i2);
                    out[cur + i2].index = (int32_t)(cur + i2);
                }
        if (is == 2) dx /= 2;
        if (js == 2) dy /= 2;
        if (ks == 2) dz /= 2;
        prev += nlev * 2;
        cur += nlev;
        nlev /= 2;
    }
    return levels;
}
