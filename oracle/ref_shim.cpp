// ref_shim.cpp -- exports the reference's own CPU predicates (compiled from its sources by
// oracle/build_oracle.py into oracle/_ref/) under C names, so the oracle can be built against
// them and the tests can compare them with the restated predicates.  Test infrastructure only.
//
// Signatures as declared in the reference's includes/Utilities.h:238,240.
int TriBoxOverlap(float boxcenter[3], float boxhalfsize[3], float triverts[3][3]);
int triangle_ray_intersection(const float V1[3], const float V2[3], const float V3[3],
                              const float O[3], const float D[3], float *out);

extern "C" int ref_tri_box(const float c[3], const float h[3], const float *tv) {
  float cc[3] = {c[0], c[1], c[2]}, hh[3] = {h[0], h[1], h[2]};
  float t[3][3] = {{tv[0], tv[1], tv[2]}, {tv[3], tv[4], tv[5]}, {tv[6], tv[7], tv[8]}};
  return TriBoxOverlap(cc, hh, t);
}

extern "C" int ref_tri_ray(const float *V1, const float *V2, const float *V3, const float *O,
                           const float *D, float *out) {
  return triangle_ray_intersection(V1, V2, V3, O, D, out);
}

// The reference's vector helpers (includes/FloatVector.h, header-only, compiled where it lies):
// the face normal of the loaders (src/Object.cpp:522-526) and the averaging of the normal passes
// (:3247-3248, :2410-2415).
#include <cmath>
using namespace std;
#include "FloatVector.h"

extern "C" void ref_face_normal(const float *tv, float *out) {
  Float3 v0(tv[0], tv[1], tv[2]), v1(tv[3], tv[4], tv[5]), v2(tv[6], tv[7], tv[8]);
  Float3 side1 = v1 - v0;
  Float3 side2 = v2 - v0;
  Float3 n = VectorCrossProduct(side1, side2);
  VectorNormalize(n);
  out[0] = n[0]; out[1] = n[1]; out[2] = n[2];
}

// sum / count, normalised (count > 0)
extern "C" void ref_average_normal(const float *sum, float count, float *out) {
  Float3 s(sum[0], sum[1], sum[2]);
  Float3 a = s / count;
  VectorNormalize(a);
  out[0] = a[0]; out[1] = a[1]; out[2] = a[2];
}
