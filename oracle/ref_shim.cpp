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
