"""Generates the golden fixtures in tests/golden/ from the reference's OWN predicate code.

Run here, where the reference sources exist: `python tests/golden/make_golden.py`.  It needs
oracle/_ref/ (built by oracle/build_oracle.py from the reference's src/TriBoxIntersection.cpp
and src/TriRayIntersection.cpp) and writes:

  pred_sat.npz   triangle/box cases and TriBoxOverlap's answers
  pred_ray.npz   ray/triangle cases and triangle_ray_intersection's answers (hit, t)
  normal_face.npz  face normals of the SAT-case triangles from the reference's own vector code
                 (includes/FloatVector.h: VectorCrossProduct, VectorNormalize)
  mesh_*.npz     small meshes (and the reference's cessna.obj at voxelCount 8 and 32) + grids
                 and the full two-level outputs of the reference's CPU
                 composition (E3) evaluated with the reference's predicates, voxel by voxel
                 (ClassifyInOutCPU semantics: every voxel centre against every triangle), plus
                 the Level1 and Level2 normals with the reference's vector arithmetic

The fixtures are small (tens of KB each) and travel with the repository; the GPU machine never
needs the reference.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _ref_pred():
    from oracle import build_oracle

    build_oracle.build()
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_pred.so"))
    vp = C.c_void_p
    L.ref_tri_box.argtypes = [vp, vp, vp]
    L.ref_tri_ray.argtypes = [vp, vp, vp, vp, vp, C.POINTER(C.c_float)]
    L.ref_face_normal.argtypes = [vp, vp]
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def sat_cases(rng, n):
    c = rng.uniform(-1, 2, (n, 3)).astype(np.float32)
    h = np.exp(rng.uniform(np.log(1e-3), np.log(0.3), (n, 3))).astype(np.float32)
    spread = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), (n, 1)))
    tv = (c[:, None, :] + rng.normal(size=(n, 3, 3)) * spread[:, None, :] * 1.5).astype(np.float32)
    k = n // 8
    # vertices exactly on box faces / corners
    sgn = rng.choice([-1.0, 1.0], (k, 3, 3)).astype(np.float32)
    on = (c[:k, None, :] + sgn * h[:k, None, :]).astype(np.float32)
    mask = rng.random((k, 3, 3)) < 0.5
    tv[:k] = np.where(mask, on, tv[:k])
    # degenerate triangles: repeated and collinear vertices
    tv[k:2 * k, 2] = tv[k:2 * k, 0]
    t = rng.random((k, 1)).astype(np.float32)
    tv[2 * k:3 * k, 2] = tv[2 * k:3 * k, 0] + t * (tv[2 * k:3 * k, 1] - tv[2 * k:3 * k, 0])
    # axis-aligned triangles through the box centre plane
    tv[3 * k:4 * k, :, 2] = c[3 * k:4 * k, None, 2]
    return c, h, tv.reshape(n, 9)


def ray_cases(rng, n):
    v = rng.uniform(-1, 2, (n, 3, 3)).astype(np.float32)
    scale = np.exp(rng.uniform(np.log(1e-4), np.log(1.0), (n, 1, 1))).astype(np.float32)
    v = (v[:, :1, :] + (v - v[:, :1, :]) * scale).astype(np.float32)
    e1 = v[:, 1] - v[:, 0]
    e2 = v[:, 2] - v[:, 0]
    a = rng.uniform(-0.2, 1.2, (n, 1)).astype(np.float32)
    b = rng.uniform(-0.2, 1.2, (n, 1)).astype(np.float32)
    o = (v[:, 0] + a * e1 + b * e2).astype(np.float32)
    o[:, 2] -= rng.uniform(-0.5, 1.0, n).astype(np.float32)
    k = n // 8
    # origins on vertices and edges (barycentric 0 / 1), in x/y
    bc = rng.choice([0.0, 0.5, 1.0], (k, 2)).astype(np.float32)
    o[:k, :2] = (v[:k, 0, :2] + bc[:, :1] * e1[:k, :2] + bc[:, 1:] * e2[:k, :2]).astype(np.float32)
    # determinants near the 1e-6 threshold: shrink triangles in x/y
    s = np.sqrt(np.float32(1e-6) / np.maximum(np.abs(e1[k:2 * k, 0] * e2[k:2 * k, 1] - e1[k:2 * k, 1] * e2[k:2 * k, 0]), 1e-30))
    s = (s * rng.uniform(0.9, 1.1, k)).astype(np.float32)
    v[k:2 * k, 1:, :2] = v[k:2 * k, :1, :2] + (v[k:2 * k, 1:, :2] - v[k:2 * k, :1, :2]) * s[:, None, None]
    # origins just below/above the plane (t near 1e-6)
    d = np.zeros((n, 3), np.float32)
    d[:, 2] = 1.0
    m = n // 4
    dirs = rng.normal(size=(m, 3)).astype(np.float32)
    d[-m:] = dirs / np.linalg.norm(dirs, axis=1, keepdims=True)
    return v.reshape(n, 9), o, d


def mesh_cases():
    import gpview_gb300 as gpv

    cases = {}
    t = gpv.gen_uvsphere(21, 24, 12, (0.5, 0.5, 0.5), 0.4, 0.002)
    cases["sphere288"] = (t, gpv.grid_padded(*gpv.mesh_bounds(t), 20, 4))
    t = gpv.gen_torus(22, 32, 16, (0.5, 0.5, 0.5), 0.35, 0.12, 0.01)
    cases["torus1024"] = (t, gpv.grid_padded(*gpv.mesh_bounds(t), (24, 22, 12), (2, 3, 4)))
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5),
         (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)]
    cube = np.concatenate([v[list(q)].reshape(-1) for q in f]).astype(np.float32)
    s = gpv.GridSpec()
    s.bbox_min[:] = (0, 0, 0)
    s.bbox_max[:] = (1, 1, 1)
    s.ndiv[:] = (8, 8, 8)
    s.ndiv2[:] = (4, 4, 4)
    cases["cube_exact"] = (cube, s)
    q, _ = np.linalg.qr(np.random.default_rng(23).normal(size=(3, 3)))
    t = gpv.gen_superellipsoid(23, 20, 10, (0.5, 0.5, 0.5), (0.4, 0.3, 0.25), 0.4, 1.7, q.astype(np.float32))
    cases["superellipsoid400"] = (t, gpv.grid_padded(*gpv.mesh_bounds(t), 16, 4))
    tri = np.array([0.1, 0.2, 0.3, 0.9, 0.25, 0.5, 0.4, 0.8, 0.7], np.float32)
    cases["open_triangle"] = (tri, gpv.grid_padded(*gpv.mesh_bounds(tri), 10, 4))
    return cases


def cessna_cases():
    """The reference's only mesh file (files/cessna.obj, committed here as cessna.obj), loaded with
    the reference's OBJ semantics and sized by its own rule (GLParameters::voxelCount ->
    GetNextDiv4, src/Object.cpp:3094-3107) at voxelCount 8 and 32, voxelCount2 4."""
    import gpview_gb300 as gpv

    obj = gpv.Object()
    obj.ReadObject(os.path.join(HERE, "cessna.obj"))
    obj.CreateFlatTriangleData()
    out = {}
    for vc in (8, 32):
        spec = gpv.grid_reference(obj.bBoxMin, obj.bBoxMax, obj.maxModelSize, vc, 4)
        out[f"cessna_v{vc}"] = (obj.flatCPUTriangleData, spec)
    return out


def main():
    if "--only-cessna" in sys.argv:
        write_meshes(cessna_cases())
        return
    L = _ref_pred()
    rng = np.random.default_rng(20261203)
    n = 8000
    c, h, tv = sat_cases(rng, n)
    out = np.empty(n, np.int8)
    for i in range(n):
        out[i] = L.ref_tri_box(_p(c[i]), _p(h[i]), _p(tv[i]))
    np.savez_compressed(os.path.join(HERE, "pred_sat.npz"), center=c, half=h, tri=tv, hit=out)
    print("pred_sat: pass rate", out.mean())
    fn = np.empty((n, 3), np.float32)
    for i in range(n):
        L.ref_face_normal(_p(tv[i]), _p(fn[i]))
    np.savez_compressed(os.path.join(HERE, "normal_face.npz"), tri=tv, normal=fn)

    v, o, d = ray_cases(rng, n)
    hit = np.empty(n, np.int8)
    tt = np.zeros(n, np.float32)
    for i in range(n):
        t = C.c_float(0.0)
        hit[i] = L.ref_tri_ray(_p(v[i, 0:3].copy()), _p(v[i, 3:6].copy()), _p(v[i, 6:9].copy()),
                               _p(o[i]), _p(d[i]), C.byref(t))
        tt[i] = t.value if hit[i] else 0.0
    np.savez_compressed(os.path.join(HERE, "pred_ray.npz"), tri=v, origin=o, direction=d, hit=hit, t=tt)
    print("pred_ray: hit rate", hit.mean())

    write_meshes(mesh_cases())
    write_meshes(cessna_cases())


def write_meshes(cases):
    """Full two-level outputs and normals of the reference's CPU composition on the reference's
    own predicates (oracle/_ref), brute-force Level1 fill."""
    from oracle import oracle as orc

    for name, (tris, spec) in cases.items():
        run = orc.Run(tris, spec, fill=orc.FILL_VOXEL, ref=True)
        st2, s2, r2 = run.level2_state()
        np.savez_compressed(
            os.path.join(HERE, f"mesh_{name}.npz"), tris=tris,
            bbox_min=np.array(spec.bbox_min, np.float32), bbox_max=np.array(spec.bbox_max, np.float32),
            ndiv=np.array(spec.ndiv, np.int32), ndiv2=np.array(spec.ndiv2, np.int32),
            level1=run.level1_state(), prefix=run.prefix(), bindex=run.boundary_index(), level2=st2,
            work=np.array([run.sat1_tests(), s2, run.ray1_candidates(), r2], np.int64),
            level1_normal=run.level1_normals(), level2_normal=run.level2_normals())
        print(name, "T", tris.size // 9, "B", run.B, "level1", np.bincount(run.level1_state(), minlength=3))


if __name__ == "__main__":
    main()
