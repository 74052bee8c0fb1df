"""ctypes wrapper of the CPU oracle (gpv_oracle.c).  TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg -- never by the
gpview_gb300 package.  `Oracle(ref=True)` loads the build linked against the reference's own
predicates (oracle/_ref/, present only where the reference sources were available at build time).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FILL_VOXEL, FILL_COLUMN, FILL_CAND, FILL_STENCIL = 0, 1, 2, 3


class Spec(C.Structure):
    _fields_ = [("bmin", C.c_float * 3), ("bmax", C.c_float * 3),
                ("n", C.c_int32 * 3), ("n2", C.c_int32 * 3)]


def lib_path(ref=False):
    return os.path.join(HERE, "_ref", "liboracle_ref.so") if ref else os.path.join(HERE, "liboracle.so")


def available(ref=False):
    return os.path.exists(lib_path(ref))


_libs = {}


def _load(ref=False):
    if ref in _libs:
        return _libs[ref]
    path = lib_path(ref)
    if not os.path.exists(path):
        if ref:
            raise FileNotFoundError(path)
        from oracle import build_oracle  # noqa: WPS433  (build on demand)
        build_oracle.build()
    L = C.CDLL(path)
    vp, i64 = C.c_void_p, C.c_int64
    L.orc_create.argtypes = [vp, i64, C.POINTER(Spec), C.c_int, C.c_int]
    L.orc_create.restype = vp
    L.orc_free.argtypes = [vp]
    for fn in ("orc_num_boundary", "orc_num_pairs", "orc_sat1_tests", "orc_ray1_candidates"):
        getattr(L, fn).argtypes = [vp]
        getattr(L, fn).restype = i64
    L.orc_level1_state.argtypes = [vp, vp]
    L.orc_prefix.argtypes = [vp, vp]
    L.orc_boundary_index.argtypes = [vp, vp]
    L.orc_voxel_tris.argtypes = [vp, i64, vp, i64]
    L.orc_voxel_tris.restype = i64
    L.orc_level2.argtypes = [vp, i64, i64, vp, C.c_int, C.POINTER(i64), C.POINTER(i64)]
    L.orc_level2_list.argtypes = [vp, i64, vp, vp, C.c_int, C.POINTER(i64), C.POINTER(i64)]
    L.orc_count_ops.argtypes = [vp, i64, i64, C.c_int, vp]
    L.orc_level2_work.argtypes = [vp, C.c_int, C.POINTER(i64), C.POINTER(i64)]
    L.orc_voxel_fill_columns.argtypes = [vp, i64, vp, vp]
    L.orc_face_normal.argtypes = [vp, vp]
    L.orc_build_hierarchy.argtypes = [vp, vp]
    L.orc_build_hierarchy.restype = C.c_int
    L.orc_level1_normals.argtypes = [vp, vp]
    L.orc_level2_normals.argtypes = [vp, i64, i64, vp, C.c_int]
    L.orc_tri_box.argtypes = [vp, vp, vp]
    L.orc_tri_ray.argtypes = [vp, vp, vp, vp, vp, C.POINTER(C.c_float)]
    L.orc_tri_ray_z.argtypes = [vp, vp]
    L.orc_grid_tables.argtypes = [C.POINTER(Spec), vp, vp, vp, vp, vp, vp, vp]
    L.orc_reference_divisions.argtypes = [vp, vp, C.c_float, C.c_int, vp]
    if hasattr(L, "orc_gen_star"):
        f3 = C.POINTER(C.c_float)
        for name, extra in (("orc_gen_uvsphere", [C.c_int32, C.c_int32, f3, C.c_float, C.c_float]),
                            ("orc_gen_torus", [C.c_int32, C.c_int32, f3, C.c_float, C.c_float, C.c_float]),
                            ("orc_gen_star", [C.c_int32, f3, C.c_float, C.c_float, f3])):
            fn = getattr(L, name)
            fn.argtypes = [C.c_uint64, *extra, vp]
            fn.restype = C.c_int64
    _libs[ref] = L
    return L


def spec_from(grid):
    """Accepts a gpview_gb300.GridSpec or a (bmin, bmax, n, n2) tuple."""
    s = Spec()
    if hasattr(grid, "bbox_min"):
        bmin, bmax, n, n2 = grid.bbox_min, grid.bbox_max, grid.ndiv, grid.ndiv2
    else:
        bmin, bmax, n, n2 = grid
    s.bmin[:] = [float(x) for x in bmin]
    s.bmax[:] = [float(x) for x in bmax]
    s.n[:] = [int(x) for x in n]
    s.n2[:] = [int(x) for x in n2]
    return s


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Run:
    """One oracle voxelization (Level1 done at construction, Level2 on demand)."""

    def __init__(self, tris, grid, fill=FILL_CAND, threads=0, ref=False):
        self.L = _load(ref)
        self.tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
        self.spec = spec_from(grid)
        self.h = self.L.orc_create(_p(self.tris), self.tris.size // 9, C.byref(self.spec),
                                   int(fill), int(threads))
        self.N1 = int(np.prod(list(self.spec.n)))
        self.cells = int(np.prod(list(self.spec.n2)))
        self.B = int(self.L.orc_num_boundary(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_free(self.h)
            self.h = None

    def level1_state(self):
        out = np.empty(self.N1, np.uint8)
        self.L.orc_level1_state(self.h, _p(out))
        return out

    def level1_bytes(self):
        return (self.level1_state() * 127).astype(np.uint8)

    def prefix(self):
        out = np.empty(self.N1, np.int32)
        self.L.orc_prefix(self.h, _p(out))
        return out

    def boundary_index(self):
        out = np.empty(self.B, np.int32)
        self.L.orc_boundary_index(self.h, _p(out))
        return out

    def voxel_tris(self, v):
        n = self.L.orc_voxel_tris(self.h, int(v), None, 0)
        out = np.empty(n, np.int32)
        self.L.orc_voxel_tris(self.h, int(v), _p(out), n)
        return out

    def num_pairs(self):
        return int(self.L.orc_num_pairs(self.h))

    def sat1_tests(self):
        return int(self.L.orc_sat1_tests(self.h))

    def ray1_candidates(self):
        return int(self.L.orc_ray1_candidates(self.h))

    def level2_state(self, b0=0, b1=None, threads=0):
        """States (0/1/2) of boundary voxels [b0,b1), plus (sat2, ray2) work counts."""
        b1 = self.B if b1 is None else b1
        out = np.empty(max(b1 - b0, 0) * self.cells, np.uint8)
        s2, r2 = C.c_int64(), C.c_int64()
        if b1 > b0:
            self.L.orc_level2(self.h, int(b0), int(b1), _p(out), int(threads), C.byref(s2), C.byref(r2))
        return out, int(s2.value), int(r2.value)

    def voxel_fill_columns(self, cols):
        """ClassifyInOutCPU as written (every voxel centre against every triangle, one thread)
        on the given columns (j*nx + i): parity uint8 [len(cols), nz]."""
        cols = np.ascontiguousarray(cols, np.int64)
        nz = int(self.spec.n[2])
        out = np.zeros(cols.size * nz, np.uint8)
        self.L.orc_voxel_fill_columns(self.h, cols.size, _p(cols), _p(out))
        return out.reshape(cols.size, nz)

    def level2_list(self, blist, threads=0):
        """States of the listed boundary voxels (one block each, list order) in one parallel
        pass, plus their (sat2, ray2) work counts."""
        blist = np.ascontiguousarray(blist, np.int64)
        out = np.empty(blist.size * self.cells, np.uint8)
        s2, r2 = C.c_int64(), C.c_int64()
        if blist.size:
            self.L.orc_level2_list(self.h, blist.size, _p(blist), _p(out), int(threads),
                                   C.byref(s2), C.byref(r2))
        return out, int(s2.value), int(r2.value)

    def level2_work(self, threads=0):
        """(sat2, ray2): the algorithmic Level2 test counts of the whole mesh, without running
        the predicates (equal to the counts level2_state reports over every boundary voxel)."""
        s2, r2 = C.c_int64(), C.c_int64()
        self.L.orc_level2_work(self.h, int(threads), C.byref(s2), C.byref(r2))
        return int(s2.value), int(r2.value)

    def count_ops(self, b0=0, b1=None, threads=0):
        """Executed FP32 operations of the reference predicates over the algorithmic tests
        (early exits included): sat1/ray1 over the mesh, sat2/ray2 over boundary voxels [b0,b1)."""
        b1 = self.B if b1 is None else b1
        out = np.zeros(4, np.int64)
        self.L.orc_count_ops(self.h, int(b0), int(b1), int(threads), _p(out))
        return dict(zip(("sat1", "ray1", "sat2", "ray2"), (int(x) for x in out)))

    def level1_normals(self):
        """float32 [N1, 3]: Level1 normals (zero where no triangle is recorded)."""
        out = np.empty(self.N1 * 3, np.float32)
        self.L.orc_level1_normals(self.h, _p(out))
        return out.reshape(-1, 3)

    def level2_normals(self, b0=0, b1=None, threads=0):
        """float32 [(b1-b0)*cells, 3]: Level2 normals of boundary voxels [b0,b1)."""
        b1 = self.B if b1 is None else b1
        out = np.zeros(max(b1 - b0, 0) * self.cells * 3, np.float32)
        if b1 > b0:
            self.L.orc_level2_normals(self.h, int(b0), int(b1), _p(out), int(threads))
        return out.reshape(-1, 3)

    def hierarchy(self):
        """Object::BuildHierarchy over the Level1 voxels: (levels, structured array of N1-1 boxes
        with mid, half, solid, child1, child2, index); levels = -1 unless N1 is a power of two."""
        out = np.zeros(max(self.N1 - 1, 1), dtype=BOX_DTYPE)
        lv = int(self.L.orc_build_hierarchy(self.h, _p(out)))
        return lv, out[:self.N1 - 1]

    def level2_bytes(self, b0=0, b1=None, threads=0):
        st, _, _ = self.level2_state(b0, b1, threads)
        return (st * 127).astype(np.uint8)


BOX_DTYPE = np.dtype([("mid", np.float32, 3), ("half", np.float32, 3), ("solid", np.int32),
                      ("child1", np.int32), ("child2", np.int32), ("index", np.int32)])


def face_normal(tv, ref=False):
    L = _load(ref)
    tv = np.ascontiguousarray(tv, np.float32)
    out = np.empty(3, np.float32)
    L.orc_face_normal(_p(tv), _p(out))
    return out


def normal_bytes(n):
    """The .raw encoding of normals (src/Object.cpp:2940-2941, :3033-3035): unsigned char of
    n * float(256/3) + 127 in float."""
    n = np.asarray(n, np.float32)
    return (n * np.float32(256.0 / 3.0) + np.float32(127.0)).astype(np.int32).astype(np.uint8)


def tri_box(c, h, tv, ref=False):
    L = _load(ref)
    c = np.asarray(c, np.float32); h = np.asarray(h, np.float32); tv = np.asarray(tv, np.float32)
    return int(L.orc_tri_box(_p(c), _p(h), _p(tv)))


def tri_ray(v1, v2, v3, o, d, ref=False):
    L = _load(ref)
    a = [np.ascontiguousarray(x, np.float32) for x in (v1, v2, v3, o, d)]
    t = C.c_float(0.0)
    hit = int(L.orc_tri_ray(*[_p(x) for x in a], C.byref(t)))
    return hit, float(t.value)


def tri_ray_z(tv, o, ref=False):
    """The +z test through the column/t split used by the fill (D = (0,0,1))."""
    L = _load(ref)
    tv = np.ascontiguousarray(tv, np.float32); o = np.ascontiguousarray(o, np.float32)
    return int(L.orc_tri_ray_z(_p(tv), _p(o)))


def reference_divisions(bmin, bmax, max_model_size, voxel_count):
    L = _load(False)
    out = (C.c_int32 * 3)()
    L.orc_reference_divisions((C.c_float * 3)(*bmin), (C.c_float * 3)(*bmax),
                              C.c_float(max_model_size), int(voxel_count), out)
    return tuple(out)


def grid_tables(grid):
    L = _load(False)
    s = spec_from(grid)
    n = list(s.n)
    n2 = [max(int(x), 1) for x in s.n2]
    g, e1, g2, e2 = (np.empty(3, np.float32) for _ in range(4))
    c1 = np.empty(sum(n), np.float32)
    c2s = np.empty(sum(a * b for a, b in zip(n, n2)), np.float32)
    o2 = np.empty_like(c2s)
    L.orc_grid_tables(C.byref(s), _p(g), _p(e1), _p(g2), _p(e2), _p(c1), _p(c2s), _p(o2))
    return dict(g=g, e1=e1, g2=g2, e2=e2, c1=c1, c2s=c2s, o2=o2)


# ---- seeded workload meshes, without the GPU library --------------------------------------------
# The same generator source as gpview_gb300's gpv_gen_* (gpv_meshgen.cpp), built into this library:
# a CPU-only process (the benchmark's reference arm) makes bit-identical inputs with these.
def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def _gen(name, seed, *args):
    fn = getattr(_load(False), name)
    n = fn(C.c_uint64(seed), *args, None)
    out = np.empty(9 * n, dtype=np.float32)
    assert fn(C.c_uint64(seed), *args, out.ctypes.data_as(C.c_void_p)) == n
    return out


def gen_uvsphere(seed, nlon=128, nlat=64, center=(0.5, 0.5, 0.5), radius=0.4, jitter=0.002):
    return _gen("orc_gen_uvsphere", seed, int(nlon), int(nlat), _f3(center), float(radius), float(jitter))


def gen_torus(seed, nu=512, nv=256, center=(0.5, 0.5, 0.5), R=0.35, r=0.12, noise=0.01):
    return _gen("orc_gen_torus", seed, int(nu), int(nv), _f3(center), float(R), float(r), float(noise))


def gen_star(seed, subdiv=8, center=(0.5, 0.5, 0.5), radius=0.3, amp=0.2, scale=(1, 1, 6)):
    return _gen("orc_gen_star", seed, int(subdiv), _f3(center), float(radius), float(amp), _f3(scale))


def grid_padded(mesh_min, mesh_max, n, n2):
    """gpv_grid_padded in float32 arithmetic: n cells over the mesh box grown by one cell of size
    extent/(n-2) on each side (returns a (bmin, bmax, ndiv, ndiv2) tuple for Run)."""
    mn = np.asarray(mesh_min, np.float32)
    mx = np.asarray(mesh_max, np.float32)
    n3 = np.array([n] * 3 if np.isscalar(n) else n, np.int32)
    n23 = np.array([n2] * 3 if np.isscalar(n2) else n2, np.int32)
    ext = (mx - mn).astype(np.float32)
    ext = np.where(ext > 0, ext, np.float32(1e-3)).astype(np.float32)
    cell = (ext / (n3 - 2).astype(np.float32)).astype(np.float32)
    return ((mn - cell).astype(np.float32), (mx + cell).astype(np.float32), n3, n23)
