"""gpview_gb300 -- GB300-native two-level voxelizer (Python bindings over libgpview.so).

The compute path is the C ABI in include/gpview.h, implemented by hand-written sm_103a kernels in
csrc/.  This module binds it with ctypes and mirrors the reference's Object interface
(includes/Object.h:106-135: ReadObject, ReadOFFObject, CreateFlatTriangleData,
PerformVoxelization, SaveVoxelization) so reference-shaped code reads the same.

There is no CPU fallback: if libgpview.so is missing or no CUDA device is present, the
voxelization calls raise.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgpview.so")

GPV_OK = 0
ERRORS = {
    -1: "GPV_ERR_INVALID", -2: "GPV_ERR_CUDA", -3: "GPV_ERR_OOM", -4: "GPV_ERR_IO",
    -5: "GPV_ERR_PARSE", -6: "GPV_ERR_DEVICE", -7: "GPV_ERR_BUDGET", -8: "GPV_ERR_PENDING",
    -9: "GPV_ERR_NOTFOUND",
}


class GpvError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")


class GridSpec(C.Structure):
    _fields_ = [("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3),
                ("ndiv", C.c_int32 * 3), ("ndiv2", C.c_int32 * 3)]

    def __repr__(self):
        return (f"GridSpec(min={list(self.bbox_min)}, max={list(self.bbox_max)}, "
                f"ndiv={list(self.ndiv)}, ndiv2={list(self.ndiv2)})")


class Work(C.Structure):
    _fields_ = [("sat1", C.c_int64), ("sat2", C.c_int64), ("ray1", C.c_int64), ("ray2", C.c_int64)]

    def total(self):
        return self.sat1 + self.sat2 + self.ray1 + self.ray2


class Result(C.Structure):
    _fields_ = [("spec", GridSpec), ("grid_size", C.c_float * 3), ("grid_size2", C.c_float * 3),
                ("num_level1", C.c_int64), ("num_boundary", C.c_int64),
                ("num_level1_inside", C.c_int64), ("num_level2_inside", C.c_int64),
                ("num_level2_boundary", C.c_int64), ("num_pairs", C.c_int64), ("work", Work),
                ("level1_inout", C.c_void_p), ("level1_prefix", C.c_void_p),
                ("boundary_index", C.c_void_p), ("level2_inout", C.c_void_p),
                ("handle", C.c_uint64), ("level1_normal", C.c_void_p),
                ("level2_normal", C.c_void_p), ("normal_mode", C.c_int32),
                ("hierarchy_levels", C.c_int32), ("hierarchy", C.c_void_p)]


# gpv_box: one node of the voxel box hierarchy
BOX_DTYPE = np.dtype([("mid", np.float32, 3), ("half", np.float32, 3), ("solid", np.int32),
                      ("child1", np.int32), ("child2", np.int32), ("index", np.int32)])


NORMALS_OFF, NORMALS_BYTES, NORMALS_FLOAT = 0, 1, 2
# inside fill: +z ray parity (ClassifyInOutCPU / ClassifyInOutLevel2CPU) or the rasterised
# stencil parity (ClassifyInOut2x / ClassifyInOut2xLevel2)
FILL_RAY, FILL_STENCIL = 0, 1
# Level2 SAT organisation (identical results): chosen per launch, queued records, or per lane
LEVEL2_AUTO, LEVEL2_QUEUED, LEVEL2_INLINE = 0, 1, 2


class VoxelConfig(C.Structure):
    _fields_ = [("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3), ("ndiv", C.c_int32 * 3),
                ("grid_size", C.c_float * 3), ("num_level1_inside", C.c_int64),
                ("num_boundary", C.c_int64), ("has_level2", C.c_int32), ("ndiv2", C.c_int32 * 3),
                ("grid_size2", C.c_float * 3), ("num_level2_inside", C.c_int64),
                ("num_level2_boundary", C.c_int64)]


class MeshC(C.Structure):
    _fields_ = [("tris", C.POINTER(C.c_float)), ("num_triangles", C.c_int64),
                ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3),
                ("max_model_size", C.c_float)]


_lib = None


def lib():
    """Loads libgpview.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GpvError(-2, f"{LIB_PATH} is missing; run gpview_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    f3 = C.POINTER(C.c_float)
    L.gpv_init.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    L.gpv_destroy.argtypes = [C.c_void_p]
    L.gpv_last_error.argtypes = [C.c_void_p]
    L.gpv_last_error.restype = C.c_char_p
    L.gpv_set_tile.argtypes = [C.c_void_p, C.c_int]
    L.gpv_set_timing.argtypes = [C.c_void_p, C.c_int]
    L.gpv_stage_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int]
    L.gpv_host_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int]
    L.gpv_kernel_launches.restype = C.c_uint64
    L.gpv_grid_padded.argtypes = [f3, f3, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(GridSpec)]
    L.gpv_grid_reference.argtypes = [f3, f3, C.c_float, C.c_int32, C.c_int32, C.POINTER(GridSpec)]
    L.gpv_voxelize.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(GridSpec),
                               C.POINTER(Result), C.c_void_p]
    L.gpv_voxelize_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(GridSpec),
                                    C.POINTER(Result), C.c_void_p]
    L.gpv_result_copy_to_host.argtypes = [C.c_void_p, C.POINTER(Result), C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p]
    L.gpv_voxelize_to_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(GridSpec),
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                       C.c_int32, C.POINTER(Result), C.c_void_p]
    L.gpv_result_release.argtypes = [C.c_void_p, C.POINTER(Result)]
    L.gpv_load_obj.argtypes = [C.c_char_p, C.POINTER(MeshC)]
    L.gpv_load_off.argtypes = [C.c_char_p, C.POINTER(MeshC)]
    L.gpv_mesh_free.argtypes = [C.POINTER(MeshC)]
    L.gpv_write_raw.argtypes = [C.c_char_p, C.POINTER(Result), C.c_void_p, C.c_void_p, C.c_void_p]
    L.gpv_write_raw_normals.argtypes = [C.c_char_p, C.POINTER(Result), C.c_void_p, C.c_void_p]
    L.gpv_set_normals.argtypes = [C.c_void_p, C.c_int]
    L.gpv_set_hierarchy.argtypes = [C.c_void_p, C.c_int]
    L.gpv_set_fill.argtypes = [C.c_void_p, C.c_int]
    L.gpv_result_copy_hierarchy_to_host.argtypes = [C.c_void_p, C.POINTER(Result), C.c_void_p,
                                                    C.c_void_p]
    L.gpv_read_voxel_config.argtypes = [C.c_char_p, C.POINTER(VoxelConfig)]
    L.gpv_read_raw.argtypes = [C.c_char_p, C.POINTER(VoxelConfig), C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_void_p]
    L.gpv_result_copy_normals_to_host.argtypes = [C.c_void_p, C.POINTER(Result), C.c_void_p,
                                                  C.c_void_p, C.c_void_p]
    for name, extra in (("gpv_gen_uvsphere", [C.c_int32, C.c_int32, f3, C.c_float, C.c_float]),
                        ("gpv_gen_torus", [C.c_int32, C.c_int32, f3, C.c_float, C.c_float, C.c_float]),
                        ("gpv_gen_star", [C.c_int32, f3, C.c_float, C.c_float, f3]),
                        ("gpv_gen_superellipsoid", [C.c_int32, C.c_int32, f3, f3, C.c_float,
                                                    C.c_float, f3])):
        fn = getattr(L, name)
        fn.argtypes = [C.c_uint64, *extra, C.c_void_p]
        fn.restype = C.c_int64
    L.gpv_voxelize_level1_noalloc.argtypes = [C.c_void_p, C.c_int64, C.POINTER(GridSpec),
                                              C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.POINTER(C.c_int64), C.c_void_p]
    L.gpv_noalloc_last_error.restype = C.c_char_p
    L.gpv_set_level2_chunk.argtypes = [C.c_void_p, C.c_int]
    L.gpv_set_level2_mode.argtypes = [C.c_void_p, C.c_int]
    L.gpv_set_debug.argtypes = [C.c_void_p, C.c_int, C.c_int64]
    L.gpv_set_host_expand.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_int32, C.c_int64]
    L.gpv_get_debug.argtypes = [C.c_void_p, C.c_int]
    L.gpv_get_debug.restype = C.c_int64
    L.gpv_set_graphs.argtypes = [C.c_void_p, C.c_int]
    L.gpv_autotune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_int64),
                               C.POINTER(GridSpec), C.c_void_p, C.POINTER(C.c_int32),
                               C.POINTER(C.c_int32), C.POINTER(C.c_float)]
    L.gpv_server_create.argtypes = [C.c_int, C.c_int64, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]
    L.gpv_server_set_tunables.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.gpv_server_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(GridSpec),
                                    C.POINTER(C.c_uint64)]
    L.gpv_server_poll.argtypes = [C.c_void_p, C.c_uint64, C.c_int32, C.POINTER(Result),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.gpv_server_release.argtypes = [C.c_void_p, C.c_uint64]
    L.gpv_server_add_mesh.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_uint64)]
    L.gpv_server_submit_mesh.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(GridSpec),
                                         C.POINTER(C.c_uint64)]
    L.gpv_server_remove_mesh.argtypes = [C.c_void_p, C.c_uint64]
    L.gpv_server_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    L.gpv_server_destroy.argtypes = [C.c_void_p]
    if hasattr(L, "gpv_voxelize_batch"):
        L.gpv_voxelize_batch.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p),
                                         C.POINTER(C.c_int64), C.POINTER(GridSpec),
                                         C.POINTER(Result), C.c_void_p]
    _lib = L
    return L


def kernel_launches():
    """Kernels launched by libgpview.so in this process so far."""
    return int(lib().gpv_kernel_launches())


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def _i3(v):
    return (C.c_int32 * 3)(*[int(x) for x in v])


# ---- grids ------------------------------------------------------------------------------------
def grid_padded(mesh_min, mesh_max, ndiv, ndiv2=(0, 0, 0)):
    """n^3 cells over the mesh box grown by one cell on each side."""
    if np.isscalar(ndiv):
        ndiv = (ndiv,) * 3
    if np.isscalar(ndiv2):
        ndiv2 = (ndiv2,) * 3
    s = GridSpec()
    rc = lib().gpv_grid_padded(_f3(mesh_min), _f3(mesh_max), _i3(ndiv), _i3(ndiv2), C.byref(s))
    if rc:
        raise GpvError(rc, "grid_padded")
    return s


def grid_reference(bbox_min, bbox_max, max_model_size, voxel_count=8, voxel_count2=4):
    """GPView's own sizing from GLParameters::voxelCount / voxelCount2."""
    s = GridSpec()
    rc = lib().gpv_grid_reference(_f3(bbox_min), _f3(bbox_max), float(max_model_size),
                                  int(voxel_count), int(voxel_count2), C.byref(s))
    if rc:
        raise GpvError(rc, "grid_reference")
    return s


def mesh_bounds(tris):
    v = np.asarray(tris, dtype=np.float32).reshape(-1, 3)
    return v.min(axis=0), v.max(axis=0)


# ---- synthetic meshes -------------------------------------------------------------------------
def _gen(name, seed, *args):
    fn = getattr(lib(), name)
    n = fn(C.c_uint64(seed), *args, None)
    out = np.empty(9 * n, dtype=np.float32)
    got = fn(C.c_uint64(seed), *args, out.ctypes.data_as(C.c_void_p))
    assert got == n
    return out


def gen_uvsphere(seed, nlon=128, nlat=64, center=(0.5, 0.5, 0.5), radius=0.4, jitter=0.002):
    return _gen("gpv_gen_uvsphere", seed, int(nlon), int(nlat), _f3(center), float(radius),
                float(jitter))


def gen_torus(seed, nu=512, nv=256, center=(0.5, 0.5, 0.5), R=0.35, r=0.12, noise=0.01):
    return _gen("gpv_gen_torus", seed, int(nu), int(nv), _f3(center), float(R), float(r),
                float(noise))


def gen_star(seed, subdiv=8, center=(0.5, 0.5, 0.5), radius=0.3, amp=0.2, scale=(1, 1, 6)):
    return _gen("gpv_gen_star", seed, int(subdiv), _f3(center), float(radius), float(amp),
                _f3(scale))


def gen_superellipsoid(seed, nlon, nlat, center, semi, e1, e2, rot=None):
    rot = np.eye(3, dtype=np.float32) if rot is None else np.asarray(rot, np.float32)
    return _gen("gpv_gen_superellipsoid", seed, int(nlon), int(nlat), _f3(center), _f3(semi),
                float(e1), float(e2), (C.c_float * 9)(*rot.reshape(-1).tolist()))


# ---- context ----------------------------------------------------------------------------------
class Context:
    """A libgpview context on one device: stream-ordered pool, pinned staging, results."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        rc = lib().gpv_init(int(device), C.byref(self._h))
        if rc:
            raise GpvError(rc, "gpv_init (no CUDA device?)")
        self.device = device

    def close(self):
        if self._h:
            lib().gpv_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self):
        return lib().gpv_last_error(self._h).decode()

    STAGES = ("prep", "level1", "fill_finish", "expand", "sort_lists", "level2", "level2_kernel",
              "pair_bases", "between_phases")

    def set_timing(self, on=True):
        self._check(lib().gpv_set_timing(self._h, int(bool(on))), "set_timing")

    def stage_times(self):
        """(calls, {stage: accumulated ms}) from the per-stage CUDA events."""
        ms = (C.c_double * 9)()
        calls = lib().gpv_stage_times(self._h, ms, 9)
        return calls, {k: ms[i] for i, k in enumerate(self.STAGES)}

    HOST_SEGMENTS = ("setup", "first_phase", "planning", "second_phase", "results")

    def host_times(self):
        """(calls, {segment: accumulated host ms}) from the host clock around each call."""
        ms = (C.c_double * 5)()
        calls = lib().gpv_host_times(self._h, ms, 5)
        return calls, {k: ms[i] for i, k in enumerate(self.HOST_SEGMENTS)}

    GRAPHS_ONE, GRAPHS_TWO = 1, 2

    def set_graphs(self, mode=True):
        """True / GRAPHS_ONE (default): CUDA graphs, a call repeating the previous call's meshes
        and grids as one graph; GRAPHS_TWO: two graphs per call; False / 0: direct launches."""
        m = self.GRAPHS_ONE if mode is True else (0 if mode is False else int(mode))
        self._check(lib().gpv_set_graphs(self._h, m), "set_graphs")

    def set_tile(self, t):
        rc = lib().gpv_set_tile(self._h, int(t))
        if rc:
            raise GpvError(rc, "set_tile")

    def set_level2_chunk(self, max_voxels):
        """Largest number of boundary voxels of one Level1 column per Level2 work item."""
        self._check(lib().gpv_set_level2_chunk(self._h, int(max_voxels)), "set_level2_chunk")

    def set_level2_mode(self, mode):
        """LEVEL2_AUTO (default), LEVEL2_QUEUED or LEVEL2_INLINE: the Level2 SAT organisation."""
        self._check(lib().gpv_set_level2_mode(self._h, int(mode)), "set_level2_mode")

    def set_host_expand(self, threads=-1, slab_mask=0xff, share=45, min_level2_bytes=64 << 20):
        """Packed Level2 transfer of voxelize_to_host (gpv_set_host_expand): host threads (-1 by
        the machine, 0 off), the z slabs (bit mask of 8) that send 2-bit codes for the first
        `share` percent of their boundary voxels, and the Level2 output size from which it
        applies."""
        self._check(lib().gpv_set_host_expand(self._h, int(threads), int(slab_mask), int(share),
                                              int(min_level2_bytes)), "set_host_expand")

    DEBUG = {"wait_limit": 1, "fail_wait": 2, "pair_capacity": 3, "fail_allocs": 4, "replans": 5,
             "one_graph_capacity": 6, "one_graph_calls": 7, "one_graph_replans": 8}

    def set_debug(self, what, value):
        """Failure-detection hooks (gpv_set_debug): 'wait_limit', 'fail_wait', 'pair_capacity',
        'fail_allocs'."""
        self._check(lib().gpv_set_debug(self._h, self.DEBUG[what], int(value)), "set_debug")

    def get_debug(self, what):
        return int(lib().gpv_get_debug(self._h, self.DEBUG[what]))

    def _check(self, rc, what):
        if rc:
            raise GpvError(rc, f"{what}: {self.error()}")

    def voxelize_device(self, d_ptr, num_triangles, spec, stream=0):
        """Plain path on device triangles (pointer to float[T*9], 16-byte aligned)."""
        res = Result()
        self._check(lib().gpv_voxelize(self._h, C.c_void_p(d_ptr), int(num_triangles),
                                       C.byref(spec), C.byref(res), C.c_void_p(stream)),
                    "gpv_voxelize")
        return res

    def voxelize_host(self, tris, spec, stream=0):
        tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
        res = Result()
        self._check(lib().gpv_voxelize_host(self._h, tris.ctypes.data_as(C.c_void_p),
                                            tris.size // 9, C.byref(spec), C.byref(res),
                                            C.c_void_p(stream)), "gpv_voxelize_host")
        return res

    def voxelize_to_host(self, tris_ptr, num_triangles, spec, l1_ptr, prefix_ptr, bindex_ptr,
                         l2_ptr, l2_bytes, slabs=0, stream=0):
        """Host triangles in, host outputs out (pointers, ideally page-locked), copies overlapped
        with the computation.  Returns (status, result); status GPV_ERR_BUDGET (-7) when the
        Level2 buffer is too small (the result is still complete and must be released)."""
        res = Result()
        rc = lib().gpv_voxelize_to_host(self._h, C.c_void_p(tris_ptr), int(num_triangles),
                                        C.byref(spec), C.c_void_p(l1_ptr), C.c_void_p(prefix_ptr),
                                        C.c_void_p(bindex_ptr), C.c_void_p(l2_ptr), int(l2_bytes),
                                        int(slabs), C.byref(res), C.c_void_p(stream))
        if rc not in (0, -7):
            raise GpvError(rc, f"gpv_voxelize_to_host: {self.error()}")
        return rc, res

    def voxelize_batch(self, d_ptrs, counts, specs, stream=0):
        n = len(d_ptrs)
        ptrs = (C.c_void_p * n)(*[C.c_void_p(p) for p in d_ptrs])
        cnts = (C.c_int64 * n)(*[int(c) for c in counts])
        sp = (GridSpec * n)(*specs)
        res = (Result * n)()
        self._check(lib().gpv_voxelize_batch(self._h, n, ptrs, cnts, sp, res, C.c_void_p(stream)),
                    "gpv_voxelize_batch")
        return list(res)

    def autotune(self, d_ptrs, counts, specs, stream=0):
        """Picks the (Level1 tile, Level2 chunk) pair that runs this sample batch fastest."""
        n = len(d_ptrs)
        ptrs = (C.c_void_p * n)(*[C.c_void_p(p) for p in d_ptrs])
        cnts = (C.c_int64 * n)(*[int(c) for c in counts])
        sp = (GridSpec * n)(*specs)
        t, ch, ms = C.c_int32(), C.c_int32(), C.c_float()
        self._check(lib().gpv_autotune(self._h, n, ptrs, cnts, sp, C.c_void_p(stream), C.byref(t),
                                       C.byref(ch), C.byref(ms)), "gpv_autotune")
        return t.value, ch.value, ms.value

    def fetch(self, res, stream=0):
        """Copies a result to host numpy arrays: (level1 u8, prefix i32, boundary i32, level2 u8)."""
        cells = res.spec.ndiv2[0] * res.spec.ndiv2[1] * res.spec.ndiv2[2]
        l1 = np.empty(res.num_level1, np.uint8)
        pre = np.empty(res.num_level1, np.int32)
        bi = np.empty(res.num_boundary, np.int32)
        l2 = np.empty(res.num_boundary * cells, np.uint8)
        self._check(lib().gpv_result_copy_to_host(
            self._h, C.byref(res), l1.ctypes.data_as(C.c_void_p), pre.ctypes.data_as(C.c_void_p),
            bi.ctypes.data_as(C.c_void_p), l2.ctypes.data_as(C.c_void_p), C.c_void_p(stream)),
            "copy_to_host")
        return l1, pre, bi, l2

    def set_normals(self, mode):
        """NORMALS_OFF, NORMALS_BYTES (the .raw encoding) or NORMALS_FLOAT for the next calls."""
        self._check(lib().gpv_set_normals(self._h, int(mode)), "set_normals")

    def fetch_normals(self, res, stream=0):
        """Copies a result's normals to host: (level1 [N1, 3], level2 [B*cells, 3]), uint8 or
        float32 per the result's normal mode."""
        cells = res.spec.ndiv2[0] * res.spec.ndiv2[1] * res.spec.ndiv2[2]
        dt = np.float32 if res.normal_mode == NORMALS_FLOAT else np.uint8
        l1 = np.empty((res.num_level1, 3), dt)
        l2 = np.empty((res.num_boundary * cells, 3), dt)
        self._check(lib().gpv_result_copy_normals_to_host(
            self._h, C.byref(res), l1.ctypes.data_as(C.c_void_p), l2.ctypes.data_as(C.c_void_p),
            C.c_void_p(stream)), "copy_normals_to_host")
        return l1, l2

    def set_fill(self, mode):
        """FILL_RAY (default) or FILL_STENCIL for the next calls."""
        self._check(lib().gpv_set_fill(self._h, int(mode)), "set_fill")

    def set_hierarchy(self, on=True):
        """Build the voxel box hierarchy (Object::BuildHierarchy) with the next calls."""
        self._check(lib().gpv_set_hierarchy(self._h, int(bool(on))), "set_hierarchy")

    def fetch_hierarchy(self, res, stream=0):
        """The result's hierarchy as a structured array of num_level1 - 1 boxes (BOX_DTYPE)."""
        out = np.empty(max(res.num_level1 - 1, 1), BOX_DTYPE)
        self._check(lib().gpv_result_copy_hierarchy_to_host(
            self._h, C.byref(res), out.ctypes.data_as(C.c_void_p), C.c_void_p(stream)),
            "copy_hierarchy_to_host")
        return out[:res.num_level1 - 1]

    def release(self, res):
        self._check(lib().gpv_result_release(self._h, C.byref(res)), "release")


# ---- reference-shaped host interface ----------------------------------------------------------
class GLParameters:
    """The voxelization knobs of GLParameters (src/GLParameters.cpp:28-69)."""

    def __init__(self, voxelCount=8, voxelCount2=4, level2Voxels=True, saveVoxels=True):
        self.voxelCount = voxelCount
        self.voxelCount2 = voxelCount2
        self.level2Voxels = level2Voxels
        self.saveVoxels = saveVoxels


class VoxelData:
    """Result fields named as in the reference's VoxelData (includes/Utilities.h:79-154)."""

    def __init__(self, res, l1, prefix, bindex, l2):
        s = res.spec
        self.numDivX, self.numDivY, self.numDivZ = (int(v) for v in s.ndiv)
        self.numDivX2, self.numDivY2, self.numDivZ2 = (int(v) for v in s.ndiv2)
        self.gridSizeX, self.gridSizeY, self.gridSizeZ = (float(v) for v in res.grid_size)
        self.gridSizeX2, self.gridSizeY2, self.gridSizeZ2 = (float(v) for v in res.grid_size2)
        self.level1InOut = l1            # uint8 .raw encoding (state*127)
        self.boundaryPrefixSum = prefix
        self.boundaryIndex = bindex
        self.level2InOut = l2
        self.numLevel1InsideVoxels = int(res.num_level1_inside)
        self.numLevel1BoundaryVoxels = int(res.num_boundary)
        self.numLevel2InsideVoxels = int(res.num_level2_inside)
        self.numLevel2BoundaryVoxels = int(res.num_level2_boundary)
        self.level1Normal = None         # float32 [N1, 3] when computed
        self.level2Normal = None         # float32 [B * n2^3, 3] when computed


class Object:
    """Mirror of the reference's Object for the voxelization path (includes/Object.h:85-135)."""

    def __init__(self, ctx=None, objID=-1):
        self.ctx = ctx
        self.objID = objID
        self.flatCPUTriangleData = None
        self.totalNumTriangles = 0
        self.bBoxMin = None
        self.bBoxMax = None
        self.maxModelSize = 0.0
        self.voxelData = None
        self._result = None

    def _load(self, fn, path):
        m = MeshC()
        rc = fn(path.encode(), C.byref(m))
        if rc:
            raise GpvError(rc, path)
        try:
            n = int(m.num_triangles)
            self._tris = np.ctypeslib.as_array(m.tris, shape=(9 * n,)).copy() if n else np.zeros(0, np.float32)
            self.bBoxMin = np.array(m.bbox_min, np.float32)
            self.bBoxMax = np.array(m.bbox_max, np.float32)
            self.maxModelSize = float(m.max_model_size)
        finally:
            lib().gpv_mesh_free(C.byref(m))

    def ReadObject(self, path):
        self._load(lib().gpv_load_obj, path)

    def ReadOFFObject(self, path):
        self._load(lib().gpv_load_off, path)

    def ReadRAWObject(self, fName):
        """Object::ReadRAWObject (src/Object.cpp:319-392): a 48 x 64 x 64 Level1InOut file read as
        the Level1 states; `solid` per voxel is int(value) % 2 (the grid spans bBoxMin..bBoxMax)."""
        n = (48, 64, 64)
        with open(fName, "rb") as f:
            data = np.frombuffer(f.read(n[0] * n[1] * n[2]), np.uint8)
        vd = VoxelData.__new__(VoxelData)
        vd.numDivX, vd.numDivY, vd.numDivZ = n
        if self.bBoxMin is not None:
            span = (np.asarray(self.bBoxMax, np.float64) - np.asarray(self.bBoxMin, np.float64))
            vd.gridSizeX, vd.gridSizeY, vd.gridSizeZ = (float(np.float32(span[a] / (n[a] * 1.0)))
                                                        for a in range(3))
        full = np.zeros(n[0] * n[1] * n[2], np.uint8)
        full[:data.size] = data
        vd.level1InOut = full
        vd.solid = (full.astype(np.int32) % 2).astype(np.uint8)
        self.voxelData = vd
        return vd

    def CreateFlatTriangleData(self):
        self.flatCPUTriangleData = self._tris
        self.totalNumTriangles = self._tris.size // 9

    def PerformVoxelization(self, glParam, bufferSize=-1, spec=None, normals=True, fill=FILL_RAY):
        """Voxelizes on the GPU.  `spec` overrides the reference sizing (explicit grids).  Normals
        are computed as the reference does (float, src/Object.cpp:3219-3253, :2402-2424) unless
        `normals` is False.  `fill` picks the inside fill: FILL_RAY, the CPU path
        (ClassifyInOutCPU, :3159), or FILL_STENCIL, the rasterised path the reference calls at
        :3158 and :3297 (ClassifyInOut2x, ClassifyInOut2xLevel2)."""
        del bufferSize  # the device path has no fixed per-voxel buffer
        if self.flatCPUTriangleData is None:
            self.CreateFlatTriangleData()
        if self.ctx is None:
            self.ctx = Context()
        if spec is None:
            spec = grid_reference(self.bBoxMin, self.bBoxMax, self.maxModelSize,
                                  glParam.voxelCount, glParam.voxelCount2 if glParam.level2Voxels else 0)
        self.ctx.set_normals(NORMALS_FLOAT if normals else NORMALS_OFF)
        self.ctx.set_fill(fill)
        try:
            res = self.ctx.voxelize_host(self.flatCPUTriangleData, spec)
        finally:
            self.ctx.set_normals(NORMALS_OFF)
            self.ctx.set_fill(FILL_RAY)
        try:
            l1, pre, bi, l2 = self.ctx.fetch(res)
            nrm = self.ctx.fetch_normals(res) if normals else (None, None)
        finally:
            self._result = res
        self.voxelData = VoxelData(res, l1, pre, bi, l2)
        self.voxelData.level1Normal, self.voxelData.level2Normal = nrm
        if glParam.saveVoxels:
            self.SaveVoxelization(glParam)
        self.ctx.release(res)
        return self.voxelData

    def SaveVoxelization(self, glParam, prefix=None):
        vd = self.voxelData
        prefix = prefix or f"Obj{self.objID}"
        rc = lib().gpv_write_raw(prefix.encode(), C.byref(self._result),
                                 vd.level1InOut.ctypes.data_as(C.c_void_p),
                                 vd.boundaryPrefixSum.ctypes.data_as(C.c_void_p),
                                 vd.level2InOut.ctypes.data_as(C.c_void_p))
        if rc:
            raise GpvError(rc, "SaveVoxelization")
        if vd.level1Normal is not None:
            n1 = normal_bytes(vd.level1Normal)
            n2 = normal_bytes(vd.level2Normal)
            rc = lib().gpv_write_raw_normals(prefix.encode(), C.byref(self._result),
                                             n1.ctypes.data_as(C.c_void_p), n2.ctypes.data_as(C.c_void_p))
            if rc:
                raise GpvError(rc, "SaveVoxelization (normals)")


def read_voxel_config(prefix):
    """Parses <prefix>VoxelConfig.txt (the line order of Object::SaveVoxelization)."""
    cfg = VoxelConfig()
    rc = lib().gpv_read_voxel_config(str(prefix).encode(), C.byref(cfg))
    if rc:
        raise GpvError(rc, f"{prefix}VoxelConfig.txt")
    return cfg


def read_raw(prefix, cfg=None, normals=True):
    """Reads a saved voxelization back: dict of the config and the .raw arrays (Level1InOut,
    Level1BoundaryPrefixSum, Level2InOut and, when present, the two normal files)."""
    cfg = cfg or read_voxel_config(prefix)
    n1 = int(np.prod(list(cfg.ndiv)))
    cells = int(np.prod(list(cfg.ndiv2))) if cfg.has_level2 else 0
    nb = int(cfg.num_boundary)
    out = {"config": cfg, "level1InOut": np.empty(n1, np.uint8)}
    if cfg.has_level2:
        out["boundaryPrefixSum"] = np.empty(n1, np.int32)
        out["level2InOut"] = np.empty(nb * cells, np.uint8)
    have_n = normals and os.path.exists(f"{prefix}Level1Normal.raw")
    if have_n:
        out["level1Normal"] = np.empty((n1, 3), np.uint8)
        if cfg.has_level2:
            out["level2Normal"] = np.empty((nb * cells, 3), np.uint8)
    ptr = lambda k: out[k].ctypes.data_as(C.c_void_p) if k in out else None  # noqa: E731
    rc = lib().gpv_read_raw(str(prefix).encode(), C.byref(cfg), ptr("level1InOut"),
                            ptr("boundaryPrefixSum"), ptr("level2InOut"), ptr("level1Normal"),
                            ptr("level2Normal"))
    if rc:
        raise GpvError(rc, f"read_raw {prefix}")
    return out


def normal_bytes(n):
    """The .raw encoding of normals, uint8(n * float(256/3) + 127) in float arithmetic
    (src/Object.cpp:2940-2941, :3033-3035); the device's GPV_NORMALS_BYTES mode writes the same."""
    n = np.ascontiguousarray(n, np.float32)
    return (n * np.float32(256.0 / 3.0) + np.float32(127.0)).astype(np.int32).astype(np.uint8)


class Server:
    """Continuous-batching voxelization server (gpv_server_* in include/gpview.h)."""

    def __init__(self, device=0, budget_bytes=150 << 30, workers=2, max_batch=256):
        self._h = C.c_void_p()
        rc = lib().gpv_server_create(int(device), int(budget_bytes), int(workers), int(max_batch),
                                     C.byref(self._h))
        if rc:
            raise GpvError(rc, "gpv_server_create")
        self._keep = {}

    def set_tunables(self, tile, level2_chunk):
        rc = lib().gpv_server_set_tunables(self._h, int(tile), int(level2_chunk))
        if rc:
            raise GpvError(rc, "set_tunables")

    def submit(self, tris, spec):
        """tris: float32 array (pinned torch tensor or numpy), kept alive until release."""
        ptr = tris.data_ptr() if hasattr(tris, "data_ptr") else tris.ctypes.data
        n = (tris.numel() if hasattr(tris, "numel") else tris.size) // 9
        t = C.c_uint64()
        rc = lib().gpv_server_submit(self._h, C.c_void_p(ptr), int(n), C.byref(spec), C.byref(t))
        if rc:
            raise GpvError(rc, "submit")
        self._keep[t.value] = tris
        return t.value

    def add_mesh(self, tris):
        """Uploads a mesh once into the server's device pool; returns its id."""
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1)
        mid = C.c_uint64()
        rc = lib().gpv_server_add_mesh(self._h, tris.ctypes.data_as(C.c_void_p), tris.size // 9,
                                       C.byref(mid))
        if rc:
            raise GpvError(rc, "add_mesh")
        return mid.value

    def submit_mesh(self, mesh_id, spec):
        """A voxelization of a resident mesh (no host-to-device copy)."""
        t = C.c_uint64()
        rc = lib().gpv_server_submit_mesh(self._h, C.c_uint64(mesh_id), C.byref(spec), C.byref(t))
        if rc:
            raise GpvError(rc, "submit_mesh")
        return t.value

    def remove_mesh(self, mesh_id):
        return lib().gpv_server_remove_mesh(self._h, C.c_uint64(mesh_id))

    def poll(self, ticket, timeout_ms=0):
        """(status, result, latency_ms, queue_ms); status GPV_ERR_PENDING (-8) while running."""
        res = Result()
        lat, q = C.c_double(), C.c_double()
        rc = lib().gpv_server_poll(self._h, C.c_uint64(ticket), int(timeout_ms), C.byref(res),
                                   C.byref(lat), C.byref(q))
        return rc, res, lat.value, q.value

    def release(self, ticket):
        rc = lib().gpv_server_release(self._h, C.c_uint64(ticket))
        self._keep.pop(ticket, None)
        return rc

    def stats(self):
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_uint64(), C.c_uint64()
        lib().gpv_server_stats(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return dict(in_use_bytes=a.value, pending=b.value, batches=c.value, served=d.value)

    def close(self):
        if self._h:
            lib().gpv_server_destroy(self._h)
            self._h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
