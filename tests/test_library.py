"""CPU tests of libgpview.so: it loads, exports every declared symbol, and its host code
(grids, loaders, generators, .raw writer) follows the reference."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exports_every_header_symbol(built):
    text = open(os.path.join(ROOT, "include", "gpview.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text))
    names -= {"if", "sizeof", "defined"}
    decl = [n for n in names if n.startswith("gpv_") or n.startswith("THRUSTDevice") or n in (
        "CUDAClassifyTessellation", "CUDAClassifyTessellationLevel2", "CUDAClassifyInOutLevel2")]
    assert len(decl) >= 20
    assert {"THRUSTDeviceFindMax", "THRUSTDeviceFindMaxFloat4", "THRUSTDeviceMinMaxSort"} <= set(decl)
    L = built.lib()
    missing = [n for n in decl if not hasattr(L, n)]
    assert not missing, missing
    # the application's C++-linkage helpers are not exported under C names
    assert not hasattr(L, "InitializeCUDA") and not hasattr(L, "CUDACheckErrors")


def test_generator_counts_and_determinism(built):
    gpv = built
    assert gpv.lib().gpv_gen_uvsphere(1, 128, 64, (C.c_float * 3)(0.5, 0.5, 0.5), 0.4, 0.002, None) == 16128
    assert gpv.lib().gpv_gen_torus(1, 512, 256, (C.c_float * 3)(0.5, 0.5, 0.5), 0.35, 0.12, 0.01, None) == 262144
    assert gpv.lib().gpv_gen_star(1, 8, (C.c_float * 3)(0.5, 0.5, 0.5), 0.3, 0.2,
                                  (C.c_float * 3)(1, 1, 6), None) == 1310720
    a = gpv.gen_torus(5, 64, 32)
    b = gpv.gen_torus(5, 64, 32)
    c = gpv.gen_torus(6, 64, 32)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def _edges_shared_twice(tris):
    v = tris.reshape(-1, 3, 3)
    keys = {}
    for t in v:
        pts = [tuple(p) for p in t]
        for a, b in ((0, 1), (1, 2), (2, 0)):
            e = tuple(sorted((pts[a], pts[b])))
            keys[e] = keys.get(e, 0) + 1
    return all(c == 2 for c in keys.values())


@pytest.mark.parametrize("kind", ["sphere", "torus", "star", "superellipsoid"])
def test_generated_meshes_are_closed(built, kind):
    gpv = built
    t = {"sphere": lambda: gpv.gen_uvsphere(3, 16, 8),
         "torus": lambda: gpv.gen_torus(3, 16, 8),
         "star": lambda: gpv.gen_star(3, 2),
         "superellipsoid": lambda: gpv.gen_superellipsoid(3, 16, 8, (0.5, 0.5, 0.5), (0.3, 0.2, 0.25), 0.5, 1.5)}[kind]()
    assert np.isfinite(t).all()
    assert _edges_shared_twice(t)


def _pad_ref(mn, mx):
    """Object::ReadObject's padding in float/double as the reference evaluates it."""
    d = (mx - mn).astype(np.float32)
    s = np.float32(d[0] * d[0] + d[1] * d[1])
    s = np.float32(s + np.float32(d[2] * d[2]))
    mag = np.float32(np.sqrt(np.float64(s)))
    off = np.float32(0.001 * np.float64(mag))
    return (mn - off).astype(np.float32), (off + mx).astype(np.float32)


def test_obj_loader(built, tmp_path):
    gpv = built
    p = tmp_path / "quad.obj"
    p.write_text("# comment\nv 0 0 0\nv 1 0 0\nv 1 2 0\nv 0 1 3.5\nvn 0 0 1\nvt 0 0\n"
                 "f 1 2 3\nf 1/1 3/1 4/1\nf 2//1 3//1 4//1\nf 1/1/1 2/1/1 4/1/1\nf 1 2 4")  # last line unterminated
    o = gpv.Object()
    o.ReadObject(str(p))
    o.CreateFlatTriangleData()
    assert o.totalNumTriangles == 4  # the unterminated last line is ignored, as in the reference
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 2, 0], [0, 1, 3.5]], np.float32)
    np.testing.assert_array_equal(o.flatCPUTriangleData[:9], v[[0, 1, 2]].reshape(-1))
    np.testing.assert_array_equal(o.flatCPUTriangleData[27:36], v[[0, 1, 3]].reshape(-1))
    mn, mx = _pad_ref(v.min(0), v.max(0))
    np.testing.assert_array_equal(o.bBoxMin, mn)
    np.testing.assert_array_equal(o.bBoxMax, mx)
    assert o.maxModelSize == pytest.approx(float(max(mx - mn)), rel=0, abs=0)


def test_off_loader_and_errors(built, tmp_path):
    gpv = built
    p = tmp_path / "t.off"
    p.write_text("OFF\n4 2 0\n0 0 0\n1 0 0\n0 1 0\n0 0 1\n3 0 1 2\n4 0 1 3 2\n")
    o = gpv.Object()
    o.ReadOFFObject(str(p))
    o.CreateFlatTriangleData()
    assert o.totalNumTriangles == 2
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3 4\n")
    with pytest.raises(gpv.GpvError) as e:
        gpv.Object().ReadObject(str(bad))
    assert e.value.code == -5
    with pytest.raises(gpv.GpvError) as e:
        gpv.Object().ReadObject(str(tmp_path / "missing.obj"))
    assert e.value.code == -4


def test_cessna_fixture(built):
    """The reference's only mesh file (files/cessna.obj, committed as tests/golden/cessna.obj)."""
    gpv = built
    o = gpv.Object()
    o.ReadObject(os.path.join(ROOT, "tests", "golden", "cessna.obj"))
    o.CreateFlatTriangleData()
    assert o.totalNumTriangles == 7446
    assert _edges_shared_twice(o.flatCPUTriangleData)  # closed and manifold


def test_grid_reference_matches_oracle(built):
    from oracle import oracle as orc

    gpv = built
    for bmin, bmax, vc in (((0, 0, 0), (1, 1, 1), 8), ((-19.6, -5.1, -22.2), (21.6, 5.1, 22.2), 32),
                           ((0, 0, 0), (2.0, 0.3, 0.07), 17)):
        size = max(b - a for a, b in zip(bmin, bmax))
        s = gpv.grid_reference(bmin, bmax, size, vc, 4)
        assert tuple(s.ndiv) == orc.reference_divisions(bmin, bmax, size, vc)
        assert all(n % 4 == 0 for n in s.ndiv)


def test_write_raw(built, tmp_path):
    gpv = built
    r = gpv.Result()
    r.spec = gpv.grid_padded((0, 0, 0), (1, 1, 1), (4, 3, 3), 2)
    r.num_level1 = 36
    r.num_boundary = 3
    l1 = np.arange(36, dtype=np.uint8)
    pre = np.arange(36, dtype=np.int32)
    l2 = np.arange(24, dtype=np.uint8)
    prefix = str(tmp_path / "Obj-1")
    rc = gpv.lib().gpv_write_raw(prefix.encode(), C.byref(r), l1.ctypes.data_as(C.c_void_p),
                                 pre.ctypes.data_as(C.c_void_p), l2.ctypes.data_as(C.c_void_p))
    assert rc == 0
    assert (tmp_path / "Obj-1Level1InOut.raw").read_bytes() == l1.tobytes()
    assert (tmp_path / "Obj-1Level1BoundaryPrefixSum.raw").read_bytes() == pre.tobytes()
    assert (tmp_path / "Obj-1Level2InOut.raw").read_bytes() == l2.tobytes()
    cfg = (tmp_path / "Obj-1VoxelConfig.txt").read_text().splitlines()
    assert cfg[0].endswith("Obj-1") and cfg[3] == "4\t3\t3" and cfg[7] == "2\t2\t2"


def test_invalid_grid_rejected(built):
    gpv = built
    with pytest.raises(gpv.GpvError):
        gpv.grid_padded((0, 0, 0), (1, 1, 1), 2, 4)  # needs at least 3 cells per axis


def test_raw_round_trip_and_config(built, tmp_path):
    """gpv_write_raw + gpv_write_raw_normals, then gpv_read_voxel_config + gpv_read_raw give back
    the same arrays and counts (the golden sphere's outputs)."""
    import glob

    gpv = built
    z = np.load(sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "mesh_sphere288.npz")))[0])
    res = gpv.Result()
    spec = res.spec
    spec.bbox_min[:] = z["bbox_min"]
    spec.bbox_max[:] = z["bbox_max"]
    spec.ndiv[:] = z["ndiv"]
    spec.ndiv2[:] = z["ndiv2"]
    l1 = (z["level1"] * 127).astype(np.uint8)
    l2 = (z["level2"] * 127).astype(np.uint8)
    res.num_level1 = l1.size
    res.num_boundary = z["bindex"].size
    res.num_level1_inside = int((l1 == 127).sum())
    res.num_level2_inside = int((l2 == 127).sum())
    res.num_level2_boundary = int((l2 == 254).sum())
    for a in range(3):
        res.grid_size[a] = 0.125
        res.grid_size2[a] = 0.03125
    pre = z["prefix"].astype(np.int32)
    n1 = gpv.normal_bytes(z["level1_normal"])
    n2 = gpv.normal_bytes(z["level2_normal"])
    p = str(tmp_path / "Obj-1")
    L = gpv.lib()
    v = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert L.gpv_write_raw(p.encode(), C.byref(res), v(l1), v(pre), v(l2)) == 0
    assert L.gpv_write_raw_normals(p.encode(), C.byref(res), v(n1), v(n2)) == 0
    back = gpv.read_raw(p)
    cfg = back["config"]
    assert list(cfg.ndiv) == list(z["ndiv"]) and list(cfg.ndiv2) == list(z["ndiv2"])
    assert cfg.num_boundary == res.num_boundary and cfg.has_level2 == 1
    assert cfg.num_level1_inside == res.num_level1_inside
    assert cfg.num_level2_boundary == res.num_level2_boundary
    np.testing.assert_array_equal(back["level1InOut"], l1)
    np.testing.assert_array_equal(back["boundaryPrefixSum"], pre)
    np.testing.assert_array_equal(back["level2InOut"], l2)
    np.testing.assert_array_equal(back["level1Normal"], n1)
    np.testing.assert_array_equal(back["level2Normal"], n2)
    # a truncated file is an I/O error, a missing config a parse/IO error
    with open(p + "Level2InOut.raw", "r+b") as f:
        f.truncate(10)
    with pytest.raises(gpv.GpvError):
        gpv.read_raw(p)
    with pytest.raises(gpv.GpvError):
        gpv.read_voxel_config(str(tmp_path / "nothing"))


def test_read_raw_object_reference_layout(built, tmp_path):
    """Object.ReadRAWObject: 48 x 64 x 64 bytes, solid = value % 2 (src/Object.cpp:319-392)."""
    gpv = built
    data = np.random.default_rng(3).choice(np.array([0, 127, 254], np.uint8), 48 * 64 * 64)
    path = tmp_path / "x.raw"
    data.tofile(path)
    obj = gpv.Object()
    obj.bBoxMin = np.zeros(3, np.float32)
    obj.bBoxMax = np.ones(3, np.float32)
    vd = obj.ReadRAWObject(str(path))
    np.testing.assert_array_equal(vd.level1InOut, data)
    np.testing.assert_array_equal(vd.solid, data % 2)
    assert (vd.numDivX, vd.numDivY, vd.numDivZ) == (48, 64, 64)
