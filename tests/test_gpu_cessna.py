"""The reference's own mesh end to end: files/cessna.obj (committed as tests/golden/cessna.obj)
loaded with the reference's OBJ semantics and 0.001 x diagonal padding (src/Object.cpp:395-584),
sized by GPView's own rule at voxelCount 8 and 32 with voxelCount2 4 (src/Object.cpp:3094-3130),
voxelized on the GPU and written as GPView's .raw files (src/Object.cpp:2934-3075).  Every byte of
every file equals the golden outputs of the reference's CPU composition on the reference's own
predicates (tests/golden/mesh_cessna_v*.npz, made by tests/golden/make_golden.py) and the oracle's
on the same grid."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _read(path, dtype):
    return np.fromfile(path, dtype=dtype)


@pytest.mark.parametrize("voxel_count", [8, 32])
def test_cessna_host_api_and_raw_files(ctx, tmp_path, voxel_count):
    torch = pytest.importorskip("torch")
    import gpview_gb300 as gpv

    z = np.load(os.path.join(GOLD, f"mesh_cessna_v{voxel_count}.npz"))
    obj = gpv.Object(ctx)
    obj.ReadObject(os.path.join(GOLD, "cessna.obj"))
    obj.CreateFlatTriangleData()
    spec = gpv.grid_reference(obj.bBoxMin, obj.bBoxMax, obj.maxModelSize, voxel_count, 4)
    assert list(spec.ndiv) == z["ndiv"].tolist() and list(spec.ndiv2) == [4, 4, 4]
    np.testing.assert_array_equal(np.array(list(spec.bbox_min), np.float32), z["bbox_min"])
    np.testing.assert_array_equal(obj.flatCPUTriangleData, z["tris"])
    # host triangles in, host outputs out (page-locked), then GPView's .raw files
    T = obj.totalNumTriangles
    N1 = int(np.prod(z["ndiv"]))
    B = int(z["bindex"].size)
    h_tris = torch.from_numpy(obj.flatCPUTriangleData).pin_memory()
    h_l1 = torch.empty(N1, dtype=torch.uint8).pin_memory()
    h_pre = torch.empty(N1, dtype=torch.int32).pin_memory()
    h_bi = torch.empty(max(B, 1), dtype=torch.int32).pin_memory()
    h_l2 = torch.empty(max(B * 64, 1), dtype=torch.uint8).pin_memory()
    rc, res = ctx.voxelize_to_host(h_tris.data_ptr(), T, spec, h_l1.data_ptr(), h_pre.data_ptr(),
                                   h_bi.data_ptr(), h_l2.data_ptr(), h_l2.numel())
    assert rc == 0 and res.num_boundary == B
    prefix = str(tmp_path / "Obj-1")
    rc = gpv.lib().gpv_write_raw(prefix.encode(), gpv.C.byref(res), gpv.C.c_void_p(h_l1.data_ptr()),
                                 gpv.C.c_void_p(h_pre.data_ptr()), gpv.C.c_void_p(h_l2.data_ptr()))
    assert rc == 0
    ctx.release(res)
    ref = orc.Run(z["tris"], (z["bbox_min"], z["bbox_max"], z["ndiv"], z["ndiv2"]))
    st2, _, _ = ref.level2_state()
    for exp_gold, exp_orc, name, dt in (
            ((z["level1"] * 127).astype(np.uint8), ref.level1_bytes(), "Level1InOut.raw", np.uint8),
            (z["prefix"], ref.prefix(), "Level1BoundaryPrefixSum.raw", np.int32),
            ((z["level2"] * 127).astype(np.uint8), (st2 * 127).astype(np.uint8), "Level2InOut.raw",
             np.uint8)):
        got = _read(prefix + name, dt)
        np.testing.assert_array_equal(got, exp_gold, err_msg=name)
        np.testing.assert_array_equal(got, exp_orc, err_msg=name)
    cfg = gpv.read_voxel_config(prefix)
    assert list(cfg.ndiv) == z["ndiv"].tolist() and cfg.num_boundary == B


def test_cessna_object_mirror_with_normals(tmp_path):
    """The Python mirror of Object (ReadObject, PerformVoxelization, SaveVoxelization) at
    voxelCount 32: the six files, normals included, equal the golden outputs."""
    import gpview_gb300 as gpv

    z = np.load(os.path.join(GOLD, "mesh_cessna_v32.npz"))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        obj = gpv.Object(gpv.Context(0), objID=-1)
        obj.ReadObject(os.path.join(GOLD, "cessna.obj"))
        obj.PerformVoxelization(gpv.GLParameters(voxelCount=32, voxelCount2=4, saveVoxels=True))
    finally:
        os.chdir(cwd)
    p = str(tmp_path / "Obj-1")
    np.testing.assert_array_equal(_read(p + "Level1InOut.raw", np.uint8), (z["level1"] * 127).astype(np.uint8))
    np.testing.assert_array_equal(_read(p + "Level1BoundaryPrefixSum.raw", np.int32), z["prefix"])
    np.testing.assert_array_equal(_read(p + "Level2InOut.raw", np.uint8), (z["level2"] * 127).astype(np.uint8))
    np.testing.assert_array_equal(_read(p + "Level1Normal.raw", np.uint8),
                                  orc.normal_bytes(z["level1_normal"]).reshape(-1))
    np.testing.assert_array_equal(_read(p + "Level2Normal.raw", np.uint8),
                                  orc.normal_bytes(z["level2_normal"]).reshape(-1))
