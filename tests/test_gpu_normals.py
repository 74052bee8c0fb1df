"""GPU normals: Level1 and Level2 voxel normals (float mode) bit for bit against the oracle and
the reference-arithmetic fixtures; the byte mode is the .raw encoding of the float mode; results
are the same alone and inside a batch; occupancy is unchanged by the id-ordered lists."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc
import workloads as W

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _normals(ctx, tris, spec, mode):
    import gpview_gb300 as gpv

    ctx.set_normals(mode)
    try:
        res = ctx.voxelize_host(tris, spec)
    finally:
        ctx.set_normals(gpv.NORMALS_OFF)
    out = ctx.fetch(res), ctx.fetch_normals(res)
    assert res.normal_mode == mode
    ctx.release(res)
    return out


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "mesh_*.npz"))),
                         ids=lambda p: os.path.basename(p)[5:-4])
def test_normals_match_golden_meshes(ctx, path):
    import gpview_gb300 as gpv

    z = np.load(path)
    spec = gpv.GridSpec()
    spec.bbox_min[:] = z["bbox_min"]
    spec.bbox_max[:] = z["bbox_max"]
    spec.ndiv[:] = z["ndiv"]
    spec.ndiv2[:] = z["ndiv2"]
    (l1, pre, bi, l2), (n1, n2) = _normals(ctx, z["tris"], spec, gpv.NORMALS_FLOAT)
    np.testing.assert_array_equal(l1, (z["level1"] * 127).astype(np.uint8))
    np.testing.assert_array_equal(l2, (z["level2"] * 127).astype(np.uint8))
    np.testing.assert_array_equal(n1, z["level1_normal"])
    np.testing.assert_array_equal(n2, z["level2_normal"])


def test_sphere16k_normals_full(ctx):
    import gpview_gb300 as gpv

    tris, spec = W.make(W.C1)
    (l1, _, _, l2), (n1, n2) = _normals(ctx, tris, spec, gpv.NORMALS_FLOAT)
    ref = orc.Run(tris, spec)
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(n1, ref.level1_normals())
    np.testing.assert_array_equal(n2, ref.level2_normals())
    # byte mode = the .raw encoding of the float normals
    _, (b1, b2) = _normals(ctx, tris, spec, gpv.NORMALS_BYTES)
    np.testing.assert_array_equal(b1, gpv.normal_bytes(n1))
    np.testing.assert_array_equal(b2, gpv.normal_bytes(n2))


def test_torus262k_normals_sampled(ctx):
    """Level1 normals in full, Level2 normals on two seeded ranges of boundary voxels."""
    import gpview_gb300 as gpv

    tris, spec = W.make(W.C2)
    (_, _, _, _), (n1, n2) = _normals(ctx, tris, spec, gpv.NORMALS_FLOAT)
    ref = orc.Run(tris, spec)
    np.testing.assert_array_equal(n1, ref.level1_normals())
    cells = 8 ** 3
    rng = np.random.default_rng(7)
    for b0 in rng.integers(0, ref.B - 600, 2):
        b0 = int(b0)
        np.testing.assert_array_equal(n2[b0 * cells:(b0 + 500) * cells], ref.level2_normals(b0, b0 + 500))


def test_level1_only_normals_in_a_mixed_batch(ctx):
    """A batch of a Level2 mesh and a Level1-only mesh: each one's normals equal its oracle."""
    import torch

    import gpview_gb300 as gpv

    t1 = gpv.gen_uvsphere(31, 40, 20, (0.5, 0.5, 0.5), 0.4, 0.002)
    t2 = gpv.gen_torus(32, 48, 24, (0.5, 0.5, 0.5), 0.3, 0.1, 0.01)
    s1 = gpv.grid_padded(*gpv.mesh_bounds(t1), 24, 4)
    s2 = gpv.grid_padded(*gpv.mesh_bounds(t2), 28, 0)
    d1 = torch.from_numpy(t1).cuda()
    d2 = torch.from_numpy(t2).cuda()
    ctx.set_normals(gpv.NORMALS_FLOAT)
    try:
        res = ctx.voxelize_batch([d1.data_ptr(), d2.data_ptr()], [t1.size // 9, t2.size // 9], [s1, s2])
    finally:
        ctx.set_normals(gpv.NORMALS_OFF)
    torch.cuda.synchronize()
    for r, t, s in zip(res, (t1, t2), (s1, s2)):
        l1, _, _, l2 = ctx.fetch(r)
        n1, n2 = ctx.fetch_normals(r)
        ref = orc.Run(t, s)
        np.testing.assert_array_equal(l1, ref.level1_bytes())
        np.testing.assert_array_equal(n1, ref.level1_normals())
        np.testing.assert_array_equal(n2, ref.level2_normals())
        ctx.release(r)


def test_normals_files_written(ctx, tmp_path):
    """Object.PerformVoxelization writes the reference's six files, normals included."""
    import gpview_gb300 as gpv

    tris = gpv.gen_uvsphere(33, 24, 12, (0.5, 0.5, 0.5), 0.4, 0.002)
    obj = gpv.Object(ctx=ctx)
    obj._tris = tris
    mn, mx = gpv.mesh_bounds(tris)
    spec = gpv.grid_padded(mn, mx, 16, 4)
    vd = obj.PerformVoxelization(gpv.GLParameters(saveVoxels=False), spec=spec)
    obj.SaveVoxelization(gpv.GLParameters(), prefix=str(tmp_path / "Obj0"))
    ref = orc.Run(tris, spec)
    n1 = np.fromfile(tmp_path / "Obj0Level1Normal.raw", np.uint8)
    n2 = np.fromfile(tmp_path / "Obj0Level2Normal.raw", np.uint8)
    np.testing.assert_array_equal(n1, orc.normal_bytes(ref.level1_normals()).reshape(-1))
    np.testing.assert_array_equal(n2, orc.normal_bytes(ref.level2_normals()).reshape(-1))
    np.testing.assert_array_equal(vd.level1Normal, ref.level1_normals())


@pytest.mark.parametrize("ndiv", [(16, 8, 4), (32, 32, 32), (64, 64, 64)])
def test_hierarchy_matches_oracle(ctx, ndiv):
    """Object::BuildHierarchy on the device equals the oracle's restatement bit for bit."""
    import gpview_gb300 as gpv

    tris = gpv.gen_torus(41, 96, 48, (0.5, 0.5, 0.5), 0.3, 0.1, 0.01)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), ndiv, 4)
    ctx.set_hierarchy(True)
    try:
        res = ctx.voxelize_host(tris, spec)
    finally:
        ctx.set_hierarchy(False)
    h = ctx.fetch_hierarchy(res)
    ref = orc.Run(tris, spec)
    lv, want = ref.hierarchy()
    assert res.hierarchy_levels == lv
    for f in ("mid", "half", "solid", "child1", "child2", "index"):
        np.testing.assert_array_equal(h[f], want[f], err_msg=f)
    ctx.release(res)


def test_hierarchy_absent_for_non_power_of_two(ctx):
    import gpview_gb300 as gpv

    tris = gpv.gen_uvsphere(42, 24, 12, (0.5, 0.5, 0.5), 0.4, 0.002)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), (12, 8, 8), 0)
    ctx.set_hierarchy(True)
    try:
        res = ctx.voxelize_host(tris, spec)
    finally:
        ctx.set_hierarchy(False)
    assert res.hierarchy_levels == 0 and not res.hierarchy
    with pytest.raises(gpv.GpvError):
        ctx.fetch_hierarchy(res)
    ctx.release(res)


@pytest.mark.parametrize("fill", ["ray", "stencil"])
def test_lists_with_and_without_normals_give_the_same_voxels(ctx, fill):
    """Without normals the pair lists come from a counting sort by voxel (a voxel's triangles in
    any order); with normals, from the radix sort (ascending triangle order).  Every Level1 and
    Level2 output and every work count is the same either way."""
    import gpview_gb300 as gpv

    tris, spec = W.make(W.C2)
    ctx.set_fill(gpv.FILL_STENCIL if fill == "stencil" else gpv.FILL_RAY)
    try:
        out = []
        for mode in (gpv.NORMALS_OFF, gpv.NORMALS_BYTES):
            ctx.set_normals(mode)
            try:
                res = ctx.voxelize_host(tris, spec)
            finally:
                ctx.set_normals(gpv.NORMALS_OFF)
            out.append((ctx.fetch(res), (res.num_pairs, res.num_boundary, res.work.sat1,
                                         res.work.sat2, res.work.ray1, res.work.ray2)))
            ctx.release(res)
    finally:
        ctx.set_fill(gpv.FILL_RAY)
    (a, wa), (b, wb) = out
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert wa == wb
