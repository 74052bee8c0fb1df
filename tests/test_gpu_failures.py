"""Failure detection, made to happen on the host or by a flag -- never by faulting or hanging the
GPU -- and each followed by a normal call on the same context, bit-exact against the oracle:
  * non-finite vertices: the prep kernel raises its status word, the call returns
    GPV_ERR_INVALID (the reference would voxelize garbage; src/Object.cpp:3200-3214 has no check);
  * a (voxel, triangle) record buffer that overflows: the call re-runs once with the exact
    capacity and its results are exact;
  * the Level1 kernel's bounded wait for its staged tile made to give up: the kernel raises its
    status word, lets the copies in flight land and returns; the call returns GPV_ERR_DEVICE;
  * a refused device allocation: GPV_ERR_OOM.
The reference only prints CUDA errors and carries on (src/CUDAUtilities.cpp:33-49)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _mesh(gpv, seed=3):
    tris = gpv.gen_torus(seed, 64, 32, (0.5, 0.5, 0.5), 0.3, 0.1, 0.01)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), 40, 4)
    return tris, spec


def _exact(ctx, tris, spec):
    res = ctx.voxelize_host(tris, spec)
    l1, pre, bi, l2 = ctx.fetch(res)
    ref = orc.Run(tris, spec)
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(pre, ref.prefix())
    np.testing.assert_array_equal(bi, ref.boundary_index())
    np.testing.assert_array_equal(l2, ref.level2_bytes())
    ctx.release(res)


def test_non_finite_vertex(ctx):
    import gpview_gb300 as gpv

    tris, spec = _mesh(gpv)
    for bad_value in (np.nan, np.inf, -np.inf):
        bad = tris.copy()
        bad[9 * 17 + 4] = bad_value
        with pytest.raises(gpv.GpvError) as e:
            ctx.voxelize_host(bad, spec)
        assert e.value.code == -1 and "non-finite" in str(e.value)
    _exact(ctx, tris, spec)


def test_non_finite_vertex_in_a_batch(ctx):
    torch = pytest.importorskip("torch")
    import gpview_gb300 as gpv

    meshes = [_mesh(gpv, s) for s in (1, 2, 3)]
    bad = meshes[1][0].copy()
    bad[0] = np.nan
    dev = [torch.from_numpy(t).cuda() for t in (meshes[0][0], bad, meshes[2][0])]
    with pytest.raises(gpv.GpvError) as e:
        ctx.voxelize_batch([d.data_ptr() for d in dev], [t.numel() // 9 for t in dev],
                           [s for _, s in meshes])
    assert e.value.code == -1
    _exact(ctx, *meshes[2])


def test_record_buffer_overflow_replans(ctx):
    import gpview_gb300 as gpv

    tris, spec = _mesh(gpv, 5)
    before = ctx.get_debug("replans")
    ctx.set_debug("pair_capacity", 1000)  # far below this mesh's records
    _exact(ctx, tris, spec)
    assert ctx.get_debug("replans") == before + 1
    assert ctx.get_debug("pair_capacity") == 0  # one-shot
    _exact(ctx, tris, spec)
    assert ctx.get_debug("replans") == before + 1


def test_level1_wait_gives_up(ctx):
    import gpview_gb300 as gpv

    tris, spec = _mesh(gpv, 7)
    ctx.set_debug("fail_wait", 1)
    try:
        with pytest.raises(gpv.GpvError) as e:
            ctx.voxelize_host(tris, spec)
        assert e.value.code == -6
    finally:
        ctx.set_debug("fail_wait", 0)
    _exact(ctx, tris, spec)
    # a runtime wait limit well above the staging time changes nothing
    ctx.set_debug("wait_limit", 1 << 20)
    try:
        _exact(ctx, tris, spec)
    finally:
        ctx.set_debug("wait_limit", 0)


def test_allocation_refused(built):
    import gpview_gb300 as gpv

    tris, spec = _mesh(gpv, 9)
    for fresh in (True, False):  # a new context (no workspace yet) and a warm one
        c = gpv.Context(0)
        if not fresh:
            _exact(c, tris, spec)
        c.set_debug("fail_allocs", 1)
        with pytest.raises(gpv.GpvError) as e:
            c.voxelize_host(tris, spec)
        assert e.value.code == -3
        assert c.get_debug("fail_allocs") == 0
        _exact(c, tris, spec)
        c.close()
