"""GPU parity: the C-ABI path against the CPU oracle, bit for bit (integer/byte outputs)."""
import numpy as np
import pytest

from oracle import oracle as orc
import workloads as W

pytestmark = pytest.mark.gpu


def _check_full(ctx, tris, spec, fill=orc.FILL_CAND):
    import gpview_gb300 as gpv

    res = ctx.voxelize_host(tris, spec)
    l1, pre, bi, l2 = ctx.fetch(res)
    ref = orc.Run(tris, spec, fill=fill)
    assert res.num_boundary == ref.B
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(pre, ref.prefix())
    np.testing.assert_array_equal(bi, ref.boundary_index())
    st2, s2, r2 = ref.level2_state()
    np.testing.assert_array_equal(l2, (st2 * 127).astype(np.uint8))
    assert res.num_pairs == ref.num_pairs()
    assert res.work.sat1 == ref.sat1_tests()
    assert res.work.ray1 == ref.ray1_candidates()
    assert res.work.sat2 == s2
    assert res.work.ray2 == r2
    assert res.num_level1_inside == int((l1 == 127).sum())
    assert res.num_level2_inside == int((l2 == 127).sum())
    assert res.num_level2_boundary == int((l2 == 254).sum())
    ctx.release(res)
    return ref


def test_sphere16k_full(ctx):
    tris, spec = W.make(W.C1)
    _check_full(ctx, tris, spec)


def test_small_sphere_vs_brute_force(ctx):
    import gpview_gb300 as gpv

    tris = gpv.gen_uvsphere(11, 24, 12, (0.5, 0.5, 0.5), 0.4, 0.002)
    mn, mx = gpv.mesh_bounds(tris)
    _check_full(ctx, tris, gpv.grid_padded(mn, mx, 20, 4), fill=orc.FILL_VOXEL)
