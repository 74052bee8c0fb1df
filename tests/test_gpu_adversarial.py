"""GPU parity on triangles aimed at the kernels' certified error bounds (tests/adversarial.py):
slivers around the ray box's conditioning cutoff, t within a few ulps of 1e-6 at Level1 centres and
Level2 origins, vertices a few ulps off Level1/Level2 box planes and binning boundaries, planes
through Level2 cell corners, near-vertical faces and degenerate triangles.  Every byte and every
work count must equal the oracle's brute-force composition (every voxel against every triangle),
through the plain path with both Level2 organisations and through one batched launch."""
import numpy as np
import pytest

import adversarial as A
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _spec(gpv, g):
    s = gpv.GridSpec()
    s.bbox_min[:] = g[0]
    s.bbox_max[:] = g[1]
    s.ndiv[:] = g[2]
    s.ndiv2[:] = g[3]
    return s


def _cases():
    out = []
    for k, g in enumerate(A.GRIDS):
        tris = A.soup(g, orc.grid_tables(g), seed=100 + k)
        out.append((g, tris))
    return out


def _expect(g, tris):
    ref = orc.Run(tris, g, fill=orc.FILL_VOXEL)
    st2, s2, r2 = ref.level2_state()
    return dict(l1=ref.level1_bytes(), pre=ref.prefix(), bi=ref.boundary_index(),
                l2=(st2 * 127).astype(np.uint8),
                work=(ref.sat1_tests(), s2, ref.ray1_candidates(), r2), pairs=ref.num_pairs())


def _check(ctx, res, exp, what):
    l1, pre, bi, l2 = ctx.fetch(res)
    np.testing.assert_array_equal(l1, exp["l1"], err_msg=what)
    np.testing.assert_array_equal(pre, exp["pre"], err_msg=what)
    np.testing.assert_array_equal(bi, exp["bi"], err_msg=what)
    np.testing.assert_array_equal(l2, exp["l2"], err_msg=what)
    assert (res.work.sat1, res.work.sat2, res.work.ray1, res.work.ray2) == exp["work"], what
    assert res.num_pairs == exp["pairs"], what


def test_adversarial_plain_path_both_level2_organisations(ctx):
    import gpview_gb300 as gpv

    try:
        for k, (g, tris) in enumerate(_cases()):
            exp = _expect(g, tris)
            spec = _spec(gpv, g)
            for mode in (gpv.LEVEL2_QUEUED, gpv.LEVEL2_INLINE):
                ctx.set_level2_mode(mode)
                res = ctx.voxelize_host(tris, spec)
                _check(ctx, res, exp, f"grid {k}, Level2 mode {mode}")
                ctx.release(res)
    finally:
        ctx.set_level2_mode(gpv.LEVEL2_AUTO)


def test_adversarial_batched(ctx):
    torch = pytest.importorskip("torch")
    cases = _cases()
    dev = [torch.from_numpy(t).cuda() for _, t in cases]
    import gpview_gb300 as gpv

    res = ctx.voxelize_batch([d.data_ptr() for d in dev], [t.size // 9 for _, t in cases],
                             [_spec(gpv, g) for g, _ in cases])
    for k, ((g, tris), r) in enumerate(zip(cases, res)):
        _check(ctx, r, _expect(g, tris), f"batched grid {k}")
    for r in res:
        ctx.release(r)
