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


def test_torus262k_full(ctx):
    tris, spec = W.make(W.C2)
    _check_full(ctx, tris, spec)


def _pad_spec(tris, n, n2):
    import gpview_gb300 as gpv

    mn, mx = gpv.mesh_bounds(tris)
    return gpv.grid_padded(mn, mx, n, n2)


def test_empty_mesh(ctx):
    import gpview_gb300 as gpv

    spec = gpv.grid_padded((0, 0, 0), (1, 1, 1), 16, 4)
    res = ctx.voxelize_host(np.zeros(0, np.float32), spec)
    l1, pre, bi, l2 = ctx.fetch(res)
    assert res.num_boundary == 0 and not l1.any() and not pre.any() and l2.size == 0
    ctx.release(res)


def test_single_open_triangle(ctx):
    tris = np.array([0.1, 0.2, 0.3, 0.9, 0.25, 0.5, 0.4, 0.8, 0.7], np.float32)
    _check_full(ctx, tris, _pad_spec(tris, 12, 4), fill=orc.FILL_VOXEL)


def test_axis_aligned_cube(ctx):
    """Faces on cell boundaries and vertices on the box maximum (the reference's decrement)."""
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                 np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5),
         (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)]
    tris = np.concatenate([v[list(t)].reshape(-1) for t in f]).astype(np.float32)
    import gpview_gb300 as gpv

    for spec in (gpv.grid_padded((0, 0, 0), (1, 1, 1), 10, 2),
                 _spec_exact((0, 0, 0), (1, 1, 1), (8, 8, 8), (4, 4, 4))):
        _check_full(ctx, tris, spec, fill=orc.FILL_VOXEL)


def _spec_exact(mn, mx, n, n2):
    import gpview_gb300 as gpv

    s = gpv.GridSpec()
    s.bbox_min[:] = mn
    s.bbox_max[:] = mx
    s.ndiv[:] = n
    s.ndiv2[:] = n2
    return s


def test_vertices_on_cell_lattice(ctx):
    """Vertices snapped to Level2 cell centres and faces: SAT and ray tests at exact ties, where
    the kernel's certified SAT decisions and slab bounds are closest to their margins."""
    import gpview_gb300 as gpv

    tris = gpv.gen_torus(9, 48, 24, (0.5, 0.5, 0.5), 0.3, 0.12, 0.0).reshape(-1, 3)
    for mn, mx, n, n2 in (((0, 0, 0), (1, 1, 1), (16, 16, 16), (4, 4, 4)),
                          ((-0.25, -0.5, 0.0), (1.25, 1.5, 1.0), (12, 20, 10), (3, 5, 2))):
        mn32, mx32 = np.float32(mn), np.float32(mx)
        half = ((mx32 - mn32) / (np.array(n) * np.array(n2)).astype(np.float32) / 2).astype(np.float32)
        snapped = (mn32 + np.round((tris - mn32) / half).astype(np.float32) * half).astype(np.float32)
        _check_full(ctx, snapped.reshape(-1), _spec_exact(mn, mx, n, n2), fill=orc.FILL_VOXEL)


def test_nonuniform_divisions_and_odd_sizes(ctx):
    import gpview_gb300 as gpv

    tris = gpv.gen_torus(5, 64, 32, (0.5, 0.5, 0.5), 0.3, 0.1, 0.01)
    _check_full(ctx, tris, _pad_spec(tris, (37, 21, 70), (3, 5, 2)))
    _check_full(ctx, tris, _pad_spec(tris, (33, 64, 40), (8, 8, 8)))


def test_superellipsoids_and_tiles(ctx):
    import gpview_gb300 as gpv

    rng = np.random.default_rng(5)
    for k, tile in enumerate((32, 64, 128, 256)):
        ctx.set_tile(tile)
        e1, e2 = rng.uniform(0.3, 2.0, 2)
        semi = rng.uniform(0.2, 0.45, 3)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        tris = gpv.gen_superellipsoid(k, 40, 20, (0.5, 0.5, 0.5), semi, e1, e2, q.astype(np.float32))
        _check_full(ctx, tris, _pad_spec(tris, 40, 4))
    ctx.set_tile(0)


def test_reference_grid_sizing(ctx):
    """GPView's own sizing (voxelCount=8 -> GetNextDiv4 divisions) on a generated mesh."""
    import gpview_gb300 as gpv

    tris = gpv.gen_uvsphere(3, 40, 20, (0.2, -0.3, 1.5), 2.0, 0.01)
    mn, mx = gpv.mesh_bounds(tris)
    pad = np.float32(0.001) * np.linalg.norm(mx - mn)
    spec = gpv.grid_reference(mn - pad, mx + pad, float((mx - mn).max() + 2 * pad), 32, 4)
    _check_full(ctx, tris, spec)


def test_graph_replay_with_other_mesh_data(ctx):
    """Back-to-back calls whose launch arguments are identical (same sizes and counts) replay the
    recorded graphs with the new mesh's data: a torus and its copy shifted by a whole number of
    voxels (exact in float) give equal counts, and both must match the oracle."""
    import gpview_gb300 as gpv

    t = gpv.gen_torus(12, 96, 48, (0.5, 0.5, 0.5), 0.3, 0.1, 0.004)
    t = (np.round(t * 65536.0) / 65536.0).astype(np.float32)  # shifts by 1.0 stay exact
    u = t.reshape(-1, 3).copy()
    u[:, 0] += np.float32(1.0)
    spec = _spec_exact((0, 0, 0), (2, 1, 1), (32, 16, 16), (4, 4, 4))
    refs = []
    for tris in (t, u.reshape(-1), t):
        res = ctx.voxelize_host(tris, spec)
        l1, pre, bi, l2 = ctx.fetch(res)
        ref = orc.Run(tris, spec)
        np.testing.assert_array_equal(l1, ref.level1_bytes())
        np.testing.assert_array_equal(bi, ref.boundary_index())
        np.testing.assert_array_equal(l2, ref.level2_bytes())
        refs.append((res.num_pairs, res.num_boundary))
        ctx.release(res)
    assert refs[0] == refs[1] == refs[2]  # identical sizes: the graphs were replayed


@pytest.mark.parametrize("n,n2", [(16, (32, 32, 32)), (20, (32, 32, 1)), (20, (1, 1, 32)),
                                  (24, (1, 1, 1)), (18, (31, 7, 17))])
def test_extreme_level2_shapes(ctx, n, n2):
    """The largest Level2 grid the API admits (32^3: one boundary voxel per work item, n2z = 32
    columns filling whole mask words), flat and needle-shaped sub-grids, a single sub-cell and odd
    divisions, each against the oracle byte for byte."""
    import gpview_gb300 as gpv

    tris = gpv.gen_uvsphere(21, 40, 20, (0.5, 0.5, 0.5), 0.4, 0.002)
    _check_full(ctx, tris, _pad_spec(tris, n, n2))


def test_large_level1_grid(ctx):
    """A 1536 x 1536 x 32 Level1 grid (75.5 M voxels, 24 words per bit-plane row) around a small
    torus: the bit planes, the column-major pair keys, the boundary scan and the prefix sums at
    large N1, against the oracle."""
    import gpview_gb300 as gpv

    tris = gpv.gen_torus(13, 96, 48, (0.5, 0.5, 0.5), 0.35, 0.12, 0.01)
    _check_full(ctx, tris, _pad_spec(tris, (1536, 1536, 32), (2, 2, 2)))
