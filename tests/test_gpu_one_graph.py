"""One-graph calls: a call that repeats the previous call's meshes and grids is recorded as one
CUDA graph (the second half sized on the device).  Its results must equal the two-graph form's
and the oracle's, byte for byte, and a size that does not fit must re-run the call."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _fresh(gpv):
    return gpv.Context(0)


def _batch(gpv, k, seed):
    """k small closed meshes of the three families, Level1 32-64, Level2 {none, 2, 4, 8} (and
    one 16^3), plus an empty mesh."""
    rng = np.random.default_rng(seed)
    meshes = []
    for i in range(k):
        fam = i % 3
        if fam == 0:
            t = gpv.gen_uvsphere(300 + i, int(rng.integers(12, 40)), int(rng.integers(6, 20)),
                                 rng.uniform(0.3, 0.7, 3), rng.uniform(0.2, 0.45), 0.002)
        elif fam == 1:
            t = gpv.gen_torus(300 + i, int(rng.integers(16, 64)), int(rng.integers(8, 32)),
                              rng.uniform(0.4, 0.6, 3), rng.uniform(0.2, 0.35),
                              rng.uniform(0.05, 0.12), 0.01)
        else:
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            t = gpv.gen_superellipsoid(300 + i, int(rng.integers(12, 40)), int(rng.integers(6, 20)),
                                       rng.uniform(0.3, 0.7, 3), rng.uniform(0.2, 0.45, 3),
                                       rng.uniform(0.3, 2.0), rng.uniform(0.3, 2.0),
                                       q.astype(np.float32))
        n1 = int(rng.choice([32, 48, 64]))
        n2 = 16 if i == 2 else int(rng.choice([0, 2, 4, 8]))
        meshes.append((t, gpv.grid_padded(*gpv.mesh_bounds(t), n1, n2)))
    meshes.append((np.zeros(0, np.float32), gpv.grid_padded((0, 0, 0), (1, 1, 1), 16, 2)))
    return meshes


def _upload(torch, meshes):
    return [torch.from_numpy(np.ascontiguousarray(t) if t.size else np.zeros(9, np.float32)).cuda()
            for t, _ in meshes]


def _run(ctx, dev, meshes):
    res = ctx.voxelize_batch([d.data_ptr() for d in dev], [t.size // 9 for t, _ in meshes],
                             [s for _, s in meshes])
    out = [(ctx.fetch(r), (r.work.sat1, r.work.sat2, r.work.ray1, r.work.ray2, r.num_level2_inside,
                           r.num_level2_boundary, r.num_level1_inside)) for r in res]
    for r in res:
        ctx.release(r)
    return out


def _same(a, b):
    for (xa, wa), (xb, wb) in zip(a, b):
        assert wa == wb
        for x, y in zip(xa, xb):
            np.testing.assert_array_equal(x, y)


def test_repeated_batch_runs_as_one_graph_and_matches(built):
    torch = pytest.importorskip("torch")
    gpv = built
    meshes = _batch(gpv, 13, seed=11)
    dev = _upload(torch, meshes)
    ctx = _fresh(gpv)
    try:
        first = _run(ctx, dev, meshes)          # two graphs; records the sizes
        assert ctx.get_debug("one_graph_calls") == 0
        second = _run(ctx, dev, meshes)         # one graph, recorded
        third = _run(ctx, dev, meshes)          # one graph, replayed
        assert ctx.get_debug("one_graph_calls") == 2
        assert ctx.get_debug("one_graph_replans") == 0
        _same(first, second)
        _same(first, third)
        two = _fresh(gpv)
        two.set_graphs(two.GRAPHS_TWO)
        _same(first, _run(two, dev, meshes))
        _same(first, _run(two, dev, meshes))
        assert two.get_debug("one_graph_calls") == 0
        two.close()
        for i in (1, 2, 4, 7):
            t, spec = meshes[i]
            (l1, pre, bi, l2), _ = third[i]
            ref = orc.Run(t, spec)
            np.testing.assert_array_equal(l1, ref.level1_bytes())
            np.testing.assert_array_equal(pre, ref.prefix())
            np.testing.assert_array_equal(bi, ref.boundary_index())
            if spec.ndiv2[0]:
                np.testing.assert_array_equal(l2, ref.level2_bytes())
    finally:
        ctx.close()


@pytest.mark.parametrize("mode", ["queued", "inline"])
def test_one_graph_each_level2_organisation(built, mode):
    torch = pytest.importorskip("torch")
    gpv = built
    meshes = _batch(gpv, 7, seed=23)
    dev = _upload(torch, meshes)
    ctx = _fresh(gpv)
    try:
        ctx.set_level2_mode(getattr(gpv, "LEVEL2_" + mode.upper()))
        first = _run(ctx, dev, meshes)
        second = _run(ctx, dev, meshes)
        assert ctx.get_debug("one_graph_calls") == 1
        _same(first, second)
    finally:
        ctx.close()


def test_plain_path_one_graph_equals_oracle(built):
    """A single mesh voxelized twice: the second call is one graph, bit-exact with the oracle."""
    torch = pytest.importorskip("torch")
    gpv = built
    tris = gpv.gen_torus(5, 128, 64, (0.5, 0.5, 0.5), 0.35, 0.12, 0.01)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), 64, 8)
    d = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    ctx = _fresh(gpv)
    try:
        ctx.set_timing(True)
        a = _run(ctx, [d], [(tris, spec)])
        b = _run(ctx, [d], [(tris, spec)])
        assert ctx.get_debug("one_graph_calls") == 1
        _same(a, b)
        ref = orc.Run(tris, spec)
        (l1, pre, bi, l2), _ = b[0]
        np.testing.assert_array_equal(l1, ref.level1_bytes())
        np.testing.assert_array_equal(l2, ref.level2_bytes())
        calls, st = ctx.stage_times()
        assert calls == 2 and all(v >= 0.0 for v in st.values())
    finally:
        ctx.close()


def test_capacity_overflow_reruns_the_call(built):
    """A one-graph call whose recorded boundary capacity is too small (hook) re-runs with exact
    sizes; so does a call whose triangles moved so that its sizes grew past the capacities."""
    torch = pytest.importorskip("torch")
    gpv = built
    meshes = _batch(gpv, 7, seed=31)
    dev = _upload(torch, meshes)
    ctx = _fresh(gpv)
    try:
        first = _run(ctx, dev, meshes)
        ctx.set_debug("one_graph_capacity", 1)
        again = _run(ctx, dev, meshes)
        assert ctx.get_debug("one_graph_replans") == 1
        _same(first, again)
        # the same counts and grids, larger spheres: the recorded sizes no longer fit
        s_small = gpv.gen_uvsphere(9, 40, 20, (0.5, 0.5, 0.5), 0.1, 0.0)
        s_large = gpv.gen_uvsphere(9, 40, 20, (0.5, 0.5, 0.5), 0.45, 0.0)
        spec = gpv.grid_padded((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 64, 4)
        ds = torch.from_numpy(np.ascontiguousarray(s_small)).cuda()
        dl = torch.from_numpy(np.ascontiguousarray(s_large)).cuda()
        _run(ctx, [ds], [(s_small, spec)])
        r0 = ctx.get_debug("one_graph_replans")
        big = _run(ctx, [dl], [(s_large, spec)])
        assert ctx.get_debug("one_graph_replans") == r0 + 1
        ref = orc.Run(s_large, spec)
        (l1, pre, bi, l2), _ = big[0]
        np.testing.assert_array_equal(l1, ref.level1_bytes())
        np.testing.assert_array_equal(l2, ref.level2_bytes())
        # and the next identical call runs as one graph again
        n0 = ctx.get_debug("one_graph_calls")
        _same(big, _run(ctx, [dl], [(s_large, spec)]))
        assert ctx.get_debug("one_graph_calls") == n0 + 1
    finally:
        ctx.close()
