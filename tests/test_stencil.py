"""The stencil (rasterised) inside fill, GPV_FILL_STENCIL: ClassifyInOut2x (src/Object.cpp:
1446-1649) and ClassifyInOut2xLevel2 (:1210-1444), which the reference runs through OpenGL.

No graphics stack exists on either machine, so parity for this fill is pinned to a restatement
of the rasterisation (oracle/gpv_oracle.c, orc_st_*).  The CPU tests check the oracle, which
accumulates one toggle per (triangle, sample), against a literal slice-by-slice form of the two
functions written here (every slice renders every triangle into a stencil buffer, then the 2x2
majority), and check that the stencil fill agrees with the ray fill away from the surface.  The
GPU tests check the library bit for bit against the oracle."""
import numpy as np
import pytest

from oracle import oracle as orc

F = np.float32


def _snap(v, lo, hi, npx):
    w = F(F(F(v) - F(lo)) / F(F(hi) - F(lo))) * F(npx)
    if not (w > F(-2097152.0)):
        w = F(-2097152.0)
    elif w > F(2097152.0):
        w = F(2097152.0)
    return int(np.rint(F(w * F(256.0))))


def _i2f(x):
    return np.array(x, np.int64).astype(np.float32)[()]


def _fragments(tv, lx, hx, ly, hy, W, H):
    """{(sx, sy): height} of the samples one triangle covers (the oracle's coverage rules)."""
    X = [_snap(tv[3 * i], lx, hx, W) for i in range(3)]
    Y = [_snap(tv[3 * i + 1], ly, hy, H) for i in range(3)]
    z = [F(tv[3 * i + 2]) for i in range(3)]
    A = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0])
    if A == 0:
        return {}
    if A < 0:
        X[1], X[2], Y[1], Y[2], z[1], z[2] = X[2], X[1], Y[2], Y[1], z[2], z[1]
        A = -A
    rA = F(1.0) / _i2f(A)
    out = {}
    for sy in range(max(0, -((128 - min(Y)) // 256)), min(H - 1, (max(Y) - 128) // 256) + 1):
        for sx in range(max(0, -((128 - min(X)) // 256)), min(W - 1, (max(X) - 128) // 256) + 1):
            px, py = 256 * sx + 128, 256 * sy + 128
            w = []
            for e in range(3):
                a, b = (e + 1) % 3, (e + 2) % 3
                dx, dy = X[b] - X[a], Y[b] - Y[a]
                we = dx * (py - Y[a]) - dy * (px - X[a])
                if not (we > 0 or (we == 0 and (dy < 0 or (dy == 0 and dx > 0)))):
                    break
                w.append(we)
            else:
                zs = F(F(F(_i2f(w[0]) * rA) * z[0]) + F(F(_i2f(w[1]) * rA) * z[1]))
                out[(sx, sy)] = F(zs + F(F(_i2f(w[2]) * rA) * z[2]))
    return out


def _majority(stencil):
    """numInsideCount > 2 over each voxel's 2x2 samples; stencil [H, W] of counts."""
    odd = (stencil % 2).astype(np.int32)
    return (odd[0::2, 0::2] + odd[0::2, 1::2] + odd[1::2, 0::2] + odd[1::2, 1::2]) > 2


def slice_loop_level1(tris, grid):
    """ClassifyInOut2x, one stencil rendering per slice: [nz, ny, nx] 0/1."""
    bmin, bmax, n, _ = grid
    bmin, bmax = np.asarray(bmin, F), np.asarray(bmax, F)
    nx, ny, nz = (int(v) for v in n)
    gz = F(float(F(bmax[2] - bmin[2])) / (nz * 1.0))  # float((max - min) / (n * 1.0))
    frags = [_fragments(tris[9 * t:9 * t + 9], bmin[0], bmax[0], bmin[1], bmax[1], 2 * nx, 2 * ny)
             for t in range(len(tris) // 9)]
    out = np.zeros((nz, ny, nx), np.uint8)
    for k in range(nz):
        clip = F((k + 0.5) * float(gz) + float(bmin[2]))
        stencil = np.zeros((2 * ny, 2 * nx), np.int64)
        for fr in frags:
            for (sx, sy), zs in fr.items():
                if zs <= clip:
                    stencil[sy, sx] += 1
        out[k] = _majority(stencil)
    return out


def slice_loop_level2(tris, grid, run, b):
    """ClassifyInOut2xLevel2 for boundary voxel b (strip = the column's recorded triangles):
    [n2z, n2y, n2x] 0/1."""
    bmin, bmax, n, n2 = grid
    bmin, bmax = np.asarray(bmin, F), np.asarray(bmax, F)
    nx, ny, nz = (int(v) for v in n)
    n2x, n2y, n2z = (int(v) for v in n2)
    g = [F(float(F(bmax[a] - bmin[a])) / (int(n[a]) * 1.0)) for a in range(3)]
    g2z = F(float(g[2]) / (n2z * 1.0))
    v = int(run.boundary_index()[b])
    k, ij = divmod(v, nx * ny)
    j, i = divmod(ij, nx)
    lx = F(F(F(i) * g[0]) + bmin[0])
    ly = F(F(F(j) * g[1]) + bmin[1])
    minz = F(F(F(k) * g[2]) + bmin[2])
    strip = []
    for z in range(nz):
        for t in run.voxel_tris(z * nx * ny + ij):
            if t not in strip:
                strip.append(int(t))
    frags = [_fragments(tris[9 * t:9 * t + 9], lx, F(lx + g[0]), ly, F(ly + g[1]), 2 * n2x, 2 * n2y)
             for t in strip]
    out = np.zeros((n2z, n2y, n2x), np.uint8)
    for s in range(n2z):
        clip = F(float(minz) + (s + 0.5) * float(g2z))
        stencil = np.zeros((2 * n2y, 2 * n2x), np.int64)
        for fr in frags:
            for (sx, sy), zs in fr.items():
                if zs <= clip:
                    stencil[sy, sx] += 1
        out[s] = _majority(stencil)
    return out


def _uvsphere(nu, nv, c, r, rot=0.3):
    """Closed UV sphere, float32 triangle soup."""
    th = np.linspace(0, np.pi, nv + 1)
    ph = np.linspace(0, 2 * np.pi, nu + 1)[:-1] + rot
    P = lambda a, b: (c[0] + r * np.sin(a) * np.cos(b), c[1] + r * np.sin(a) * np.sin(b), c[2] + r * np.cos(a))
    tris = []
    for a in range(nv):
        for b in range(nu):
            p00, p01 = P(th[a], ph[b]), P(th[a], ph[(b + 1) % nu])
            p10, p11 = P(th[a + 1], ph[b]), P(th[a + 1], ph[(b + 1) % nu])
            if a > 0:
                tris.append(p00 + p10 + p01)
            if a < nv - 1:
                tris.append(p01 + p10 + p11)
    return np.asarray(tris, np.float32).reshape(-1)


def _cube(lo, hi):
    v = np.array([[lo[0], lo[1], lo[2]], [hi[0], lo[1], lo[2]], [hi[0], hi[1], lo[2]], [lo[0], hi[1], lo[2]],
                  [lo[0], lo[1], hi[2]], [hi[0], lo[1], hi[2]], [hi[0], hi[1], hi[2]], [lo[0], hi[1], hi[2]]],
                 np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5),
         (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)]
    return np.concatenate([v[list(t)].reshape(-1) for t in f]).astype(np.float32)


CASES = {
    "sphere": (_uvsphere(14, 9, (0.5, 0.45, 0.55), 0.37), ((0, 0, 0), (1, 1, 1), (9, 8, 7), (2, 3, 2))),
    # faces on cell boundaries, sample centres and clip heights: ties everywhere
    "cube": (_cube((0.25, 0.25, 0.25), (0.75, 0.75, 0.75)), ((0, 0, 0), (1, 1, 1), (8, 8, 8), (2, 2, 2))),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_level1_equals_slice_loop(case):
    tris, grid = CASES[case]
    r = orc.Run(tris, grid, fill=orc.FILL_STENCIL)
    st = r.level1_state().reshape(slice_loop_level1(tris, grid).shape)
    lit = slice_loop_level1(tris, grid)
    # the boundary marks (2) override the fill; compare the fill where they do not
    np.testing.assert_array_equal(np.where(st == 2, lit, st), lit)
    assert lit.sum() > 0 and r.ray1_candidates() == 0


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_level2_equals_slice_loop(case):
    tris, grid = CASES[case]
    r = orc.Run(tris, grid, fill=orc.FILL_STENCIL)
    states, _, ray2 = r.level2_state()
    n2 = tuple(int(v) for v in grid[3])
    cells = n2[0] * n2[1] * n2[2]
    assert ray2 == 0
    inside = 0
    for b in range(0, r.B, max(1, r.B // 12)):
        blk = states[b * cells:(b + 1) * cells].reshape(n2[2], n2[1], n2[0])
        lit = slice_loop_level2(tris, grid, r, b)
        np.testing.assert_array_equal(np.where(blk == 2, lit, blk), lit)
        inside += int(lit.sum())
    assert inside > 0


def test_stencil_agrees_with_ray_fill_inside():
    """Both fills classify a closed surface's interior the same way away from the surface."""
    tris = _uvsphere(48, 32, (0.5, 0.5, 0.5), 0.4)
    grid = ((0, 0, 0), (1, 1, 1), (32, 32, 32), (0, 0, 0))
    a = orc.Run(tris, grid, fill=orc.FILL_STENCIL).level1_state().reshape(32, 32, 32)
    b = orc.Run(tris, grid, fill=orc.FILL_CAND).level1_state().reshape(32, 32, 32)
    bnd = b == 2
    near = bnd.copy()
    for ax in range(3):
        near |= np.roll(bnd, 1, ax) | np.roll(bnd, -1, ax)
    assert (a[~near] == b[~near]).all()
    assert (a == 1).sum() > 0.9 * (b == 1).sum()


# ---------------------------------------------------------------------------------- GPU parity

def _check_stencil(ctx, tris, spec):
    import gpview_gb300 as gpv

    ctx.set_fill(gpv.FILL_STENCIL)
    try:
        res = ctx.voxelize_host(tris, spec)
    finally:
        ctx.set_fill(gpv.FILL_RAY)
    l1, pre, bi, l2 = ctx.fetch(res)
    ref = orc.Run(tris, spec, fill=orc.FILL_STENCIL)
    assert res.num_boundary == ref.B
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(pre, ref.prefix())
    np.testing.assert_array_equal(bi, ref.boundary_index())
    st2, s2, r2 = ref.level2_state()
    np.testing.assert_array_equal(l2, (st2 * 127).astype(np.uint8))
    assert res.work.ray1 == 0 and res.work.ray2 == 0 and r2 == 0
    assert res.work.sat2 == s2
    assert res.num_level1_inside == int((l1 == 127).sum())
    assert res.num_level2_inside == int((l2 == 127).sum())
    ctx.release(res)
    return l1, l2


def _spec(mn, mx, n, n2):
    import gpview_gb300 as gpv

    s = gpv.GridSpec()
    s.bbox_min[:] = mn
    s.bbox_max[:] = mx
    s.ndiv[:] = n
    s.ndiv2[:] = n2
    return s


@pytest.mark.gpu
def test_gpu_stencil_sphere16k(ctx):
    import workloads as W

    tris, spec = W.make(W.C1)
    l1, l2 = _check_stencil(ctx, tris, spec)
    assert (l1 == 127).sum() > 0 and (l2 == 127).sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_stencil_small_cases(ctx, case):
    tris, grid = CASES[case]
    _check_stencil(ctx, tris, _spec(*grid))


@pytest.mark.gpu
@pytest.mark.parametrize("cap", [1, 2, 5])
def test_gpu_stencil_short_chunks(ctx, cap):
    """Level2 work items of 1, 2 and 5 boundary voxels split every column into many items: each
    starts from the sample-coverage XOR of the column's triangles recorded only below it (the
    segment masks and their per-column prefix)."""
    import workloads as W

    tris, spec = W.make(W.C1)
    ctx.set_level2_chunk(cap)
    try:
        _check_stencil(ctx, tris, spec)
    finally:
        ctx.set_level2_chunk(16)


@pytest.mark.gpu
def test_gpu_stencil_torus_nonuniform(ctx):
    import gpview_gb300 as gpv

    tris = gpv.gen_torus(5, 96, 48, (0.5, 0.5, 0.5), 0.3, 0.1, 0.01)
    mn, mx = gpv.mesh_bounds(tris)
    _check_stencil(ctx, tris, gpv.grid_padded(mn, mx, (37, 21, 70), (3, 5, 2)))
    _check_stencil(ctx, tris, gpv.grid_padded(mn, mx, 48, 8))


@pytest.mark.gpu
def test_gpu_stencil_lattice_ties(ctx):
    """Vertices on Level2 cell centres and faces: samples on edges and vertices, heights equal
    to clip heights."""
    import gpview_gb300 as gpv

    tris = gpv.gen_torus(9, 48, 24, (0.5, 0.5, 0.5), 0.3, 0.12, 0.0).reshape(-1, 3)
    for mn, mx, n, n2 in (((0, 0, 0), (1, 1, 1), (16, 16, 16), (4, 4, 4)),
                          ((-0.25, -0.5, 0.0), (1.25, 1.5, 1.0), (12, 20, 10), (3, 5, 2))):
        mn32 = np.float32(mn)
        half = ((np.float32(mx) - mn32) / (np.array(n) * np.array(n2)).astype(np.float32) / 4).astype(np.float32)
        snapped = (mn32 + np.round((tris - mn32) / half).astype(np.float32) * half).astype(np.float32)
        _check_stencil(ctx, snapped.reshape(-1), _spec(mn, mx, n, n2))


@pytest.mark.gpu
def test_gpu_stencil_batch_equals_alone(ctx):
    import gpview_gb300 as gpv

    torch = pytest.importorskip("torch")

    rng = np.random.default_rng(11)
    meshes, specs = [], []
    for k in range(6):
        t = gpv.gen_uvsphere(k, 24 + 8 * k, 12 + 4 * k, tuple(rng.uniform(0.35, 0.65, 3)),
                             float(rng.uniform(0.15, 0.3)), 0.004)
        mn, mx = gpv.mesh_bounds(t)
        meshes.append(t)
        specs.append(gpv.grid_padded(mn, mx, int(rng.choice([16, 24, 32])), int(rng.choice([2, 4]))))
    dev = [torch.from_numpy(np.ascontiguousarray(t)).cuda() for t in meshes]
    ctx.set_fill(gpv.FILL_STENCIL)
    try:
        res = ctx.voxelize_batch([d.data_ptr() for d in dev], [t.size // 9 for t in meshes], specs)
        torch.cuda.synchronize()
    finally:
        ctx.set_fill(gpv.FILL_RAY)
    for t, s, r in zip(meshes, specs, res):
        l1, _, _, l2 = ctx.fetch(r)
        ref = orc.Run(t, s, fill=orc.FILL_STENCIL)
        np.testing.assert_array_equal(l1, ref.level1_bytes())
        np.testing.assert_array_equal(l2, (ref.level2_state()[0] * 127).astype(np.uint8))
        ctx.release(r)


@pytest.mark.gpu
@pytest.mark.parametrize("slabs", [0, 3])
def test_gpu_stencil_with_normals_and_hierarchy_to_host(ctx, slabs):
    """Stencil fill with normals and the box hierarchy switched on, host to host (Level2 written
    straight into page-locked memory, or copied per z slab): every output equals the oracle's."""
    import gpview_gb300 as gpv
    torch = pytest.importorskip("torch")

    tris = gpv.gen_torus(23, 128, 64, (0.5, 0.5, 0.5), 0.3, 0.1, 0.006)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), 32, 4)
    ref = orc.Run(tris, spec, fill=orc.FILL_STENCIL)
    n1, cells = 32 ** 3, 4 ** 3
    h_tris = torch.from_numpy(tris).pin_memory()
    l1 = torch.empty(n1, dtype=torch.uint8).pin_memory()
    pre = torch.empty(n1, dtype=torch.int32).pin_memory()
    bi = torch.empty(ref.B, dtype=torch.int32).pin_memory()
    l2 = torch.empty(ref.B * cells, dtype=torch.uint8).pin_memory()
    ctx.set_fill(gpv.FILL_STENCIL)
    ctx.set_normals(gpv.NORMALS_FLOAT)
    ctx.set_hierarchy(True)
    try:
        rc, res = ctx.voxelize_to_host(h_tris.data_ptr(), tris.size // 9, spec, l1.data_ptr(),
                                       pre.data_ptr(), bi.data_ptr(), l2.data_ptr(),
                                       ref.B * cells, slabs)
    finally:
        ctx.set_fill(gpv.FILL_RAY)
        ctx.set_normals(gpv.NORMALS_OFF)
        ctx.set_hierarchy(False)
    assert rc == 0 and res.num_boundary == ref.B
    np.testing.assert_array_equal(l1.numpy(), ref.level1_bytes())
    np.testing.assert_array_equal(pre.numpy(), ref.prefix())
    np.testing.assert_array_equal(bi.numpy(), ref.boundary_index())
    np.testing.assert_array_equal(l2.numpy(), ref.level2_bytes())
    m1, m2 = ctx.fetch_normals(res)
    np.testing.assert_array_equal(m1, ref.level1_normals())
    np.testing.assert_array_equal(m2, ref.level2_normals())
    lv, want = ref.hierarchy()
    h = ctx.fetch_hierarchy(res)
    assert res.hierarchy_levels == lv
    for f in ("mid", "half", "solid", "child1", "child2", "index"):
        np.testing.assert_array_equal(h[f], want[f], err_msg=f)
    ctx.release(res)
