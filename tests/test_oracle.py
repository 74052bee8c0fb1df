"""CPU tests of the oracle: pinned to the reference's own predicate code through the golden
fixtures (tests/golden/make_golden.py), and its fill modes checked against each other."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_sat_predicate_matches_reference_vectors():
    z = np.load(os.path.join(GOLD, "pred_sat.npz"))
    got = np.array([orc.tri_box(c, h, t) for c, h, t in zip(z["center"], z["half"], z["tri"])], np.int8)
    np.testing.assert_array_equal(got, z["hit"])
    assert 0.2 < z["hit"].mean() < 0.8  # both outcomes well represented


def test_ray_predicate_matches_reference_vectors():
    z = np.load(os.path.join(GOLD, "pred_ray.npz"))
    tv, o, d = z["tri"], z["origin"], z["direction"]
    for i in range(len(tv)):
        hit, t = orc.tri_ray(tv[i, 0:3], tv[i, 3:6], tv[i, 6:9], o[i], d[i])
        assert hit == z["hit"][i], i
        if hit:
            assert np.float32(t).view(np.uint32) == z["t"][i].view(np.uint32), i
        if d[i][0] == 0 and d[i][1] == 0 and d[i][2] == 1:
            assert orc.tri_ray_z(tv[i], o[i]) == z["hit"][i], i


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "mesh_*.npz"))),
                         ids=lambda p: os.path.basename(p)[5:-4])
@pytest.mark.parametrize("fill", [orc.FILL_VOXEL, orc.FILL_COLUMN, orc.FILL_CAND])
def test_oracle_matches_golden_meshes(path, fill):
    z = np.load(path)
    grid = (z["bbox_min"], z["bbox_max"], z["ndiv"], z["ndiv2"])
    r = orc.Run(z["tris"], grid, fill=fill)
    np.testing.assert_array_equal(r.level1_state(), z["level1"])
    np.testing.assert_array_equal(r.prefix(), z["prefix"])
    np.testing.assert_array_equal(r.boundary_index(), z["bindex"])
    st2, s2, r2 = r.level2_state()
    np.testing.assert_array_equal(st2, z["level2"])
    np.testing.assert_array_equal([r.sat1_tests(), s2, r.ray1_candidates(), r2], z["work"])


@pytest.mark.skipif(not orc.available(ref=True), reason="reference sources not built here")
def test_restated_predicates_match_reference_live():
    import ctypes as C

    L = C.CDLL(os.path.join(os.path.dirname(orc.__file__), "_ref", "libref_pred.so"))
    L.ref_tri_box.argtypes = [C.c_void_p] * 3
    rng = np.random.default_rng(99)
    n = 20000
    c = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    h = rng.uniform(0.001, 0.05, (n, 3)).astype(np.float32)
    tv = (c[:, None, :] + rng.normal(0, 0.05, (n, 3, 3))).astype(np.float32).reshape(n, 9)
    for i in range(n):
        ref = L.ref_tri_box(c[i].ctypes.data, h[i].ctypes.data, tv[i].ctypes.data)
        assert orc.tri_box(c[i], h[i], tv[i]) == ref


def test_fill_modes_agree_on_sphere16k():
    import workloads as W

    tris, spec = W.make(W.C1)
    a = orc.Run(tris, spec, fill=orc.FILL_COLUMN)
    b = orc.Run(tris, spec, fill=orc.FILL_CAND)
    np.testing.assert_array_equal(a.level1_state(), b.level1_state())
    assert a.B == b.B > 0


@pytest.mark.parametrize("name", ["torus262k", "star1310k"])
def test_candidate_fill_equals_unfiltered_fill_in_full(name):
    """The large plain configurations in full: the candidate-list fill (the mode the GPU parity
    tests compare against) equals the unfiltered per-column fill, which tests every triangle
    against every column with the reference predicate's float operations.  Level2 has no
    prefilter in either mode (its candidate set is the reference's column union)."""
    import workloads as W

    cfg = {"torus262k": W.C2, "star1310k": W.C3}[name]
    tris, grid = W.make(cfg, cpu=True)
    a = orc.Run(tris, grid, fill=orc.FILL_COLUMN)
    b = orc.Run(tris, grid, fill=orc.FILL_CAND)
    assert a.B == b.B > 0
    np.testing.assert_array_equal(a.level1_state(), b.level1_state())
    np.testing.assert_array_equal(a.prefix(), b.prefix())


@pytest.mark.parametrize("k", range(4))
def test_adversarial_soups_candidate_fill_equals_brute_force(k):
    """On the triangles aimed at the certified bounds (tests/adversarial.py), the oracle's
    candidate-list fill equals ClassifyInOutCPU's brute force, and the soups really sit at the
    bounds: slivers on both sides of the rel = 1/8 cutoff, and +z ray tests whose float t lies
    within a few ulps of 1e-6 on both sides."""
    import adversarial as A

    g = A.GRIDS[k]
    tab = orc.grid_tables(g)
    tris = A.soup(g, tab, seed=100 + k)
    a = orc.Run(tris, g, fill=orc.FILL_VOXEL)
    b = orc.Run(tris, g, fill=orc.FILL_CAND)
    assert a.B == b.B > 0
    np.testing.assert_array_equal(a.level1_state(), b.level1_state())
    V = tris.reshape(-1, 9)
    rel, adet = A.sliver_rel(V)
    live = adet > 1e-6
    assert ((rel > 0.11) & (rel <= 0.125) & live).sum() >= 3
    assert ((rel > 0.125) & (rel < 0.14) & live).sum() >= 3
    # the t ~ 1e-6 family: re-find each triangle's nearest threshold crossing over the grid's
    # Level1 centres and Level2 origins directly below its centroid
    n, n2 = [int(x) for x in g[2]], [int(x) for x in g[3]]
    (cx, cy, cz), (ox, oy, oz), _ = A._tables(tab, n, n2)
    ulp = float(np.spacing(np.float32(1e-6)))
    near_hit = near_miss = 0
    for xs, ys, zs in ((cx, cy, cz), (ox, oy, oz)):
        cen = V.reshape(-1, 3, 3).mean(1)
        i = np.clip(np.searchsorted(xs, cen[:, 0]) - 1, 0, len(xs) - 1)
        j = np.clip(np.searchsorted(ys, cen[:, 1]) - 1, 0, len(ys) - 1)
        for di in (0, 1):
            for dj in (0, 1):
                ii = np.clip(i + di, 0, len(xs) - 1)
                jj = np.clip(j + dj, 0, len(ys) - 1)
                kz = np.clip(np.searchsorted(zs, cen[:, 2]) - 1, 0, len(zs) - 1)
                O = np.stack([xs[ii], ys[jj], zs[kz]], 1)
                ins, t, hit = A.ray_z(V, O)
                close = ins & (np.abs(t.astype(np.float64) - 1e-6) <= 8 * ulp)
                near_hit += int((close & hit).sum())
                near_miss += int((close & ~hit).sum())
    assert near_hit >= 10 and near_miss >= 10, (near_hit, near_miss)


def test_as_written_fill_equals_oracle_on_sampled_columns():
    """ClassifyInOutCPU as the reference writes it (every voxel centre against every triangle
    with the general-direction ray test), on seeded columns of sphere16k, gives the oracle's
    inside states wherever no boundary state overrides them."""
    import workloads as W

    tris, grid = W.make(W.C1, cpu=True)
    run = orc.Run(tris, grid, fill=orc.FILL_CAND)
    nx, ny, nz = (int(v) for v in run.spec.n)
    st = run.level1_state().reshape(nz, ny, nx)
    cols = np.random.default_rng(3).choice(nx * ny, 48, replace=False)
    cols = np.concatenate([cols, [(ny // 2) * nx + nx // 2]])  # one column through the middle
    par = run.voxel_fill_columns(cols)
    for c, p in zip(cols, par):
        s = st[:, c // nx, c % nx]
        keep = s != 2
        np.testing.assert_array_equal(p[keep], s[keep])
    assert par.any()


def test_level2_counts_and_list_sampling():
    """The count-only pass and the list form of Level2 agree with the range form."""
    import workloads as W

    tris, grid = W.make(W.C1, cpu=True)
    run = orc.Run(tris, grid)
    st, s2, r2 = run.level2_state()
    assert run.level2_work() == (s2, r2)
    pick = np.array([0, 5, 17, run.B // 2, run.B - 1], np.int64)
    got, _, _ = run.level2_list(pick)
    exp = np.concatenate([st[b * run.cells:(b + 1) * run.cells] for b in pick])
    np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("name", ["sphere16k", "torus262k", "star1310k"])
def test_cpu_workload_generation_is_bit_identical(name, built):
    """The benchmark's reference arm makes its mesh and grid with the oracle library's build of
    the generator source; they equal the GPU library's, bit for bit."""
    import workloads as W

    cfg = {"sphere16k": W.C1, "torus262k": W.C2, "star1310k": W.C3}[name]
    a, spec = W.make(cfg)
    b, grid = W.make(cfg, cpu=True)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    for x, y in ((spec.bbox_min, grid[0]), (spec.bbox_max, grid[1])):
        np.testing.assert_array_equal(np.array(list(x), np.float32).view(np.uint32),
                                      np.asarray(y, np.float32).view(np.uint32))
    assert list(spec.ndiv) == list(grid[2]) and list(spec.ndiv2) == list(grid[3])


def test_reference_sizing_formula():
    # maxModelSize/voxelCount and GetNextDiv4 (src/Object.cpp:3094-3107)
    assert orc.reference_divisions((0, 0, 0), (1.0, 0.5, 0.26), 1.0, 8) == (8, 4, 4)
    assert orc.reference_divisions((0, 0, 0), (1.0, 0.01, 0.3), 1.0, 10) == (12, 4, 4)


def test_op_counts_fixture_sphere16k():
    """The committed algorithmic-work fixture matches a fresh count, and every class's average
    lies between its cheapest and dearest exit (SAT 27..124, ray 20..52 operations)."""
    import json

    import workloads as W

    with open(os.path.join(GOLD, "op_counts.json")) as f:
        fix = json.load(f)
    tris, spec = W.make(W.C1)
    run = orc.Run(tris, spec)
    _, s2, r2 = run.level2_state(0, run.B)
    ops = run.count_ops()
    tests = {"sat1": run.sat1_tests(), "ray1": run.ray1_candidates(), "sat2": s2, "ray2": r2}
    for k in tests:
        assert fix["sphere16k"][k] == {"tests": tests[k], "ops": ops[k]}
    for name in ("sphere16k", "torus262k", "star1310k"):
        for k, (lo, hi) in {"sat1": (27, 124), "sat2": (27, 124), "ray1": (20, 52), "ray2": (20, 52)}.items():
            e = fix[name][k]
            assert lo * e["tests"] <= e["ops"] <= hi * e["tests"], (name, k)


def test_face_normals_match_reference_vectors():
    z = np.load(os.path.join(GOLD, "normal_face.npz"))
    got = np.stack([orc.face_normal(t) for t in z["tri"]])
    np.testing.assert_array_equal(got, z["normal"])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "mesh_*.npz"))),
                         ids=lambda p: os.path.basename(p)[5:-4])
def test_oracle_normals_match_golden_meshes(path):
    z = np.load(path)
    grid = (z["bbox_min"], z["bbox_max"], z["ndiv"], z["ndiv2"])
    r = orc.Run(z["tris"], grid)
    np.testing.assert_array_equal(r.level1_normals(), z["level1_normal"])
    np.testing.assert_array_equal(r.level2_normals(), z["level2_normal"])


def test_normal_bytes_encoding():
    # n * float(256/3) + 127, truncated: -1 -> 41, 0 -> 127, 1 -> 212
    assert list(orc.normal_bytes([-1.0, 0.0, 1.0, 0.5])) == [41, 127, 212, 169]


def test_oracle_hierarchy_structure():
    """Structural checks of the restated BuildHierarchy: N1-1 nodes, the root bounds every solid
    leaf, children indices point one level down, empty nodes have zero boxes."""
    import workloads as W

    tris, spec = W.make(W.C1)
    r = orc.Run(tris, spec)
    lv, h = r.hierarchy()
    assert lv == 18 and h.shape == (r.N1 - 1,)
    assert (h["index"] == np.arange(r.N1 - 1)).all()
    root = h[-1]
    assert root["solid"] == 1
    empty = h["solid"] == 0
    assert (h["mid"][empty] == 0).all() and (h["half"][empty] == 0).all()
    # level-1 children are leaf pairs (2i, 2i+1)
    n1 = r.N1 // 2
    assert (h["child1"][:n1] == 2 * np.arange(n1)).all() and (h["child2"][:n1] == 2 * np.arange(n1) + 1).all()
    # every inside voxel (parity 1) lies in the root box
    tab = orc.grid_tables(spec)
    n = [int(x) for x in spec.ndiv]
    st = r.level1_state().reshape(n[2], n[1], n[0])
    k, j, i = np.nonzero(st == 1)
    c = [tab["c1"][:n[0]][i], tab["c1"][n[0]:n[0] + n[1]][j], tab["c1"][n[0] + n[1]:][k]]
    for a in range(3):
        lo = root["mid"][a] - root["half"][a]
        hi = root["mid"][a] + root["half"][a]
        assert (c[a] - tab["e1"][a] >= lo - 1e-6).all() and (c[a] + tab["e1"][a] <= hi + 1e-6).all()
