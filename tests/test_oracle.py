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
