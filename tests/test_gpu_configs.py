"""GPU parity on the two largest benchmark configurations, against the oracle:
  * the large, skewed plain mesh (star1310k: 1,310,720 triangles, 256^3 / 16^3) with every Level1
    and Level2 byte and every work count compared;
  * a seeded 256-mesh subset of the 4096-mesh batched workload -- every Level1 size up to 128^3,
    every Level2 size up to 8^3 and the meshes above 100k triangles included -- run as one batch
    with the tunables the autotuner picks for it (tile 256, Level2 chunk 16) under each Level2
    organisation, every mesh's outputs compared with its own oracle run.
The oracle's candidate-list fill is checked equal to its unfiltered fill on the large plain
configurations by the CPU tests."""
import hashlib

import numpy as np
import pytest

import workloads as W
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_star1310k_full(ctx):
    tris, spec = W.make(W.C3)
    res = ctx.voxelize_host(tris, spec)
    l1, pre, bi, l2 = ctx.fetch(res)
    ref = orc.Run(tris, spec, fill=orc.FILL_CAND)
    assert res.num_boundary == ref.B
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(pre, ref.prefix())
    np.testing.assert_array_equal(bi, ref.boundary_index())
    assert res.num_pairs == ref.num_pairs()
    del l1, pre, bi
    st2, s2, r2 = ref.level2_state()
    assert st2.size == l2.size
    # compare in slabs of boundary voxels so a mismatch names its place
    cells = ref.cells
    step = 16384
    for b0 in range(0, ref.B, step):
        b1 = min(b0 + step, ref.B)
        got = l2[b0 * cells:b1 * cells]
        exp = (st2[b0 * cells:b1 * cells] * 127).astype(np.uint8)
        if not np.array_equal(got, exp):
            bad = np.nonzero(got != exp)[0][:5] + b0 * cells
            raise AssertionError(f"Level2 differs at cells {bad.tolist()} (boundary voxels "
                                 f"{(bad // cells).tolist()})")
    assert (res.work.sat1, res.work.sat2, res.work.ray1, res.work.ray2) == \
           (ref.sat1_tests(), s2, ref.ray1_candidates(), r2)
    assert res.num_level2_inside == int((st2 == 1).sum())
    assert res.num_level2_boundary == int((st2 == 2).sum())
    ctx.release(res)


def _subset(meshes, count=256, seed=77):
    """Every mesh with T >= 100k on a 128^3 / 8^3 grid, then T >= 100k on any grid, then seeded
    picks, up to `count`; and at least one mesh of every Level1 and Level2 size."""
    rng = np.random.default_rng(seed)
    T = np.array([t.size // 9 for t, _ in meshes])
    n1 = np.array([s.ndiv[0] for _, s in meshes])
    n2 = np.array([s.ndiv2[0] for _, s in meshes])
    chosen = list(np.nonzero((T >= 100000) & (n1 == 128) & (n2 == 8))[0][:40])
    for i in np.nonzero(T >= 100000)[0]:
        if len(chosen) >= 80:
            break
        if i not in chosen:
            chosen.append(i)
    for a in (32, 48, 64, 96, 128):
        for b in (2, 4, 8):
            hit = np.nonzero((n1 == a) & (n2 == b))[0]
            if hit.size and not set(hit) & set(chosen):
                chosen.append(int(hit[0]))
    rest = [i for i in rng.permutation(len(meshes)) if i not in set(chosen)]
    chosen += rest[:max(0, count - len(chosen))]
    return sorted(int(i) for i in chosen[:count])


def _digest(arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_batch4096_subset_vs_oracle(ctx):
    torch = pytest.importorskip("torch")
    import gpview_gb300 as gpv

    meshes = W.batch4096(4096)
    pick = _subset(meshes)
    sub = [meshes[i] for i in pick]
    T = [t.size // 9 for t, _ in sub]
    assert len(sub) >= 256 and max(T) >= 100000
    assert {s.ndiv[0] for _, s in sub} == {32, 48, 64, 96, 128}
    assert {s.ndiv2[0] for _, s in sub} == {2, 4, 8}
    dev = [torch.from_numpy(t).cuda() for t, _ in sub]
    ptrs = [d.data_ptr() for d in dev]
    specs = [s for _, s in sub]
    got = {}
    ctx.set_tile(256)
    ctx.set_level2_chunk(16)
    try:
        for mode in (gpv.LEVEL2_AUTO, gpv.LEVEL2_QUEUED, gpv.LEVEL2_INLINE):
            ctx.set_level2_mode(mode)
            res = ctx.voxelize_batch(ptrs, T, specs)
            got[mode] = [(_digest(ctx.fetch(r)), (r.work.sat1, r.work.sat2, r.work.ray1, r.work.ray2))
                         for r in res]
            for r in res:
                ctx.release(r)
    finally:
        ctx.set_level2_mode(gpv.LEVEL2_AUTO)
        ctx.set_tile(0)
        ctx.set_level2_chunk(8)
    for k, (tris, spec) in enumerate(sub):
        ref = orc.Run(tris, spec, fill=orc.FILL_CAND)
        st2, s2, r2 = ref.level2_state()
        exp = (_digest([ref.level1_bytes(), ref.prefix(), ref.boundary_index(),
                        (st2 * 127).astype(np.uint8)]),
               (ref.sat1_tests(), s2, ref.ray1_candidates(), r2))
        for mode, lst in got.items():
            assert lst[k] == exp, (f"mesh {pick[k]} (T={T[k]}, Level1 {list(spec.ndiv)}, "
                                   f"Level2 {list(spec.ndiv2)}) differs from the oracle "
                                   f"under Level2 mode {mode}")
