"""Batched path: a mixed batch gives, mesh by mesh, exactly what each mesh gives alone, and
what the oracle gives."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _mixed_meshes(gpv, k, seed=7):
    rng = np.random.default_rng(seed)
    meshes = []
    for i in range(k):
        fam = i % 3
        if fam == 0:
            t = gpv.gen_uvsphere(100 + i, int(rng.integers(12, 40)), int(rng.integers(6, 20)),
                                 rng.uniform(0.3, 0.7, 3), rng.uniform(0.2, 0.45), 0.002)
        elif fam == 1:
            t = gpv.gen_torus(100 + i, int(rng.integers(16, 64)), int(rng.integers(8, 32)),
                              rng.uniform(0.4, 0.6, 3), rng.uniform(0.2, 0.35), rng.uniform(0.05, 0.12), 0.01)
        else:
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            t = gpv.gen_superellipsoid(100 + i, int(rng.integers(12, 40)), int(rng.integers(6, 20)),
                                       rng.uniform(0.3, 0.7, 3), rng.uniform(0.2, 0.45, 3),
                                       rng.uniform(0.3, 2.0), rng.uniform(0.3, 2.0), q.astype(np.float32))
        n1 = int(rng.choice([32, 48, 64]))
        n2 = int(rng.choice([0, 2, 4, 8])) if i else 0
        spec = gpv.grid_padded(*gpv.mesh_bounds(t), n1, n2)
        meshes.append((t, spec))
    meshes.append((np.zeros(0, np.float32), gpv.grid_padded((0, 0, 0), (1, 1, 1), 16, 2)))
    return meshes


def test_batch_equals_alone_and_oracle(ctx):
    torch = pytest.importorskip("torch")
    import gpview_gb300 as gpv

    meshes = _mixed_meshes(gpv, 14)
    dev = [torch.from_numpy(np.ascontiguousarray(t) if t.size else np.zeros(9, np.float32)).cuda()
           for t, _ in meshes]
    res = ctx.voxelize_batch([d.data_ptr() for d in dev], [t.size // 9 for t, _ in meshes],
                             [s for _, s in meshes])
    for i, ((t, spec), rb) in enumerate(zip(meshes, res)):
        a = ctx.fetch(rb)
        ra = ctx.voxelize_host(t, spec)
        b = ctx.fetch(ra)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
        assert (rb.work.sat1, rb.work.sat2, rb.work.ray1, rb.work.ray2) == \
               (ra.work.sat1, ra.work.sat2, ra.work.ray1, ra.work.ray2)
        ctx.release(ra)
        if i % 4 == 1 and t.size:
            ref = orc.Run(t, spec)
            np.testing.assert_array_equal(a[0], ref.level1_bytes())
            np.testing.assert_array_equal(a[1], ref.prefix())
            if spec.ndiv2[0]:
                np.testing.assert_array_equal(a[3], ref.level2_bytes())
    for rb in res:
        ctx.release(rb)


def test_golden_fixtures_on_gpu(ctx):
    import glob
    import os

    import gpview_gb300 as gpv

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for path in sorted(glob.glob(os.path.join(gold, "mesh_*.npz"))):
        z = np.load(path)
        s = gpv.GridSpec()
        s.bbox_min[:] = z["bbox_min"].tolist()
        s.bbox_max[:] = z["bbox_max"].tolist()
        s.ndiv[:] = z["ndiv"].tolist()
        s.ndiv2[:] = z["ndiv2"].tolist()
        r = ctx.voxelize_host(z["tris"], s)
        l1, pre, bi, l2 = ctx.fetch(r)
        np.testing.assert_array_equal(l1, (z["level1"] * 127).astype(np.uint8), err_msg=path)
        np.testing.assert_array_equal(pre, z["prefix"], err_msg=path)
        np.testing.assert_array_equal(bi, z["bindex"], err_msg=path)
        np.testing.assert_array_equal(l2, (z["level2"] * 127).astype(np.uint8), err_msg=path)
        assert [r.work.sat1, r.work.sat2, r.work.ray1, r.work.ray2] == z["work"].tolist()
        ctx.release(r)


def test_large_batch_host_work_in_threads(ctx):
    """A batch of 200 meshes: the per-mesh grid derivation and table packing run on several host
    threads; every sampled mesh still equals its single-mesh result."""
    torch = pytest.importorskip("torch")
    import gpview_gb300 as gpv

    meshes = _mixed_meshes(gpv, 200, seed=11)
    dev = [torch.from_numpy(np.ascontiguousarray(t) if t.size else np.zeros(9, np.float32)).cuda()
           for t, _ in meshes]
    res = ctx.voxelize_batch([d.data_ptr() for d in dev], [t.size // 9 for t, _ in meshes],
                             [s for _, s in meshes])
    for i in range(0, len(meshes), 17):
        t, spec = meshes[i]
        ra = ctx.voxelize_host(t, spec)
        for x, y in zip(ctx.fetch(res[i]), ctx.fetch(ra)):
            np.testing.assert_array_equal(x, y)
        ctx.release(ra)
    for rb in res:
        ctx.release(rb)
