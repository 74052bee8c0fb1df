"""Continuous-batching server: results are identical alone and in the mix, requests that arrive
while others run join later batches, and impossible requests are refused on the host."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(gpv, k, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        fam = i % 3
        if fam == 0:
            t = gpv.gen_uvsphere(200 + i, int(rng.integers(16, 96)), int(rng.integers(8, 48)))
        elif fam == 1:
            t = gpv.gen_torus(200 + i, int(rng.integers(32, 128)), int(rng.integers(16, 64)))
        else:
            t = gpv.gen_superellipsoid(200 + i, int(rng.integers(16, 64)), int(rng.integers(8, 32)),
                                       (0.5, 0.5, 0.5), rng.uniform(0.2, 0.45, 3), rng.uniform(0.3, 2),
                                       rng.uniform(0.3, 2))
        spec = gpv.grid_padded(*gpv.mesh_bounds(t), int(rng.choice([32, 64, 96])), int(rng.choice([4, 8])))
        out.append((np.ascontiguousarray(t), spec))
    return out


def test_results_identical_alone_and_in_the_mix(ctx):
    import gpview_gb300 as gpv

    reqs = _requests(gpv, 30)
    srv = gpv.Server(0, budget_bytes=8 << 30, workers=2, max_batch=8)
    tickets = [None] * len(reqs)

    def submit(lo, hi):  # two client threads submitting concurrently
        for i in range(lo, hi):
            tickets[i] = srv.submit(reqs[i][0], reqs[i][1])

    th = [threading.Thread(target=submit, args=(0, 15)), threading.Thread(target=submit, args=(15, 30))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, (tris, spec) in enumerate(reqs):
        rc, res, lat, q = srv.poll(tickets[i], timeout_ms=-1)
        assert rc == 0 and lat >= q >= 0
        mix = ctx.fetch(res)
        alone = ctx.voxelize_host(tris, spec)
        ref = ctx.fetch(alone)
        ctx.release(alone)
        for a, b in zip(mix, ref):
            np.testing.assert_array_equal(a, b)
        assert srv.release(tickets[i]) == 0
    st = srv.stats()
    assert st["served"] == 30 and st["batches"] >= 4 and st["pending"] == 0
    assert st["in_use_bytes"] == 0
    srv.close()


def test_oversize_request_refused_on_host(built):
    gpv = built
    srv = gpv.Server(0, budget_bytes=1 << 20, workers=1, max_batch=4)
    t = gpv.gen_uvsphere(1, 64, 32)
    with pytest.raises(gpv.GpvError) as e:
        srv.submit(t, gpv.grid_padded(*gpv.mesh_bounds(t), 64, 4))
    assert e.value.code == -7
    srv.close()


def test_resident_meshes_identical_and_budgeted(ctx):
    """Meshes uploaded once to the server's pool and requested by id give the same results as
    the same meshes voxelized alone (mixed with host-triangle requests in the same batches); the
    pool counts against the budget until each mesh is removed."""
    import gpview_gb300 as gpv

    reqs = _requests(gpv, 12, seed=9)
    srv = gpv.Server(0, budget_bytes=8 << 30, workers=2, max_batch=6)
    ids = [srv.add_mesh(t) for t, _ in reqs[:6]]
    pool_bytes = sum(t.size * 4 for t, _ in reqs[:6])
    assert srv.stats()["in_use_bytes"] == pool_bytes
    tickets = []
    for k in range(2):  # each resident mesh twice, interleaved with host requests
        for i, mid in enumerate(ids):
            tickets.append((i, srv.submit_mesh(mid, reqs[i][1])))
            tickets.append((6 + (i + 3 * k) % 6, srv.submit(*reqs[6 + (i + 3 * k) % 6])))
    for i, tk in tickets:
        rc, res, lat, q = srv.poll(tk, timeout_ms=-1)
        assert rc == 0
        alone = ctx.voxelize_host(*reqs[i])
        for a, b in zip(ctx.fetch(res), ctx.fetch(alone)):
            np.testing.assert_array_equal(a, b)
        ctx.release(alone)
        assert srv.release(tk) == 0
    assert srv.stats()["in_use_bytes"] == pool_bytes
    for mid in ids:
        assert srv.remove_mesh(mid) == 0
    assert srv.remove_mesh(ids[0]) == -9
    assert srv.stats()["in_use_bytes"] == 0
    with pytest.raises(gpv.GpvError) as e:
        srv.submit_mesh(ids[0], reqs[0][1])
    assert e.value.code == -9
    srv.close()


def test_pool_bigger_than_budget_refused(built):
    gpv = built
    srv = gpv.Server(0, budget_bytes=1 << 20, workers=1, max_batch=4)
    t = gpv.gen_uvsphere(1, 256, 128)  # 65k triangles, 2.3 MB
    with pytest.raises(gpv.GpvError) as e:
        srv.add_mesh(t)
    assert e.value.code == -7
    assert srv.stats()["in_use_bytes"] == 0
    srv.close()
