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
