"""The allocation-free Level1 entry point against the plain path (collected last on purpose).

gpv_voxelize_level1_noalloc exists for callers that cannot call cudaMalloc (allocator hooks,
paths that must not synchronise the device, plugin hosts that own all device memory).  It keeps
its intermediates in a fixed device array shared by every call, so two calls in a row -- with
different meshes and grids -- must each reproduce gpv_voxelize's Level1 outputs exactly.
"""
import ctypes as C

import numpy as np
import pytest

import workloads as W
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _noalloc(gpv, torch, tris, spec):
    L = gpv.lib()
    n1 = int(np.prod(list(spec.ndiv)))
    d_tris = torch.from_numpy(np.ascontiguousarray(tris, np.float32)).cuda()
    # poison the outputs so that stale or unwritten entries show up
    l1 = torch.full((n1,), 0xAB, dtype=torch.uint8, device="cuda")
    pre = torch.full((n1,), -7, dtype=torch.int32, device="cuda")
    bi = torch.full((n1,), -7, dtype=torch.int32, device="cuda")
    nb = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gpv_voxelize_level1_noalloc(C.c_void_p(d_tris.data_ptr()), tris.size // 9, C.byref(spec),
                                       C.c_void_p(l1.data_ptr()), C.c_void_p(pre.data_ptr()),
                                       C.c_void_p(bi.data_ptr()), C.byref(nb), C.c_void_p(stream))
    assert rc == 0, L.gpv_noalloc_last_error()
    return l1.cpu().numpy(), pre.cpu().numpy(), bi.cpu().numpy()[: nb.value], nb.value


def test_noalloc_two_calls_match_plain_path(built):
    torch = pytest.importorskip("torch")
    gpv = built
    ctx = gpv.Context(0)
    cases = [W.make(W.C1),
             (lambda t: (t, gpv.grid_padded(*gpv.mesh_bounds(t), (40, 33, 52), 0)))(
                 gpv.gen_torus(9, 96, 48, (0.5, 0.5, 0.5), 0.3, 0.1, 0.01))]
    for tris, spec in cases:  # two calls in a row on the shared scratch
        res = ctx.voxelize_host(tris, spec)
        l1, pre, bi, _ = ctx.fetch(res)
        ctx.release(res)
        a1, apre, abi, nb = _noalloc(gpv, torch, tris, spec)
        assert nb == res.num_boundary
        np.testing.assert_array_equal(a1, l1)
        np.testing.assert_array_equal(apre, pre)
        np.testing.assert_array_equal(abi, bi)
        # and directly against the oracle (the reference's CPU composition)
        ref = orc.Run(tris, spec, fill=orc.FILL_CAND)
        assert nb == ref.B
        np.testing.assert_array_equal(a1, ref.level1_bytes())
        np.testing.assert_array_equal(apre, ref.prefix())
        np.testing.assert_array_equal(abi, ref.boundary_index())
    ctx.close()


def test_noalloc_rejects_bad_level2_divisions(built):
    """A spec gpv_voxelize rejects (Level2 divisions partly zero) is rejected here too."""
    gpv = built
    L = gpv.lib()
    spec = gpv.grid_padded((0, 0, 0), (1, 1, 1), 16, 0)
    spec.ndiv2[:] = (4, 0, 4)
    nb = C.c_int64(-1)
    dummy = C.c_void_p(256)  # never dereferenced: the spec check fails first
    rc = L.gpv_voxelize_level1_noalloc(dummy, 10, C.byref(spec), dummy, dummy, dummy,
                                       C.byref(nb), None)
    assert rc == -1
    assert b"Level2" in L.gpv_noalloc_last_error()


def test_noalloc_rejects_oversize(built):
    gpv = built
    L = gpv.lib()
    spec = gpv.grid_padded((0, 0, 0), (1, 1, 1), 64, 0)
    nb = C.c_int64(-1)
    dummy = C.c_void_p(256)  # never dereferenced: the size check fails first
    rc = L.gpv_voxelize_level1_noalloc(dummy, 10_000_000, C.byref(spec), dummy, dummy, dummy,
                                       C.byref(nb), None)
    assert rc == -1
    assert b"scratch" in L.gpv_noalloc_last_error()


def test_noalloc_refuses_a_capturing_stream(built):
    """A call copies its tables from host memory and waits for its stream, so it cannot be
    recorded into a graph: on a capturing stream it is refused before any work is enqueued, and
    the caller's capture stays usable."""
    torch = pytest.importorskip("torch")
    gpv = built
    L = gpv.lib()
    tris, spec = W.make(W.C1)
    n1 = int(np.prod(list(spec.ndiv)))
    d_tris = torch.from_numpy(np.ascontiguousarray(tris, np.float32)).cuda()
    l1 = torch.empty((n1,), dtype=torch.uint8, device="cuda")
    pre = torch.empty((n1,), dtype=torch.int32, device="cuda")
    bi = torch.empty((n1,), dtype=torch.int32, device="cuda")
    nb = C.c_int64(-1)
    x = torch.zeros(4, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = L.gpv_voxelize_level1_noalloc(C.c_void_p(d_tris.data_ptr()), tris.size // 9, C.byref(spec),
                                           C.c_void_p(l1.data_ptr()), C.c_void_p(pre.data_ptr()),
                                           C.c_void_p(bi.data_ptr()), C.byref(nb),
                                           C.c_void_p(s.cuda_stream))
        x.add_(1.0)  # the capture goes on
    g.replay()
    torch.cuda.synchronize()
    assert rc == -1
    assert b"capturing" in L.gpv_noalloc_last_error()
    assert x.tolist() == [1.0, 1.0, 1.0, 1.0]


def test_noalloc_unaligned_outputs(built):
    """Output buffers off the 4- and 16-byte boundaries (a caller's sub-array) take the per-voxel
    stores of the expansion and give the same outputs."""
    torch = pytest.importorskip("torch")
    gpv = built
    L = gpv.lib()
    tris, spec = W.make(W.C1)
    n1 = int(np.prod(list(spec.ndiv)))
    ref = orc.Run(tris, spec, fill=orc.FILL_CAND)
    d_tris = torch.from_numpy(np.ascontiguousarray(tris, np.float32)).cuda()
    l1 = torch.zeros((n1 + 16,), dtype=torch.uint8, device="cuda")
    pre = torch.zeros((n1 + 4,), dtype=torch.int32, device="cuda")
    bi = torch.zeros((n1 + 4,), dtype=torch.int32, device="cuda")
    nb = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gpv_voxelize_level1_noalloc(C.c_void_p(d_tris.data_ptr()), tris.size // 9, C.byref(spec),
                                       C.c_void_p(l1.data_ptr() + 1), C.c_void_p(pre.data_ptr() + 4),
                                       C.c_void_p(bi.data_ptr() + 4), C.byref(nb), C.c_void_p(stream))
    assert rc == 0, L.gpv_noalloc_last_error()
    torch.cuda.synchronize()
    assert nb.value == ref.B
    np.testing.assert_array_equal(l1.cpu().numpy()[1:1 + n1], ref.level1_bytes())
    np.testing.assert_array_equal(pre.cpu().numpy()[1:1 + n1], ref.prefix())
    np.testing.assert_array_equal(bi.cpu().numpy()[1:1 + nb.value], ref.boundary_index())
