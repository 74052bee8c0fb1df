"""gpv_voxelize_to_host: host outputs equal the plain path's (and the oracle's) whether the Level2
kernel writes a pinned buffer directly (slabs = 0) or each z slab is copied while later slabs
compute (any slab count, or a pageable buffer); a Level2 buffer that is too small is reported,
not overrun."""
import numpy as np
import pytest

from oracle import oracle as orc
import workloads as W

pytestmark = pytest.mark.gpu


def _to_host(ctx, tris, spec, slabs, l2_bytes=None):
    import torch

    n1 = int(np.prod(list(spec.ndiv)))
    cells = int(np.prod(list(spec.ndiv2))) if spec.ndiv2[0] else 0
    ref = ctx.voxelize_host(tris, spec)  # sizes
    B = ref.num_boundary
    ctx.release(ref)
    h_tris = torch.from_numpy(tris).pin_memory()
    l1 = torch.empty(n1, dtype=torch.uint8).pin_memory()
    pre = torch.empty(n1, dtype=torch.int32).pin_memory()
    bi = torch.empty(max(B, 1), dtype=torch.int32).pin_memory()
    need = B * cells
    l2 = torch.full((max(need, 1),), 77, dtype=torch.uint8).pin_memory()
    rc, res = ctx.voxelize_to_host(h_tris.data_ptr(), tris.size // 9, spec, l1.data_ptr(),
                                   pre.data_ptr(), bi.data_ptr(), l2.data_ptr(),
                                   need if l2_bytes is None else l2_bytes, slabs)
    return rc, res, l1.numpy().copy(), pre.numpy().copy(), bi.numpy()[:B].copy(), l2.numpy()[:need].copy()


@pytest.mark.parametrize("slabs", [0, 1, 3, 4, 8])
def test_to_host_equals_oracle_sphere16k(ctx, slabs):
    tris, spec = W.make(W.C1)
    rc, res, l1, pre, bi, l2 = _to_host(ctx, tris, spec, slabs)
    assert rc == 0
    ref = orc.Run(tris, spec)
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(pre, ref.prefix())
    np.testing.assert_array_equal(bi, ref.boundary_index())
    np.testing.assert_array_equal(l2, ref.level2_bytes())
    # the returned device result matches too
    d1, dpre, dbi, dl2 = ctx.fetch(res)
    np.testing.assert_array_equal(dl2, l2)
    ctx.release(res)


@pytest.mark.parametrize("slabs", [0, 4])
def test_to_host_equals_plain_torus262k(ctx, slabs):
    tris, spec = W.make(W.C2)
    rc, res, l1, pre, bi, l2 = _to_host(ctx, tris, spec, slabs)
    assert rc == 0
    ctx.release(res)
    plain = ctx.voxelize_host(tris, spec)
    p1, ppre, pbi, pl2 = ctx.fetch(plain)
    ctx.release(plain)
    np.testing.assert_array_equal(l1, p1)
    np.testing.assert_array_equal(pre, ppre)
    np.testing.assert_array_equal(bi, pbi)
    np.testing.assert_array_equal(l2, pl2)


@pytest.mark.parametrize("slabs", [0, 4])
def test_to_host_small_buffer_is_reported(ctx, slabs):
    tris, spec = W.make(W.C1)
    rc, res, l1, pre, bi, l2 = _to_host(ctx, tris, spec, slabs, l2_bytes=100)
    assert rc == -7  # GPV_ERR_BUDGET: nothing copied to the Level2 buffer
    assert (l2 == 77).all()
    ref = orc.Run(tris, spec)
    np.testing.assert_array_equal(l1, ref.level1_bytes())  # Level1 outputs still delivered
    ctx.release(res)


def test_to_host_pageable_buffers(ctx):
    """Pageable host buffers: the Level2 bytes come through the slab copies."""
    tris, spec = W.make(W.C1)
    ref = orc.Run(tris, spec)
    cells = int(np.prod(list(spec.ndiv2)))
    n1 = int(np.prod(list(spec.ndiv)))
    l1 = np.zeros(n1, np.uint8)
    pre = np.zeros(n1, np.int32)
    bi = np.zeros(ref.B, np.int32)
    l2 = np.zeros(ref.B * cells, np.uint8)
    rc, res = ctx.voxelize_to_host(tris.ctypes.data, tris.size // 9, spec, l1.ctypes.data,
                                   pre.ctypes.data, bi.ctypes.data, l2.ctypes.data, l2.size, 0)
    assert rc == 0
    np.testing.assert_array_equal(l1, ref.level1_bytes())
    np.testing.assert_array_equal(pre, ref.prefix())
    np.testing.assert_array_equal(bi, ref.boundary_index())
    np.testing.assert_array_equal(l2, ref.level2_bytes())
    ctx.release(res)


def test_pinned_triangles_read_in_place(ctx):
    """gpv_voxelize_host on page-locked triangles (read by the kernels in place) equals the
    pageable path."""
    import ctypes as C

    import torch
    import gpview_gb300 as gpv

    tris, spec = W.make(W.C1)
    h = torch.from_numpy(tris).pin_memory()
    res = gpv.Result()
    rc = gpv.lib().gpv_voxelize_host(ctx._h, C.c_void_p(h.data_ptr()), tris.size // 9,
                                     C.byref(spec), C.byref(res), C.c_void_p(0))
    assert rc == 0
    a = ctx.fetch(res)
    ctx.release(res)
    ref = ctx.voxelize_host(tris, spec)
    b = ctx.fetch(ref)
    ctx.release(ref)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_to_host_level1_only(ctx):
    import gpview_gb300 as gpv

    tris = gpv.gen_uvsphere(51, 32, 16, (0.5, 0.5, 0.5), 0.4, 0.002)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), 24, 0)
    rc, res, l1, pre, bi, l2 = _to_host(ctx, tris, spec, 4)
    assert rc == 0
    np.testing.assert_array_equal(l1, orc.Run(tris, spec).level1_bytes())
    ctx.release(res)


@pytest.mark.parametrize("mask,share", [(0xff, 100), (0x0f, 100), (0x55, 100), (0x80, 100),
                                        (0xff, 50), (0xff, 1), (0x3c, 37)])
def test_packed_transfer_equals_plain_torus262k(ctx, mask, share):
    """The packed Level2 transfer (2-bit codes expanded by host threads) gives the bytes the
    kernel writes directly, whichever slabs and whichever share of their voxels send codes; the
    size threshold is lowered so that this 56 MB output takes it."""
    tris, spec = W.make(W.C2)
    plain = ctx.voxelize_host(tris, spec)
    p = ctx.fetch(plain)
    ctx.release(plain)
    ctx.set_host_expand(-1, mask, share=share, min_level2_bytes=0)
    try:
        rc, res, l1, pre, bi, l2 = _to_host(ctx, tris, spec, 0)
    finally:
        ctx.set_host_expand()
    assert rc == 0
    for a, b in zip((l1, pre, bi, l2), p):
        np.testing.assert_array_equal(a, b)
    assert res.num_level2_inside == int((l2 == 127).sum())
    ctx.release(res)


def test_packed_transfer_star1310k_and_threads(ctx):
    """The largest plain configuration through the default packed transfer, then with 3 host
    threads and part of the slabs, then with it off: identical bytes each time, equal to the
    device result."""
    tris, spec = W.make(W.C3)
    plain = ctx.voxelize_host(tris, spec)
    p = ctx.fetch(plain)
    ctx.release(plain)
    try:
        for threads, mask, share in ((-1, 0xff, 100), (3, 0x3f, 60), (-1, 0xff, 50), (0, 0xff, 100)):
            ctx.set_host_expand(threads, mask, share=share)
            rc, res, l1, pre, bi, l2 = _to_host(ctx, tris, spec, 0)
            assert rc == 0
            ctx.release(res)
            for a, b in zip((l1, pre, bi, l2), p):
                np.testing.assert_array_equal(a, b)
    finally:
        ctx.set_host_expand()
