"""The reference-named shims (includes/CUDAUtilities.h:63-64, :87-89) driven the way
Object::ClassifyTessellationCUDA / ClassifyInOutTessellationLevel2CUDA drive them."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


class F3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class I3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


def _setup(gpv, L):
    vp = C.c_void_p
    L.CUDAClassifyTessellation.argtypes = [vp, C.c_int, vp, vp, vp, F3, F3, F3, I3, C.c_int]
    L.CUDAClassifyTessellationLevel2.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, I3, F3, F3]
    L.CUDAClassifyInOutLevel2.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int, I3, I3, F3, F3]
    L.THRUSTDeviceFindMax.argtypes = [vp, C.c_int, C.c_int]
    L.THRUSTDeviceFindMax.restype = C.c_float
    L.THRUSTDeviceFindMaxFloat4.argtypes = [vp, C.c_int, vp, C.POINTER(C.c_int)]
    L.THRUSTDeviceFindMaxFloat4.restype = C.c_float
    L.THRUSTDeviceMinMaxSort.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp]


def test_shims_follow_reference(built):
    torch = pytest.importorskip("torch")
    gpv = built
    L = gpv.lib()
    _setup(gpv, L)
    tris = gpv.gen_uvsphere(31, 24, 12, (0.5, 0.5, 0.5), 0.4, 0.002)
    spec = gpv.grid_padded(*gpv.mesh_bounds(tris), 14, 2)
    ref = orc.Run(tris, spec, fill=orc.FILL_VOXEL)
    tab = orc.grid_tables(spec)
    nd = list(spec.ndiv)
    N1 = int(np.prod(nd))
    T = tris.size // 9
    e1 = F3(*[float(v) for v in tab["e1"]])
    e2 = F3(*[float(v) for v in tab["e2"]])
    d_tris = torch.from_numpy(tris).cuda()

    # ---- Level1 (buffer first too small, then retried larger, as PerformVoxelization does)
    st1 = ref.level1_state()
    counts = np.array([len(ref.voxel_tris(v)) for v in range(N1)])
    for buf in (2, int(counts.max())):
        inout = torch.zeros(N1, dtype=torch.float32, device="cuda")
        cnt = torch.zeros(N1, dtype=torch.int32, device="cuda")
        idx = torch.full((N1 * buf,), -1, dtype=torch.int32, device="cuda")
        rc = L.CUDAClassifyTessellation(d_tris.data_ptr(), T, inout.data_ptr(), cnt.data_ptr(),
                                        idx.data_ptr(), F3(*spec.bbox_min), F3(*spec.bbox_max), e1,
                                        I3(*nd), buf)
        torch.cuda.synchronize()
        assert rc == 1
        np.testing.assert_array_equal(inout.cpu().numpy() == 2, st1 == 2)
        np.testing.assert_array_equal(cnt.cpu().numpy(), counts)
        got = idx.cpu().numpy().reshape(N1, buf)
        for v in np.nonzero(counts)[0]:
            lst = set(ref.voxel_tris(v).tolist())
            stored = got[v][: min(counts[v], buf)]
            assert set(stored.tolist()) <= lst and len(set(stored.tolist())) == len(stored)
            if buf >= counts[v]:
                assert set(stored.tolist()) == lst

    # ---- Level2 inputs as the reference host builds them (src/Object.cpp:2146-2180, :2560-2577)
    bidx = ref.boundary_index()
    B = len(bidx)
    n2 = list(spec.ndiv2)
    cells = int(np.prod(n2))
    c1 = tab["c1"]
    cx, cy, cz = c1[:nd[0]], c1[nd[0]:nd[0] + nd[1]], c1[nd[0] + nd[1]:]
    ks, rem = np.divmod(bidx, nd[0] * nd[1])
    js, is_ = np.divmod(rem, nd[0])
    mid = np.stack([cx[is_], cy[js], cz[ks]], 1).astype(np.float32).reshape(-1)
    flat_index = np.zeros(N1, np.int32)
    flat_index[1:] = np.cumsum(counts)[:-1]
    flat = np.concatenate([ref.voxel_tris(v) for v in range(N1)]).astype(np.int32)
    l2 = torch.zeros(B * cells, dtype=torch.float32, device="cuda")
    nrm = torch.zeros(B * cells * 4, dtype=torch.float32, device="cuda")
    tmid = torch.from_numpy(mid).cuda()
    tl2i = torch.from_numpy(bidx.astype(np.int32)).cuda()
    tcnt = torch.from_numpy(counts.astype(np.int32)).cuda()
    tfi = torch.from_numpy(flat_index).cuda()
    tfl = torch.from_numpy(flat).cuda()
    rc = L.CUDAClassifyTessellationLevel2(d_tris.data_ptr(), l2.data_ptr(), nrm.data_ptr(),
                                          tmid.data_ptr(), tl2i.data_ptr(), tcnt.data_ptr(),
                                          tfi.data_ptr(), tfl.data_ptr(), B, I3(*n2), e1, e2)
    assert rc == 1
    st2, _, _ = ref.level2_state()
    np.testing.assert_array_equal(l2.cpu().numpy() == 2, st2 == 2)
    nn = nrm.cpu().numpy().reshape(-1, 4)
    np.testing.assert_array_equal(nn[:, 3], np.where(st2 == 2, nn[:, 3], 0))
    assert (nn[st2 == 2, 3] >= 1).all()

    # ---- CUDAClassifyInOutLevel2 against a CPU evaluation of the same definition:
    # origin (2p+1)*e2 + mid - e1 in float, x/y column list over all z, odd count -> 1
    xy = bidx % (nd[0] * nd[1])
    cols = {}
    for v in range(N1):
        c = v % (nd[0] * nd[1])
        for t in ref.voxel_tris(v):
            cols.setdefault(c, [])
            if t not in cols[c]:
                cols[c].append(int(t))
    xcnt = np.zeros(nd[0] * nd[1], np.int32)
    xidx = np.zeros(nd[0] * nd[1], np.int32)
    xflat = []
    for c in range(nd[0] * nd[1]):
        xidx[c] = len(xflat)
        lst = cols.get(c, [])
        xcnt[c] = len(lst)
        xflat += lst
    l2b = torch.zeros(B * cells, dtype=torch.float32, device="cuda")
    # keep every device buffer referenced until the kernel has run
    txc = torch.from_numpy(xcnt).cuda()
    txi = torch.from_numpy(xidx).cuda()
    txf = torch.from_numpy(np.array(xflat or [0], np.int32)).cuda()
    rc = L.CUDAClassifyInOutLevel2(d_tris.data_ptr(), l2b.data_ptr(), tmid.data_ptr(), tl2i.data_ptr(),
                                   txc.data_ptr(), txi.data_ptr(), txf.data_ptr(),
                                   B, I3(*nd), I3(*n2), e1, e2)
    torch.cuda.synchronize()
    assert rc == 1
    got = l2b.cpu().numpy()
    f32 = np.float32
    exp = np.zeros(B * cells, np.float32)
    for b in range(B):
        m = mid[3 * b:3 * b + 3]
        for c in range(cells):
            r, q, p = c // (n2[0] * n2[1]), (c // n2[0]) % n2[1], c % n2[0]
            o = [f32(f32(f32(2 * s + 1) * f32(e)) + f32(mm)) - f32(h)
                 for s, e, mm, h in zip((p, q, r), tab["e2"], m, tab["e1"])]
            o = np.array(o, np.float32)
            hits = sum(orc.tri_ray_z(tris[9 * t:9 * t + 9], o) for t in cols.get(int(xy[b]), []))
            if hits % 2:
                exp[b * cells + c] = 1.0
    np.testing.assert_array_equal(got, exp)


def _first_max_index(x):
    """thrust::max_element's answer read from the start: the first element stays while nothing
    compares greater (a NaN first element stays; later NaNs never win; -0 == +0)."""
    best = 0
    for i in range(1, len(x)):
        if x[best] < x[i]:
            best = i
    return best


def test_thrust_entry_points(built):
    torch = pytest.importorskip("torch")
    gpv = built
    L = gpv.lib()
    _setup(gpv, L)
    rng = np.random.default_rng(5)
    cases = [rng.normal(size=100003).astype(np.float32),
             np.array([-3.0, 7.0, 7.0, -0.0, 7.0], np.float32),          # ties: first
             np.array([np.nan, 1.0, 5.0], np.float32),                   # NaN first stays
             np.array([1.0, np.nan, 5.0, np.nan], np.float32),           # later NaNs ignored
             np.array([-0.0, 0.0, -1.0], np.float32),                    # -0 == +0
             -np.abs(rng.normal(size=4097)).astype(np.float32)]
    for x in cases:
        d = torch.from_numpy(x).cuda()
        got = L.THRUSTDeviceFindMax(d.data_ptr(), x.size, 1)
        exp = x[_first_max_index(x)]
        assert np.float32(got).view(np.uint32) == exp.view(np.uint32) or (np.isnan(got) and np.isnan(exp))
    assert L.THRUSTDeviceFindMax(d.data_ptr(), 0, 5) == 0.0
    # float4: the element with the largest w, first on ties; x, y, z copied, w = 1
    v4 = rng.normal(size=(5000, 4)).astype(np.float32)
    v4[4000, 3] = v4[:, 3].max() + 1
    v4[4500, 3] = v4[4000, 3]
    d4 = torch.from_numpy(v4).cuda()
    out = (C.c_float * 4)()
    loc = C.c_int(-1)
    w = L.THRUSTDeviceFindMaxFloat4(d4.data_ptr(), 5000, out, C.byref(loc))
    assert loc.value == 4000 and w == v4[4000, 3]
    assert list(out) == [float(v4[4000, 0]), float(v4[4000, 1]), float(v4[4000, 2]), 1.0]
    # rows sorted (non-negative ascending, then negative rows in input order); inputs unchanged
    rows = rng.integers(-5, 1000, 20000).astype(np.int32)
    dr = torch.from_numpy(rows.copy()).cuda()
    dmin = torch.zeros(20000, device="cuda")
    res = np.zeros(20000, np.int32)
    L.THRUSTDeviceMinMaxSort(dmin.data_ptr(), dmin.data_ptr(), dr.data_ptr(), 20000, None, None,
                             res.ctypes.data_as(C.c_void_p))
    exp = np.concatenate([np.sort(rows[rows >= 0], kind="stable"), rows[rows < 0]])
    np.testing.assert_array_equal(res, exp)
    np.testing.assert_array_equal(dr.cpu().numpy(), rows)


def test_level1_shim_on_torus262k(built):
    """CUDAClassifyTessellation on the mid-size configuration through the engine: boundary flags,
    per-voxel counts and stored ids against the oracle's records."""
    torch = pytest.importorskip("torch")
    import workloads as W

    gpv = built
    L = gpv.lib()
    _setup(gpv, L)
    tris, spec = W.make(W.C2)
    ref = orc.Run(tris, spec)
    tab = orc.grid_tables(spec)
    nd = list(spec.ndiv)
    N1 = int(np.prod(nd))
    d_tris = torch.from_numpy(tris).cuda()
    buf = 64
    inout = torch.zeros(N1, dtype=torch.float32, device="cuda")
    cnt = torch.zeros(N1, dtype=torch.int32, device="cuda")
    idx = torch.full((N1 * buf,), -1, dtype=torch.int32, device="cuda")
    rc = L.CUDAClassifyTessellation(d_tris.data_ptr(), tris.size // 9, inout.data_ptr(), cnt.data_ptr(),
                                    idx.data_ptr(), F3(*spec.bbox_min), F3(*spec.bbox_max),
                                    F3(*[float(v) for v in tab["e1"]]), I3(*nd), buf)
    torch.cuda.synchronize()
    assert rc == 1
    st1 = ref.level1_state()
    np.testing.assert_array_equal(inout.cpu().numpy() == 2, st1 == 2)
    c = cnt.cpu().numpy()
    assert c.sum() == ref.num_pairs()
    got = idx.cpu().numpy().reshape(N1, buf)
    rs = np.random.default_rng(0)
    for v in rs.choice(np.nonzero(c)[0], 2000, replace=False):
        lst = np.sort(ref.voxel_tris(v))
        assert c[v] == lst.size
        stored = got[v][:min(c[v], buf)]
        if c[v] <= buf:
            np.testing.assert_array_equal(np.sort(stored), lst)
        else:  # a full buffer holds distinct ids of the voxel's list
            assert set(stored.tolist()) <= set(lst.tolist()) and len(set(stored.tolist())) == buf


def test_reference_caller_runs_on_gpu(built, tmp_path):
    """The C++ caller of tests/test_link.py, linked against libgpview.so, run with its GPU calls."""
    import subprocess

    import test_link as TL

    inc, cudalib = TL._cuda_dirs()
    if not inc or not cudalib:
        pytest.skip("no CUDA toolkit")
    src = tmp_path / "caller.cpp"
    src.write_text(TL.CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.join(TL.ROOT, "gpview_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-I", inc, str(src), "-L", libdir, "-lgpview", "-L",
                        cudalib, "-lcudart", f"-Wl,-rpath,{libdir}:{cudalib}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "run"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "rc=1" in r.stdout and "CUDA Error" not in r.stdout, r.stdout + r.stderr
