"""Triangle soups aimed at the decisions the GPU kernels certify with float error bounds.

The kernels skip tests the reference's float arithmetic provably fails, and decide some tests in
groups, using hand-derived bounds:
  * the conservative x/y ray box of the Level1 fill and its ill-conditioning cutoff
    (rel = 4 eps (|e1x e2y| + |e1y e2x|) / |det| <= 1/8);
  * the Level2 plane slab |n.(V0 - c)| <= |n| h + E;
  * the Level2 fill's certified hits and misses around t = 1e-6;
  * the Level2 sub-cell ranges (a cell missing the triangle's box by the rounding margin).
Each family below puts triangles where those bounds are tightest, so that a wrong bound shows up
as a flipped state against the oracle:
  near_threshold_t  -- nearly horizontal triangles whose +z ray test from a Level1 voxel centre
                       or a Level2 ray origin gives t within a few ulps of 1e-6, on both sides
                       (found by stepping the triangle by single ulps, with the reference's float
                       operations evaluated here in the same order);
  slivers           -- long triangles whose x/y projection is nearly degenerate, with rel just
                       below and just above 1/8, and |det| just above the 1e-6 cutoff;
  face_snapped      -- vertices on Level1 / Level2 cell faces (the SAT's box planes) and on the
                       binning's cell boundaries, moved by -3..+3 ulps;
  corner_planes     -- triangles whose plane passes within rounding of a Level2 cell corner (the
                       SAT plane test at its tie), moved by -2..+2 ulps in z;
  edge_corners      -- edges through two Level2 sub-column corners, moved by -2..+2 ulps in x
                       (the x/y edge axes of the z-invariant SAT part at their ties);
  x_parallel        -- edges nearly parallel to x (their ends' y 0..8 ulps apart);
  near_vertical     -- tall faces whose normal has a tiny z component (wide plane slabs);
  degenerate        -- zero-area, collinear and sub-ulp triangles.
The soup is not closed; the outputs are still fully defined by the reference's algorithm, and the
tests compare every byte with the oracle.
"""
import numpy as np

F = np.float32
EPS24 = F(2.0 ** -24)
# smallest float above 1e-6: t > 1e-6 (compared in double by the reference) <=> t >= T_HIT
_f = F(1e-6)
T_HIT = _f if float(_f) > 1e-6 else np.nextafter(_f, F(1))


def ulp_shift(x, k):
    """x moved by k units in the last place (x > 0, float32)."""
    x = np.asarray(x, F)
    return (x.view(np.int32) + np.int32(k)).view(F)


def ray_z(V, O):
    """The reference's triangle_ray_intersection with D = (0, 0, 1), vectorised in float32 with
    the same operation order (src/TriRayIntersection.cpp:78-131).  V: (n, 9), O: (n, 3).
    Returns (inside, t, hit): inside = det and u/v tests pass."""
    V = np.asarray(V, F)
    O = np.asarray(O, F)
    z0 = F(0)
    e1 = V[:, 3:6] - V[:, 0:3]
    e2 = V[:, 6:9] - V[:, 0:3]
    P0 = z0 * e2[:, 2] - F(1) * e2[:, 1]
    P1 = F(1) * e2[:, 0] - z0 * e2[:, 2]
    P2 = z0 * e2[:, 1] - z0 * e2[:, 0]
    det = e1[:, 0] * P0 + e1[:, 1] * P1 + e1[:, 2] * P2
    d64 = det.astype(np.float64)
    ok = ~((d64 > -1e-6) & (d64 < 1e-6))
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = F(1) / det
        T = O - V[:, 0:3]
        u = (T[:, 0] * P0 + T[:, 1] * P1 + T[:, 2] * P2) * inv
        Q0 = T[:, 1] * e1[:, 2] - T[:, 2] * e1[:, 1]
        Q1 = T[:, 2] * e1[:, 0] - T[:, 0] * e1[:, 2]
        Q2 = T[:, 0] * e1[:, 1] - T[:, 1] * e1[:, 0]
        v = (z0 * Q0 + z0 * Q1 + F(1) * Q2) * inv
        t = (e2[:, 0] * Q0 + e2[:, 1] * Q1 + e2[:, 2] * Q2) * inv
        inside = ok & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1)
    return inside, t, inside & (t.astype(np.float64) > 1e-6)


def sliver_rel(V):
    """The Level1 ray box's conditioning figure rel = 4 eps sd / |det| in float32, as the prep
    kernel evaluates it, and |det|."""
    V = np.asarray(V, F)
    e1x, e1y = V[:, 3] - V[:, 0], V[:, 4] - V[:, 1]
    e2x, e2y = V[:, 6] - V[:, 0], V[:, 7] - V[:, 1]
    det = e1x * (-e2y) + e1y * e2x
    sd = np.abs(e1x * e2y) + np.abs(e1y * e2x)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = F(4) * EPS24 * sd / np.abs(det)
    return rel, np.abs(det)


def _tables(tab, n, n2):
    c1 = tab["c1"]
    cx, cy, cz = c1[:n[0]], c1[n[0]:n[0] + n[1]], c1[n[0] + n[1]:]
    o2 = tab["o2"]
    ox, oy, oz = o2[:n[0] * n2[0]], o2[n[0] * n2[0]:n[0] * n2[0] + n[1] * n2[1]], \
        o2[n[0] * n2[0] + n[1] * n2[1]:]
    c2 = tab["c2s"]
    sx, sy, sz = c2[:n[0] * n2[0]], c2[n[0] * n2[0]:n[0] * n2[0] + n[1] * n2[1]], \
        c2[n[0] * n2[0] + n[1] * n2[1]:]
    return (cx, cy, cz), (ox, oy, oz), (sx, sy, sz)


def near_threshold_t(rng, origins, cell, keep=4):
    """For each origin (ox, oy, oz): a small, slightly sloped triangle around (ox, oy) at height
    ~oz + 1e-6, stepped by single ulps in x (coarse: slope 1e-3) and then in y (fine: slope
    1e-5) until the reference's float t straddles 1e-6; the `keep` steps whose t is closest to
    the threshold are kept (hits and misses)."""
    out = []
    for o in origins:
        o = np.asarray(o, np.float64)
        ang = rng.uniform(0, 2 * np.pi) + np.array([0.0, 2 * np.pi / 3, 4 * np.pi / 3])
        r = 0.3 * cell * rng.uniform(0.6, 1.0)
        a, b = r * np.cos(ang), r * np.sin(ang)
        sx = rng.choice([-1.0, 1.0]) * 1e-3
        sy = rng.choice([-1.0, 1.0]) * 1e-5
        z = o[2] + 1e-6 + sx * a + sy * b
        base = np.stack([o[0] + a, o[1] + b, z], 1).astype(F).reshape(9)
        O = o.astype(F)[None, :]

        def stepped(kx, ky):
            """The base triangle with every vertex's x moved by kx ulps and y by ky ulps."""
            V = np.repeat(base[None, :], len(kx), 0)
            for vtx in range(3):
                V[:, 3 * vtx] = ulp_shift(np.full(len(kx), base[3 * vtx], F), kx.astype(np.int32))
                V[:, 3 * vtx + 1] = ulp_shift(np.full(len(ky), base[3 * vtx + 1], F), ky.astype(np.int32))
            return V

        if not (base[0::3] > 0).all() or not (base[1::3] > 0).all():
            continue
        kx = np.arange(-1500, 1501)
        V = stepped(kx, np.zeros_like(kx))
        ins, t, _ = ray_z(V, np.repeat(O, len(kx), 0))
        err = np.where(ins, np.abs(t.astype(np.float64) - 1e-6), np.inf)
        if not np.isfinite(err).any():
            continue
        bx = kx[int(np.argmin(err))]
        ky = np.arange(-1500, 1501)
        V = np.concatenate([V, stepped(np.full_like(ky, bx), ky)])
        ins, t, hit = ray_z(V, np.repeat(O, len(V), 0))
        err = np.abs(t.astype(np.float64) - 1e-6)
        # the closest hits and the closest misses (t just above and at or below 1e-6)
        for sel in (ins & hit, ins & ~hit):
            idx = np.nonzero(sel)[0]
            out.extend(V[i] for i in idx[np.argsort(err[idx])[:keep // 2]])
    return np.array(out, F).reshape(-1, 9)


def slivers(rng, bmin, bmax, count):
    """Long triangles with a nearly degenerate x/y projection: rel around the 1/8 cutoff (both
    sides) and |det| just above the 1e-6 cutoff."""
    bmin = np.asarray(bmin, np.float64)
    bmax = np.asarray(bmax, np.float64)
    span = bmax - bmin
    out = []
    tries = 0
    while len(out) < count and tries < 200000:
        tries += 1
        th = rng.uniform(np.pi / 4 - 0.3, np.pi / 4 + 0.3) + rng.choice([0, np.pi / 2])
        d = np.array([np.cos(th), np.sin(th)])
        perp = np.array([-d[1], d[0]])
        L = rng.uniform(0.75, 0.95) * min(span[0], span[1]) * np.sqrt(2)
        lam = rng.uniform(0.4, 0.9)
        # det ~ L delta and sd ~ 2 lam L^2 |dx dy|: pick delta for a target rel around 1/8
        target = np.exp(rng.uniform(np.log(0.105), np.log(0.15)))
        delta = 8 * float(EPS24) * lam * L * abs(d[0] * d[1]) / target
        c = bmin[:2] + span[:2] / 2
        p0 = c - 0.5 * L * d + rng.normal(0, 0.02, 2) * span[:2]
        zs = bmin[2] + span[2] * rng.uniform(0.1, 0.9, 3)
        V = np.array([[p0[0], p0[1], zs[0]],
                      [*(p0 + L * d), zs[1]],
                      [*(p0 + lam * L * d + delta * perp), zs[2]]])
        if (V[:, :2] <= bmin[:2]).any() or (V[:, :2] >= bmax[:2]).any():
            continue
        V = V.astype(F).reshape(1, 9)
        rel, adet = sliver_rel(V)
        if adet[0] <= 1e-6:
            continue
        # keep the band around the cutoff densely, and a few further away
        if 0.1 <= rel[0] <= 0.16 or (len(out) % 5 == 0 and 0.05 <= rel[0] <= 0.3):
            out.append(V[0])
    return np.array(out, F).reshape(-1, 9)


def face_snapped(rng, faces, cell, count):
    """Small random triangles whose vertex coordinates are, per axis, either free or on one of
    the given face coordinates (per axis arrays), moved by -3..+3 ulps."""
    out = []
    for _ in range(count):
        base = np.array([rng.choice(faces[a]) for a in range(3)], np.float64)
        V = base[None, :] + rng.uniform(-1.2, 1.2, (3, 3)) * cell
        V = V.astype(F)
        for vtx in range(3):
            for a in range(3):
                if rng.random() < 0.6:
                    f = F(rng.choice(faces[a]))
                    if f > 0:
                        V[vtx, a] = ulp_shift(f, int(rng.integers(-3, 4)))
        out.append(V.reshape(9))
    return np.array(out, F).reshape(-1, 9)


def corner_planes(rng, centres, half, count):
    """Triangles whose plane passes within rounding of a Level2 cell corner, each repeated with
    its vertices moved by -2..+2 ulps in z."""
    out = []
    for _ in range(count):
        c = np.array([rng.choice(centres[a]) for a in range(3)], np.float64)
        s = rng.choice([-1.0, 1.0], 3)
        corner = (c.astype(F) + (s * half).astype(F)).astype(np.float64)
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        u = np.cross(n, [1.0, 0.0, 0.0] if abs(n[0]) < 0.9 else [0.0, 1.0, 0.0])
        u /= np.linalg.norm(u)
        w = np.cross(n, u)
        sc = float(np.max(half)) * rng.uniform(1.0, 4.0)
        V = np.stack([corner - 0.3 * sc * u - 0.2 * sc * w, corner + 0.5 * sc * u,
                      corner + 0.4 * sc * w]).astype(F)
        if (V <= 0).any():
            continue
        for k in (-2, -1, 0, 1, 2):
            W = V.copy()
            W[:, 2] = ulp_shift(W[:, 2], k)
            out.append(W.reshape(9))
    return np.array(out, F).reshape(-1, 9)


def edge_corners(rng, centres, half, zrange, count):
    """Triangles with an edge through two Level2 sub-column corners (the x/y edge-axis test of
    the SAT at its tie, decided once per sub-column by the Level2 kernel), each repeated with
    the edge's ends moved by -2..+2 ulps in x."""
    sx, sy = centres
    out = []
    for _ in range(count):
        a = np.array([F(rng.choice(sx)) + F(half[0]) * F(rng.choice([-1.0, 1.0])),
                      F(rng.choice(sy)) + F(half[1]) * F(rng.choice([-1.0, 1.0]))], F)
        # the other end a few sub-columns away (or far away, for long edges)
        reach = float(half[0]) * 2 * rng.choice([1, 2, 3, 7, 40])
        b = (a.astype(np.float64) + reach * rng.choice([-1.0, 1.0], 2) *
             np.array([rng.integers(0, 4), rng.integers(1, 4)])).astype(F)
        b = (np.round((b.astype(np.float64) - a) / (2 * np.asarray(half[:2], np.float64))) *
             (2 * np.asarray(half[:2], np.float64)) + a).astype(F)
        c = (a.astype(np.float64) + rng.normal(size=2) * reach).astype(F)
        z = rng.uniform(zrange[0], zrange[1], 3).astype(F)
        if (a == b).all():
            continue
        V = np.array([[a[0], a[1], z[0]], [b[0], b[1], z[1]], [c[0], c[1], z[2]]], F)
        if (V <= 0).any():
            continue
        for k in (-2, -1, 0, 1, 2):
            W = V.copy()
            W[:2, 0] = ulp_shift(W[:2, 0], k)
            out.append(W.reshape(9))
    return np.array(out, F).reshape(-1, 9)


def x_parallel(rng, bmin, bmax, count):
    """Triangles with an edge nearly parallel to x: its ends' y differ by 0..8 ulps, so its
    x/y edge axis is ill-conditioned (the float test is decided by rounding)."""
    bmin = np.asarray(bmin, np.float64)
    span = np.asarray(bmax, np.float64) - bmin
    out = []
    for k in range(count):
        p = (bmin + span * rng.uniform(0.2, 0.8, 3)).astype(F)
        q = (bmin + span * rng.uniform(0.2, 0.8, 3)).astype(F)
        if p[1] <= 0:
            continue
        q[1] = ulp_shift(np.array([p[1]], F), int(k % 9))[0]
        r = (bmin + span * rng.uniform(0.2, 0.8, 3)).astype(F)
        out.append(np.stack([p, q, r]).astype(F).reshape(9))
    return np.array(out, F).reshape(-1, 9)


def near_vertical(rng, bmin, bmax, count):
    """Tall faces whose normal's z component is tiny (1e-7 .. 1e-3 of its length)."""
    bmin = np.asarray(bmin, np.float64)
    span = np.asarray(bmax, np.float64) - bmin
    out = []
    for _ in range(count):
        th = rng.uniform(0, 2 * np.pi)
        d = np.array([np.cos(th), np.sin(th), 0.0])
        tilt = np.exp(rng.uniform(np.log(1e-7), np.log(1e-3)))
        up = np.array([0.0, 0.0, 1.0]) + tilt * np.array([-d[1], d[0], 0.0])
        p = bmin + span * rng.uniform(0.2, 0.8, 3)
        p[2] = bmin[2] + span[2] * rng.uniform(0.05, 0.3)
        h = span[2] * rng.uniform(0.3, 0.6)
        wdt = span[0] * rng.uniform(0.05, 0.3)
        V = np.stack([p, p + wdt * d, p + 0.5 * wdt * d + h * up]).astype(F)
        out.append(V.reshape(9))
    return np.array(out, F).reshape(-1, 9)


def degenerate(rng, bmin, bmax, count):
    """Zero-area (repeated vertex), collinear and sub-ulp triangles."""
    bmin = np.asarray(bmin, np.float64)
    span = np.asarray(bmax, np.float64) - bmin
    out = []
    for k in range(count):
        p = (bmin + span * rng.uniform(0.2, 0.8, 3)).astype(F)
        q = (bmin + span * rng.uniform(0.2, 0.8, 3)).astype(F)
        kind = k % 3
        if kind == 0:
            V = np.stack([p, p, q])
        elif kind == 1:
            V = np.stack([p, q, ((p.astype(np.float64) + q) / 2).astype(F)])
        else:
            V = np.stack([p, ulp_shift(p, 1), ulp_shift(p, np.array([0, 1, 2], np.int32))])
        out.append(V.astype(F).reshape(9))
    return np.array(out, F).reshape(-1, 9)


def soup(spec_tuple, tab, seed=0, scale=1.0):
    """The adversarial triangle soup for one grid.  spec_tuple = (bmin, bmax, n, n2); tab =
    oracle.grid_tables of the same grid.  Returns float32[T*9]."""
    bmin, bmax, n, n2 = spec_tuple
    n = [int(v) for v in n]
    n2 = [int(v) for v in n2]
    rng = np.random.default_rng(seed)
    (cx, cy, cz), (ox, oy, oz), (sx, sy, sz) = _tables(tab, n, n2)
    g = np.asarray(tab["g"], np.float64)
    e1 = np.asarray(tab["e1"], F)
    e2 = np.asarray(tab["e2"], F)
    cell = float(g.min())
    k = lambda c: max(1, int(c * scale))  # noqa: E731
    # Level1 voxel centres and Level2 ray origins as targets of the t ~ 1e-6 family
    t1 = [(cx[rng.integers(1, n[0] - 1)], cy[rng.integers(1, n[1] - 1)], cz[rng.integers(1, n[2] - 1)])
          for _ in range(k(40))]
    t2 = [(ox[rng.integers(n2[0], (n[0] - 1) * n2[0])], oy[rng.integers(n2[1], (n[1] - 1) * n2[1])],
           oz[rng.integers(n2[2], (n[2] - 1) * n2[2])]) for _ in range(k(60))]
    parts = [near_threshold_t(rng, t1, cell), near_threshold_t(rng, t2, cell / max(n2))]
    parts.append(slivers(rng, bmin, bmax, k(40)))
    # faces: Level1 box planes (centre +- half), Level2 box planes, binning cell boundaries
    f1 = [np.concatenate([c - h, c + h]).astype(F) for c, h in zip((cx, cy, cz), e1)]
    f2 = [np.concatenate([c - h, c + h]).astype(F) for c, h in zip((sx, sy, sz), e2)]
    fb = [(F(lo) + (F(hi) - F(lo)) * (np.arange(1, m, dtype=F) / F(m))).astype(F)
          for lo, hi, m in zip(bmin, bmax, n)]
    parts.append(face_snapped(rng, f1, cell, k(120)))
    parts.append(face_snapped(rng, f2, cell / max(n2), k(160)))
    parts.append(face_snapped(rng, fb, cell, k(80)))
    parts.append(corner_planes(rng, (sx, sy, sz), np.asarray(e2, np.float64), k(50)))
    zr = (bmin[2] + 0.1 * (bmax[2] - bmin[2]), bmax[2] - 0.1 * (bmax[2] - bmin[2]))
    parts.append(edge_corners(rng, (sx, sy), np.asarray(e2, np.float64), zr, k(40)))
    parts.append(x_parallel(rng, bmin, bmax, k(30)))
    parts.append(near_vertical(rng, bmin, bmax, k(60)))
    parts.append(degenerate(rng, bmin, bmax, k(24)))
    tris = np.concatenate([p.reshape(-1, 9) for p in parts if p.size]).astype(F)
    perm = rng.permutation(len(tris))
    return np.ascontiguousarray(tris[perm].reshape(-1))


# Grids of the adversarial cases: (bmin, bmax, n, n2); non-uniform divisions and every Level2
# size the queued and per-lane kernel organisations handle differently.
GRIDS = [
    ((-0.05, -0.1, 0.02), (1.15, 1.1, 1.3), (20, 24, 18), (4, 4, 4)),
    ((0.0, 0.0, 0.0), (1.2, 1.2, 1.2), (16, 16, 16), (8, 8, 8)),
    ((0.1, -0.05, 0.0), (1.3, 1.15, 1.0), (12, 10, 14), (16, 16, 16)),
    ((0.0, 0.05, -0.1), (1.2, 1.25, 1.1), (14, 18, 11), (3, 5, 2)),
]
