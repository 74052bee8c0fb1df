"""Seeded synthetic workloads with the shapes and sizes of the benchmark configurations.

make(cfg) uses the library's generators (gpview_gb300.gen_*); make(cfg, cpu=True) makes the same
mesh and grid bit for bit from the CPU oracle's copy of the same generator source, without loading
the GPU library (the benchmark's reference arm runs that way)."""
import numpy as np


class _LazyGpv:
    """gpview_gb300, imported on first use (a CPU-only caller of make(cfg, cpu=True) never
    imports it)."""

    def __getattr__(self, name):
        import gpview_gb300

        return getattr(gpview_gb300, name)


gpv = _LazyGpv()

# name -> (generator, Level1 divisions, Level2 divisions)
C1 = dict(name="sphere16k", level1=64, level2=4)
C2 = dict(name="torus262k", level1=128, level2=8)
C3 = dict(name="star1310k", level1=256, level2=16)


def sphere16k(seed=1):
    """UV-sphere r=0.4 at the unit-cube centre, 128x64 segments, radial jitter N(0, 0.002)."""
    return gpv.gen_uvsphere(seed, 128, 64, (0.5, 0.5, 0.5), 0.4, 0.002)


def torus262k(seed=2):
    """Torus R=0.35 r=0.12, 512x256 segments, 4-octave value-noise displacement of 0.01."""
    return gpv.gen_torus(seed, 512, 256, (0.5, 0.5, 0.5), 0.35, 0.12, 0.01)


def star1310k(seed=3):
    """Star surface r=0.3(1+0.2 sum a_lm Y_lm), icosphere subdivided 8x, scaled 1:1:6 in z."""
    return gpv.gen_star(seed, 8, (0.5, 0.5, 0.5), 0.3, 0.2, (1.0, 1.0, 6.0))


GENS = {"sphere16k": sphere16k, "torus262k": torus262k, "star1310k": star1310k}
# the same meshes from the oracle library's build of the generator source
CPU_GENS = {"sphere16k": lambda seed=1: _orc().gen_uvsphere(seed, 128, 64, (0.5, 0.5, 0.5), 0.4, 0.002),
            "torus262k": lambda seed=2: _orc().gen_torus(seed, 512, 256, (0.5, 0.5, 0.5), 0.35, 0.12, 0.01),
            "star1310k": lambda seed=3: _orc().gen_star(seed, 8, (0.5, 0.5, 0.5), 0.3, 0.2, (1.0, 1.0, 6.0))}


def _orc():
    from oracle import oracle

    return oracle


def mesh_bounds(tris):
    v = np.asarray(tris, dtype=np.float32).reshape(-1, 3)
    return v.min(axis=0), v.max(axis=0)


def make(cfg, seed=None, cpu=False):
    """(triangles, grid) of a named workload.  cpu=True: generated by the oracle library and the
    grid returned as a (bmin, bmax, ndiv, ndiv2) tuple, with no GPU library loaded."""
    gen = (CPU_GENS if cpu else GENS)[cfg["name"]]
    tris = gen() if seed is None else gen(seed)
    mn, mx = mesh_bounds(tris)
    if cpu:
        return tris, _orc().grid_padded(mn, mx, cfg["level1"], cfg["level2"])
    spec = gpv.grid_padded(mn, mx, cfg["level1"], cfg["level2"])
    return tris, spec


def batch4096(count=4096, seed=4096, threads=None):
    """The batched configuration: `count` closed meshes drawn uniformly from {UV-sphere, noisy
    torus, superellipsoid (e1, e2 ~ U(0.3, 2.0), semi-axes ~ U(0.2, 0.45))}, triangle counts
    log-uniform in [500, 200000], random rotation and placement inside the unit cube; Level1
    uniform over {32, 48, 64, 96, 128}^3 and Level2 uniform over {2, 4, 8}^3 (grid = mesh box
    padded by one cell).  Parameters are drawn in order from one seed; meshes are generated in
    parallel threads (the generators are C++ and release the GIL)."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.default_rng(seed)
    params = []
    for i in range(count):
        fam = int(rng.integers(0, 3))
        T = float(np.exp(rng.uniform(np.log(500), np.log(200000))))
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        p = dict(i=i, fam=fam, q=q.astype(np.float32), gseed=seed * 7919 + i)
        if fam == 0:
            p["nlat"] = max(3, int(round(np.sqrt(T / 4.0))) + 1)
            p["r"] = float(rng.uniform(0.2, 0.45))
            p["c"] = rng.uniform(p["r"], 1.0 - p["r"], 3)
        elif fam == 1:
            p["nv"] = max(3, int(round(np.sqrt(T / 4.0))))
            p["R"] = float(rng.uniform(0.2, 0.33))
            p["rr"] = float(rng.uniform(0.05, min(0.12, p["R"] - 0.02)))
        else:
            p["nlat"] = max(3, int(round(np.sqrt(T / 4.0))) + 1)
            p["semi"] = rng.uniform(0.2, 0.45, 3)
            p["e"] = rng.uniform(0.3, 2.0, 2)
        p["place"] = rng.uniform(0, 1, 3)
        p["n1"] = int(rng.choice([32, 48, 64, 96, 128]))
        p["n2"] = int(rng.choice([2, 4, 8]))
        params.append(p)

    def make_one(p):
        if p["fam"] == 0:
            t = gpv.gen_uvsphere(p["gseed"], 2 * (p["nlat"] - 1), p["nlat"], p["c"], p["r"], 0.002)
        elif p["fam"] == 1:
            t = gpv.gen_torus(p["gseed"], 2 * p["nv"], p["nv"], (0.0, 0.0, 0.0), p["R"], p["rr"], 0.01)
            t = _place(p["place"], t.reshape(-1, 3) @ p["q"].T)
        else:
            t = gpv.gen_superellipsoid(p["gseed"], 2 * (p["nlat"] - 1), p["nlat"], (0.0, 0.0, 0.0),
                                       p["semi"], p["e"][0], p["e"][1], p["q"])
            t = _place(p["place"], t.reshape(-1, 3))
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        return t, gpv.grid_padded(*gpv.mesh_bounds(t), p["n1"], p["n2"])

    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 4) as ex:
        return list(ex.map(make_one, params))


def _place(u, pts):
    """Translates points so their box sits at position u (in [0,1]^3 of the free room) inside the
    unit cube (centred when the box is larger than the cube)."""
    pts = np.asarray(pts, np.float32)
    mn, mx = pts.min(0), pts.max(0)
    size = mx - mn
    lo = np.where(size < 1.0, np.asarray(u) * np.maximum(1.0 - size, 0), 0.5 - size / 2)
    return (pts - mn + lo).astype(np.float32)


def served_pool(count=256, seed=5000, threads=None):
    """Mesh pool of the served configuration: the three families, triangle counts log-uniform
    in [1000, 1000000], Level1 uniform over {64, 128, 256}^3, Level2 uniform over {4, 8}^3."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.default_rng(seed)
    params = []
    for i in range(count):
        fam = int(rng.integers(0, 3))
        T = float(np.exp(rng.uniform(np.log(1000), np.log(1000000))))
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        params.append(dict(fam=fam, T=T, q=q.astype(np.float32), gseed=seed * 7919 + i,
                           semi=rng.uniform(0.2, 0.45, 3), e=rng.uniform(0.3, 2.0, 2),
                           place=rng.uniform(0, 1, 3), r=float(rng.uniform(0.2, 0.45)),
                           R=float(rng.uniform(0.2, 0.33)), rr=float(rng.uniform(0.05, 0.12)),
                           n1=int(rng.choice([64, 128, 256])), n2=int(rng.choice([4, 8]))))

    def make_one(p):
        T = p["T"]
        if p["fam"] == 0:
            nlat = max(3, int(round(np.sqrt(T / 4.0))) + 1)
            t = gpv.gen_uvsphere(p["gseed"], 2 * (nlat - 1), nlat, (0.5, 0.5, 0.5), p["r"], 0.002)
        elif p["fam"] == 1:
            nv = max(3, int(round(np.sqrt(T / 4.0))))
            rr = min(p["rr"], p["R"] - 0.02)
            t = gpv.gen_torus(p["gseed"], 2 * nv, nv, (0.0, 0.0, 0.0), p["R"], rr, 0.01)
            t = _place(p["place"], t.reshape(-1, 3) @ p["q"].T)
        else:
            nlat = max(3, int(round(np.sqrt(T / 4.0))) + 1)
            t = gpv.gen_superellipsoid(p["gseed"], 2 * (nlat - 1), nlat, (0.0, 0.0, 0.0), p["semi"],
                                       p["e"][0], p["e"][1], p["q"])
            t = _place(p["place"], t.reshape(-1, 3))
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        return t, gpv.grid_padded(*gpv.mesh_bounds(t), p["n1"], p["n2"])

    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 4) as ex:
        return list(ex.map(make_one, params))
