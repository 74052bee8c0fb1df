"""Seeded synthetic workloads with the shapes and sizes of the benchmark configurations."""
import numpy as np

import gpview_gb300 as gpv

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


def make(cfg, seed=None):
    gen = GENS[cfg["name"]]
    tris = gen() if seed is None else gen(seed)
    mn, mx = gpv.mesh_bounds(tris)
    spec = gpv.grid_padded(mn, mx, cfg["level1"], cfg["level2"])
    return tris, spec
