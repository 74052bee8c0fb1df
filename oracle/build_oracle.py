"""Builds the CPU oracle (test infrastructure, never part of the product).

  oracle/liboracle.so          the C restatement (gpv_oracle.c), always built, plus the seeded
                               mesh generators of the workloads (orc_gen_*), compiled from the
                               library's own gpv_meshgen.cpp so that a CPU-only process makes
                               bit-identical inputs without loading the GPU library
  oracle/_ref/liboracle_ref.so the same composition linked against the reference's own
                               TriBoxIntersection.cpp / TriRayIntersection.cpp, built only where
                               the reference sources are present (they are compiled where they
                               lie; nothing is copied into this repository)
  oracle/_ref/libref_pred.so   the reference predicates and its normal arithmetic
                               (includes/FloatVector.h) alone, under C names

Flags: -O2 -ffp-contract=off -fno-fast-math.  Contraction must stay off: a fused multiply-add
changes the predicates' results (GCC fuses by default on aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("GPV_REFERENCE_SRC", "/root/reference/src")
REF_INC = os.path.join(os.path.dirname(REF_SRC), "includes")
FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC"]


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


MESHGEN = os.path.join(os.path.dirname(HERE), "gpview_gb300", "csrc", "gpv_meshgen.cpp")


def build(force=False):
    src = os.path.join(HERE, "gpv_oracle.c")
    out = os.path.join(HERE, "liboracle.so")
    if force or _stale(out, [src, MESHGEN]):
        obj = os.path.join(HERE, "_meshgen.o")
        _run(["g++", *FLAGS, "-std=c++17", "-DGPV_MESHGEN_ORACLE", "-c", MESHGEN, "-o", obj])
        _run(["gcc", *FLAGS, "-fopenmp", "-shared", "-o", out, src, obj, "-lm", "-lstdc++"])
        os.unlink(obj)
    ref_files = [os.path.join(REF_SRC, f) for f in ("TriBoxIntersection.cpp", "TriRayIntersection.cpp")]
    ref_hdr = os.path.join(REF_INC, "FloatVector.h")
    if all(os.path.exists(f) for f in ref_files + [ref_hdr]):
        rdir = os.path.join(HERE, "_ref")
        os.makedirs(rdir, exist_ok=True)
        shim = os.path.join(HERE, "ref_shim.cpp")
        pred = os.path.join(rdir, "libref_pred.so")
        if force or _stale(pred, ref_files + [shim, ref_hdr]):
            _run(["g++", *FLAGS, "-I", REF_INC, "-shared", "-o", pred, shim, *ref_files])
        oref = os.path.join(rdir, "liboracle_ref.so")
        if force or _stale(oref, ref_files + [shim, src, ref_hdr]):
            objs = []
            for f in [src]:
                o = os.path.join(rdir, "gpv_oracle_ref.o")
                _run(["gcc", *FLAGS, "-fopenmp", "-DORC_REF_PREDICATES", "-c", f, "-o", o])
                objs.append(o)
            _run(["g++", *FLAGS, "-I", REF_INC, "-fopenmp", "-shared", "-o", oref, *objs, shim, *ref_files,
                  "-lm"])
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built")
