"""Compile the oracle (oracle.cpp) into oracle/_build/liboracle.so with the
same flags as oracle/Makefile: portable, no multiply-add contraction,
OpenMP when the compiler supports it. Test infrastructure only.

The library also carries its own copy of the synthetic scene generator
(woodenpbrengine_gb300/csrc/scene_gen.cpp, compiled with the flags the
product library uses for it), so that the CPU baseline and the
`bench.py --impl reference` arm make their inputs without loading the
product library; both copies are built from the one source and give the
same scenes and rays."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")
CSRC = os.path.join(ROOT, "woodenpbrengine_gb300", "csrc")
SCENE_GEN = os.path.join(CSRC, "scene_gen.cpp")
DEPS = [SRC, SCENE_GEN] + [os.path.join(HERE, f) for f in (
    "oracle_math.hpp", "oracle_adjoint.inc", "oracle_spectral.inc", "oracle_texture.inc")] + [
    os.path.join(ROOT, "include", f) for f in ("wpbr_fmath.h", "wpbr_sampling.h", "wpbr_scene.h", "wpbr_record.h",
                                               "wpbr_spectrum_data.h", "wpbr_gpu.h")] + [
    os.path.join(CSRC, f) for f in ("camera.cuh", "geom.cuh", "host_xf.hpp")]
INC = ["-I" + os.path.join(ROOT, "include")]
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"] + INC
# the product library's flags for scene_gen.cpp (woodenpbrengine_gb300/build.py CXX_FLAGS)
SCENE_GEN_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wno-unused-function"] + INC + [
    "-I" + CSRC]


def _run(cmd):
    return subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)


def build_oracle(force=False):
    if not force and os.path.exists(OUT) and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in DEPS):
        return OUT
    bdir = os.path.dirname(OUT)
    os.makedirs(bdir, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    sg = os.path.join(bdir, "scene_gen.o")
    p = _run([cxx] + SCENE_GEN_FLAGS + ["-c", SCENE_GEN, "-o", sg])
    if p.returncode != 0:
        raise RuntimeError("scene generator build failed:\n" + p.stdout)
    tmp = OUT + ".tmp"
    for omp in (["-fopenmp"], []):
        p = _run([cxx] + FLAGS + omp + ["-shared", SRC, sg, "-o", tmp])
        if p.returncode == 0:
            os.replace(tmp, OUT)
            return OUT
    raise RuntimeError("oracle build failed:\n" + p.stdout)


if __name__ == "__main__":
    print(build_oracle(force=True))
