"""Compile the oracle (oracle.cpp) into oracle/_build/liboracle.so with the
same flags as oracle/Makefile: portable, no multiply-add contraction,
OpenMP when the compiler supports it. Test infrastructure only."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "liboracle.so")
SRC = [os.path.join(HERE, "oracle.cpp")]
DEPS = SRC + [os.path.join(HERE, "oracle_math.hpp"), os.path.join(HERE, "oracle_adjoint.inc"),
                                                      os.path.join(HERE, "oracle_spectral.inc"),
                                                      os.path.join(HERE, "oracle_texture.inc")] + [
    os.path.join(ROOT, "include", f) for f in ("wpbr_fmath.h", "wpbr_sampling.h", "wpbr_scene.h", "wpbr_record.h", "wpbr_spectrum_data.h")]
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-I" + os.path.join(ROOT, "include")]


def build_oracle(force=False):
    if not force and os.path.exists(OUT) and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in DEPS):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    tmp = OUT + ".tmp"
    for omp in (["-fopenmp"], []):
        p = subprocess.run([cxx] + FLAGS + omp + SRC + ["-o", tmp], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True)
        if p.returncode == 0:
            os.replace(tmp, OUT)
            return OUT
    raise RuntimeError("oracle build failed:\n" + p.stdout)


if __name__ == "__main__":
    print(build_oracle(force=True))
