"""Build libwpbr_gpu.so in-tree: nvcc for the CUDA translation units
(sm_103a only), g++ for the host-only ones, linked with the static CUDA
runtime. No CMake; translation units compile in parallel."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libwpbr_gpu.so")

CU_SOURCES = ["context.cu", "bvh_build.cu", "trace.cu", "render.cu", "sort_noalloc.cu", "batch.cu", "adjoint.cu", "spectral.cu"]
CPP_SOURCES = ["scene_gen.cpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction, so device arithmetic is
# bit-identical to the host restatements of the same expressions.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr", "-I" + INC, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
             "-I" + INC, "-I" + CSRC]


def _nvcc():
    cand = [os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found (set NVCC or install the CUDA toolkit)")


def _cuda_include(nvcc):
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def _deps():
    files = []
    for d in (CSRC, INC):
        for f in os.listdir(d):
            files.append(os.path.join(d, f))
    files.append(os.path.abspath(__file__))
    return files


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (p.returncode, " ".join(cmd), p.stdout))
    return p.stdout


def build_library(force=False, verbose=False, extra_nvcc=()):
    """Compile every translation unit and link libwpbr_gpu.so; returns its path."""
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = os.path.join(OUT_DIR, s + ".o")
        objs.append(o)
        jobs.append([nvcc] + NVCC_FLAGS + list(extra_nvcc) + ["-c", os.path.join(CSRC, s), "-o", o])
    for s in CPP_SOURCES:
        o = os.path.join(OUT_DIR, s + ".o")
        objs.append(o)
        jobs.append([cxx] + CXX_FLAGS + ["-I" + _cuda_include(nvcc), "-c", os.path.join(CSRC, s), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lrt", "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


HOST_SRC = os.path.join(PKG, "host", "wpbr_host.cpp")
HOST_BIN = os.path.join(PKG, "wpbr_host")


def build_host(force=False):
    """Compile the C++17 host runner (host/wpbr_host.cpp) against libwpbr_gpu.so."""
    lib = build_library()
    deps = [HOST_SRC, os.path.join(PKG, "host", "scene_io.hpp"), os.path.join(INC, "wpbr_gpu.h"), lib]
    if not force and not _stale(HOST_BIN, deps):
        return HOST_BIN
    cxx = os.environ.get("CXX", "g++")
    tmp = HOST_BIN + ".tmp"
    _run([cxx, "-O2", "-std=c++17", "-Wall", "-I" + INC, HOST_SRC, "-o", tmp, "-L" + PKG, "-lwpbr_gpu",
          "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, HOST_BIN)
    return HOST_BIN


if __name__ == "__main__":
    path = build_library(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(path)
    print(build_host(force="--force" in sys.argv))
