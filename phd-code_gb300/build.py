"""Build the CUDA extension ``libphdflux.so`` in-tree for sm_103a (GB300).

Each translation unit is compiled separately, in parallel, then linked into one
shared library exporting the C ABI of ``include/phdflux.h``:

* ``phd_f64.cu``  FP64 stage kernels and fused step, ``--fmad=false`` so products and
  sums round like the reference's Cython arithmetic;
* ``phd_f32.cu``  FP32 reconstruction / Riemann with FP64 accumulation, fast FP32
  division and square root (``--use_fast_math`` touches FP32 only);
* ``phd_util.cu`` mesh-preparation kernels;
* ``phd_adj.cu``  hand-written adjoint of the FP64 step, ``--fmad=false`` so its
  recomputed forward branches are those of the forward kernels;
* ``phd_frozen.cu`` the FP64 step with its branch decisions recorded / replayed (the
  finite-difference check of the adjoint), ``--fmad=false`` like the forward.

The host tessellation ``phd_tess2d.cpp`` (C ABI of ``include/phdtess.h``) is a plain
C++ library, ``libphdtess.so``, built with the host compiler and
``-ffp-contract=off`` (its robust predicates assume separately rounded products).

Usage: ``python phd-code_gb300/build.py`` (or ``__graft_entry__.build()``).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libphdflux.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]

UNITS = {
    "phd_f64.cu": ["--fmad=false"],
    "phd_f32.cu": ["--use_fast_math"],
    "phd_util.cu": [],
    "phd_adj.cu": ["--fmad=false"],
    "phd_frozen.cu": ["--fmad=false"],
}


TESS_SRC = os.path.join(CSRC, "phd_tess2d.cpp")
TESS_LIB = os.path.join(HERE, "libphdtess.so")


def cxx():
    for c in (os.environ.get("CXX"), "g++", "c++"):
        if c:
            return c
    return "g++"


def build_tess(force=False):
    """Compile the host tessellation library (seconds)."""
    hdr = os.path.join(INCLUDE, "phdtess.h")
    if (not force and os.path.exists(TESS_LIB) and
            os.path.getmtime(TESS_LIB) >= max(os.path.getmtime(TESS_SRC), os.path.getmtime(hdr))):
        return TESS_LIB
    cmd = [cxx(), "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I" + INCLUDE,
           TESS_SRC, "-o", TESS_LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host compile failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(TESS_LIB + ".tmp", TESS_LIB)
    return TESS_LIB


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _sources_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(INCLUDE, "phdflux.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    objs = []

    def compile_one(u):
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        if force or _sources_newer(obj, src):
            cmd = [nvcc()] + ARCH + COMMON + UNITS[u] + list(extra) + ["-c", src, "-o", obj + ".tmp"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (u, " ".join(cmd), r.stderr))
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
            os.replace(obj + ".tmp", obj)
        return obj

    with ThreadPoolExecutor(max_workers=len(units) + 1) as ex:
        tess = ex.submit(build_tess, force)
        objs = list(ex.map(compile_one, units))
        tess.result()
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
