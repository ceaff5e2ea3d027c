"""Build recipe for the reference's own Cython hot path (test infrastructure only).

This compiles the unmodified algorithmic code of rickyfernandez/phd-code's flux path
(``phd/reconstruction``, ``phd/riemann``, ``phd/mesh/mesh.pyx``, ``phd/equation_state``,
``phd/domain``, ``phd/hilbert`` and the containers they sit on) under Python 3 so that
the C restatement in ``oracle/phd_oracle.c`` can be pinned against the reference
itself and golden vectors can be generated.  Nothing here is shipped or imported by
the product path.

Everything is written under ``oracle/_ref/`` (git-ignored):

* ``oracle/_ref/build/phd/...``  sources staged from the read-only reference tree with
  the Python-3 compatibility edits listed in ``PY3_EDITS`` (dict views; these touch
  container bookkeeping only, never arithmetic),
* a ``phd/__init__.py`` stand-in declaring a serial run (the real one imports h5py,
  matplotlib and the gravity package, ``phd/__init__.py:1-123``),
* a ``mpi4py`` stand-in (``load_balance.pyx:3`` and ``tree.pyx:2`` import it at module
  init; the serial path never calls it),
* ``tess_stub.cpp``: the ``Tess2d``/``Tess3d`` members declared in ``phd/mesh/tess.h``
  returning -1 (CGAL is not installed; the face list is produced by our own host mesh
  builder and handed to the reference directly),
* ``phd/mesh/refhelper.pyx``: a tiny module that fills the C++ ``Mesh.neighbors``
  attribute (``mesh.pxd:34``), reachable only from Cython that cimports ``Mesh``.

Cython directives: ``language_level=2`` (the reference is Python 2 code),
``cpow=True`` (so ``range(3**dim)`` stays an int, ``boundary.pyx:378``) and
``legacy_implicit_noexcept=True`` (``tree.pyx:606``).

Usage:  python oracle/build_ref.py [--reference DIR] [--jobs 8]
        (DIR defaults to $PHD_REFERENCE_DIR, else /root/reference)
        python oracle/build_ref.py --compile-staged   (compile the staged C++ on this machine)
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
import textwrap

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REFERENCE = "/root/reference"
OUT = os.path.join(HERE, "_ref")
BUILD = os.path.join(OUT, "build")

# Cython modules (package path, extra C++ sources relative to the staged tree).
MODULES = [
    ("phd/utils/carray", []),
    ("phd/containers/containers", []),
    ("phd/utils/particle_creator", []),
    ("phd/equation_state/equation_state", []),
    ("phd/hilbert/hilbert", []),
    ("phd/load_balance/tree", []),
    ("phd/load_balance/load_balance", []),
    ("phd/domain/domain_manager", ["phd/domain/particle.cpp"]),
    ("phd/domain/boundary", ["phd/domain/particle.cpp"]),
    ("phd/mesh/pytess", ["tess_stub.cpp"]),
    ("phd/mesh/mesh", ["tess_stub.cpp"]),
    ("phd/riemann/riemann", []),
    ("phd/reconstruction/reconstruction", []),
    ("phd/mesh/refhelper", []),
]

# Files staged verbatim apart from PY3_EDITS (directories relative to phd/).
STAGE = {
    "utils": ["carray.pyx", "carray.pxd", "particle_creator.pyx", "particle_tags.py",
              "tools.py", "exchange_particles.py", "__init__.py"],
    "containers": ["containers.pyx", "containers.pxd", "__init__.py"],
    "equation_state": ["equation_state.pyx", "equation_state.pxd", "__init__.py"],
    "hilbert": ["hilbert.pyx", "hilbert.pxd", "__init__.py"],
    "load_balance": ["tree.pyx", "tree.pxd", "load_balance.pyx", "load_balance.pxd",
                     "__init__.py"],
    "domain": ["domain_manager.pyx", "domain_manager.pxd", "boundary.pyx", "boundary.pxd",
               "particle.cpp", "particle.h", "__init__.py"],
    "mesh": ["mesh.pyx", "mesh.pxd", "pytess.pyx", "pytess.pxd", "tess.h", "__init__.py"],
    "riemann": ["riemann.pyx", "riemann.pxd", "__init__.py"],
    "reconstruction": ["reconstruction.pyx", "reconstruction.pxd", "__init__.py"],
    # the integrator, for the drop-in test that installs plugin subclasses through its
    # check_class setters (integrate.py:148-161) and steps StaticMeshMUSCLHancock
    "integrate": ["integrate.py", "__init__.py"],
}

# Python-3 edits: (file, regex, replacement).  Container bookkeeping only.
PY3_EDITS = [
    ("containers/containers.pyx", r"self\.carrays\.values\(\)\[0\]",
     "list(self.carrays.values())[0]"),
    ("containers/containers.pyx", r"carray_list_names = self\.carrays\.keys\(\)",
     "carray_list_names = list(self.carrays.keys())"),
    ("containers/containers.pyx", r"carray_list = self\.carrays\.values\(\)",
     "carray_list = list(self.carrays.values())"),
    ("mesh/mesh.pyx", r"\.iteritems\(\)", ".items()"),
    ("domain/domain_manager.pyx", r"\.iteritems\(\)", ".items()"),
    ("utils/tools.py", r"\.iteritems\(\)", ".items()"),
]

PHD_INIT = '''\
"""Serial-run stand-in for the reference's package init (build artefact)."""
_in_parallel = False
_rank = 0
_size = 1
_comm = None
'''

MPI_STUB = '''\
"""Stand-in for mpi4py: the reference's serial path never calls MPI."""
class _Op(object):
    pass
class MPI(object):
    COMM_WORLD = None
    INT = DOUBLE = LONG = SUM = MIN = MAX = _Op()
'''

TESS_STUB = r'''
// Stand-in for the CGAL-backed tessellation (tess.cpp / tess3.cpp): every entry
// point reports failure.  The face list is supplied directly to the reference.
#include "phd/mesh/tess.h"
Tess2d::Tess2d(void) { ptess = 0; pvt_list = 0; }
void Tess2d::reset_tess(void) {}
int Tess2d::build_initial_tess(double *x[3], double *r, int n) { return -1; }
int Tess2d::update_initial_tess(double *x[3], int b, int e) { return -1; }
int Tess2d::count_number_of_faces(void) { return -1; }
int Tess2d::extract_geometry(double* x[3], double* d[3], double* v, double* a,
        double* c[3], double* n[3], int* pi, int* pj,
        std::vector< std::vector<int> > &nb) { return -1; }
int Tess2d::update_radius(double *x[3], double *r, std::list<FlagParticle> &f) { return -1; }
int Tess2d::reindex_ghost(std::vector<GhostID> &g) { return -1; }
Tess3d::Tess3d(void) { ptess = 0; pvt_list = 0; }
void Tess3d::reset_tess(void) {}
int Tess3d::build_initial_tess(double *x[3], double *r, int n) { return -1; }
int Tess3d::update_initial_tess(double *x[3], int b, int e) { return -1; }
int Tess3d::count_number_of_faces(void) { return -1; }
int Tess3d::extract_geometry(double* x[3], double* d[3], double* v, double* a,
        double* c[3], double* n[3], int* pi, int* pj,
        std::vector< std::vector<int> > &nb) { return -1; }
int Tess3d::update_radius(double *x[3], double *r, std::list<FlagParticle> &f) { return -1; }
int Tess3d::reindex_ghost(std::vector<GhostID> &g) { return -1; }
'''

REFHELPER = '''\
# distutils: language = c++
"""Fill the reference Mesh's C++ neighbour lists (mesh.pxd:34) from Python."""
from phd.mesh.mesh cimport Mesh

def set_neighbors(Mesh mesh, object ptr, object idx):
    cdef int n = len(ptr) - 1
    cdef int i, k
    mesh.neighbors.resize(n)
    for i in range(n):
        mesh.neighbors[i].resize(0)
        for k in range(ptr[i], ptr[i + 1]):
            mesh.neighbors[i].push_back(idx[k])

def get_neighbors(Mesh mesh):
    return [list(mesh.neighbors[i]) for i in range(mesh.neighbors.size())]
'''

SETUP = '''\
import os, sys, numpy as np
from setuptools import setup, Extension
from Cython.Build import cythonize
mods = %r
exts = []
for name, extra in mods:
    exts.append(Extension(name.replace("/", "."), [name + ".pyx"] + extra,
        include_dirs=[np.get_include(), ".", "phd/mesh", "phd/domain", "phd/utils"],
        language="c++", extra_compile_args=["-O2", "-ffp-contract=off", "-w"]))
setup(name="phd_ref_build", ext_modules=cythonize(exts, nthreads=%d, quiet=True,
      compiler_directives=dict(language_level=2, cpow=True,
                               legacy_implicit_noexcept=True)),
      script_args=["build_ext", "--inplace", "-j", "%d"])
'''


def stage(reference):
    src_phd = os.path.join(reference, "phd")
    if os.path.isdir(BUILD):
        shutil.rmtree(BUILD)
    os.makedirs(os.path.join(BUILD, "phd"))
    for sub, files in STAGE.items():
        os.makedirs(os.path.join(BUILD, "phd", sub), exist_ok=True)
        for f in files:
            src = os.path.join(src_phd, sub, f)
            dst = os.path.join(BUILD, "phd", sub, f)
            if os.path.exists(src):
                shutil.copyfile(src, dst)
            elif f == "__init__.py":
                open(dst, "w").close()
            else:
                raise FileNotFoundError(src)
    for rel, pat, rep in PY3_EDITS:
        path = os.path.join(BUILD, "phd", rel)
        with open(path) as fh:
            text = fh.read()
        new, n = re.subn(pat, rep, text)
        if n == 0:
            raise RuntimeError("edit %r found nothing in %s" % (pat, rel))
        with open(path, "w") as fh:
            fh.write(new)
    with open(os.path.join(BUILD, "phd", "__init__.py"), "w") as fh:
        fh.write(PHD_INIT)
    os.makedirs(os.path.join(BUILD, "mpi4py"), exist_ok=True)
    with open(os.path.join(BUILD, "mpi4py", "__init__.py"), "w") as fh:
        fh.write(MPI_STUB)
    with open(os.path.join(BUILD, "tess_stub.cpp"), "w") as fh:
        fh.write(TESS_STUB)
    with open(os.path.join(BUILD, "phd", "mesh", "refhelper.pyx"), "w") as fh:
        fh.write(REFHELPER)


def reference_dir():
    """Where the reference tree is read from: $PHD_REFERENCE_DIR, else the default."""
    return os.environ.get("PHD_REFERENCE_DIR", DEFAULT_REFERENCE)


def build(reference, jobs):
    stage(reference)
    with open(os.path.join(BUILD, "setup_ref.py"), "w") as fh:
        fh.write(SETUP % (MODULES, jobs, jobs))
    subprocess.check_call([sys.executable, "setup_ref.py"], cwd=BUILD)
    with open(os.path.join(OUT, "BUILT"), "w") as fh:
        fh.write("reference Cython hot path built from %s\n" % reference)


def platform_suffix():
    import sysconfig
    return sysconfig.get_config_var("EXT_SUFFIX")


def staged_built():
    """True when the staged reference modules are compiled for this interpreter."""
    return os.path.exists(os.path.join(BUILD, "phd", "riemann", "riemann" + platform_suffix()))


def compile_staged(jobs=None):
    """Compile the C++ that Cython generated from the staged reference sources (kept
    under oracle/_ref/build) for this machine, with g++ and no Cython: the step that
    turns the build into a working reference where the reference tree is absent."""
    import sysconfig
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    if not os.path.exists(os.path.join(BUILD, "phd", "riemann", "riemann.cpp")):
        return False
    py_inc = sysconfig.get_paths()["include"]
    suffix = platform_suffix()
    incs = ["-I" + py_inc, "-I" + np.get_include(), "-I.", "-Iphd/mesh", "-Iphd/domain", "-Iphd/utils"]

    def one(item):
        name, extra = item
        out = os.path.join(BUILD, name + suffix)
        cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w"] + incs + \
              [name + ".cpp"] + extra + ["-o", out + ".tmp"]
        subprocess.check_call(cmd, cwd=BUILD)
        os.replace(out + ".tmp", out)

    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        list(ex.map(one, MODULES))
    return True


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=reference_dir())
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--compile-staged", action="store_true",
                    help="compile the already staged sources for this machine (no reference tree needed)")
    a = ap.parse_args()
    if a.compile_staged:
        print("compiled" if compile_staged(a.jobs) else "nothing staged")
        return 0
    if not os.path.isdir(os.path.join(a.reference, "phd")):
        print("reference tree not found at %s; nothing to build" % a.reference)
        return 0
    build(a.reference, a.jobs)
    return 0


if __name__ == "__main__":
    sys.exit(main())
