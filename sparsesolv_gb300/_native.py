"""Build and load the native libraries of the package.

Three shared objects are built in-tree, next to their sources:

* ``libsparsesolv_gb300.so`` -- the sm_103a CUDA kernels, the C++ solver
  drivers and the C-ABI declared in ``include/sparsesolv_gb300.h``
  (``nvcc -gencode arch=compute_103a,code=sm_103a``);
* ``voxel/libvoxelgen.so`` -- the host-side seeded voxel FEM system generator
  (plain C, ``-ffp-contract=off`` so that x86-64 and aarch64 builds produce
  bit-identical matrices);
* ``SparseSolvPy<ext>`` -- the compiled Python module (pybind11 bindings of the
  C++ drop-in classes of ``include/SparseSolv/``, linked against the CUDA
  library; ``pybind/sparsesolvpy.cpp``). pybind11's headers come from the
  installed torch (``torch/include``), else from an installed pybind11.

Nothing here falls back to a CPU implementation: :func:`load_solver` raises
when the CUDA library is missing or cannot be loaded.
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
SOLVER_LIB = os.path.join(PKG_DIR, "libsparsesolv_gb300.so")
VOXEL_LIB = os.path.join(PKG_DIR, "voxel", "libvoxelgen.so")
PYBIND_SRC = os.path.join(PKG_DIR, "pybind", "sparsesolvpy.cpp")
PYBIND_MOD = os.path.join(PKG_DIR, "SparseSolvPy" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation units of the CUDA library (compiled in parallel, then linked)
CUDA_SOURCES = [
    "ss_levels.cu",
    "ss_factor.cu",
    "ss_trsv.cu",
    "ss_cluster.cu",
    "ss_spmv_vec.cu",
    "ss_solver.cu",
    "ss_batch.cu",
    "ss_build.cu",
    "ss_post.cu",
    "ss_voxel.cu",
    "ss_push.cu",
    "ss_push_plan.cpp",
    "ss_capi.cu",
]


# the IC factor restates the reference's arithmetic operation by operation; no FMA contraction there
EXTRA_FLAGS = {"ss_factor.cu": ["-fmad=false"]}


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (proc.returncode, " ".join(cmd), proc.stdout))
    return proc.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_voxel(force=False):
    src = os.path.join(PKG_DIR, "voxel", "voxelgen.c")
    if not force and _newer(VOXEL_LIB, [src]):
        return VOXEL_LIB
    _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-o", VOXEL_LIB, src, "-lm"])
    return VOXEL_LIB


def build_solver(force=False, verbose=False):
    """Compile the CUDA library for sm_103a (cross-compiles without a GPU)."""
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES]
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h", ".hpp"))]
    hdrs.append(os.path.join(INCLUDE, "sparsesolv_gb300.h"))
    if not force and _newer(SOLVER_LIB, srcs + hdrs):
        return SOLVER_LIB
    objdir = os.path.join(PKG_DIR, "_build")
    os.makedirs(objdir, exist_ok=True)
    common = [NVCC, *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", INCLUDE, "-I", CSRC]
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        out = _run(common + EXTRA_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj])
        return obj, out

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, out in results:
            sys.stdout.write(out)
    # every symbol resolved at link time: a missing definition fails the build, not the first load
    _run([NVCC, *ARCH_FLAGS, "-shared", "-Xlinker", "--no-undefined", "-o", SOLVER_LIB, *objs, "-lcudart", "-lpthread"])
    return SOLVER_LIB


def _pybind11_include():
    """pybind11's headers: torch's bundled copy (found without importing torch), else pybind11's own."""
    spec = importlib.util.find_spec("torch")
    if spec is not None and spec.submodule_search_locations:
        inc = os.path.join(list(spec.submodule_search_locations)[0], "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    spec = importlib.util.find_spec("pybind11")
    if spec is not None:
        import pybind11
        return pybind11.get_include()
    raise RuntimeError("sparsesolv_gb300: no pybind11 headers (torch/include or the pybind11 package) found")


def build_pybind(force=False):
    """Compile the SparseSolvPy module (host C++, linked against the CUDA library)."""
    hdrs = [os.path.join(INCLUDE, "SparseSolv", h) for h in os.listdir(os.path.join(INCLUDE, "SparseSolv"))]
    deps = [PYBIND_SRC, SOLVER_LIB, os.path.join(INCLUDE, "sparsesolv_gb300.h"), *hdrs]
    if not force and _newer(PYBIND_MOD, deps):
        return PYBIND_MOD
    py_inc = sysconfig.get_paths()["include"]
    if not os.path.exists(os.path.join(py_inc, "Python.h")):
        raise RuntimeError("sparsesolv_gb300: Python.h not found under %s; SparseSolvPy cannot be built" % py_inc)
    _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", "-I", INCLUDE, "-I", py_inc,
          "-I", _pybind11_include(), PYBIND_SRC, "-o", PYBIND_MOD, "-L", PKG_DIR, "-lsparsesolv_gb300",
          "-Wl,-rpath,$ORIGIN"])
    return PYBIND_MOD


def build_all(force=False, verbose=False):
    build_voxel(force)
    build_solver(force, verbose)
    build_pybind(force)


_solver = None
_voxel = None


def load_voxel():
    global _voxel
    if _voxel is None:
        if not os.path.exists(VOXEL_LIB):
            build_voxel()
        _voxel = ctypes.CDLL(VOXEL_LIB)
    return _voxel


def load_solver():
    """Load the CUDA library; raises if it is missing (there is no CPU path)."""
    global _solver
    if _solver is None:
        if not os.path.exists(SOLVER_LIB):
            raise RuntimeError(
                "sparsesolv_gb300: CUDA library %s is missing; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first" % SOLVER_LIB)
        _solver = ctypes.CDLL(SOLVER_LIB)
        from . import _capi
        _capi.declare(_solver)
    return _solver
