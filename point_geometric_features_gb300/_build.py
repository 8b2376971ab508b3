"""Build the native parts in-tree: libpgeof_cuda.so (nvcc, sm_103a) and the
``pgeof_ext`` Python module (g++, pybind11 headers bundled with PyTorch).

Usage: ``python point_geometric_features_gb300/_build.py [--force]`` (runs without
importing the package, which needs the built library).
Nothing here runs at import time; a missing library makes the package raise.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import importlib.util
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpgeof_cuda.so")
EXT = os.path.join(PKG, "pgeof_ext" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _pybind11_include():
    spec = importlib.util.find_spec("torch")
    if spec and spec.submodule_search_locations:
        inc = os.path.join(list(spec.submodule_search_locations)[0], "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    try:
        import pybind11  # noqa: PLC0415

        return pybind11.get_include()
    except ImportError as e:  # pragma: no cover
        raise RuntimeError("pybind11 headers not found (neither torch/include nor the pybind11 package)") from e


def build_library(force: bool = False, jobs: int | None = None) -> str:
    """Compile every csrc/*.cu for sm_103a in parallel and link libpgeof_cuda.so."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            todo.append((s, o))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_run, [NVCC] + NVCC_FLAGS + ["-c", s, "-o", o]) for s, o in todo]
            for f in futs:
                f.result()
    if force or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"])
        os.replace(tmp, LIB)
    return LIB


def build_extension(force: bool = False) -> str:
    """Compile the pybind11 module pgeof_ext against libpgeof_cuda.so."""
    src = os.path.join(CSRC, "pgeof_ext.cpp")
    deps = [src, LIB] + glob.glob(os.path.join(INCLUDE, "*.h"))
    if force or _stale(EXT, deps):
        tmp = EXT + f".tmp{os.getpid()}"
        cmd = [
            os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
            "-I" + sysconfig.get_paths()["include"], "-I" + _pybind11_include(), "-I" + INCLUDE,
            src, "-o", tmp, "-L" + PKG, "-lpgeof_cuda", "-Wl,-rpath,$ORIGIN",
        ]
        _run(cmd)
        os.replace(tmp, EXT)
    return EXT


def build(force: bool = False) -> None:
    build_library(force)
    build_extension(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB)
    print(EXT)
