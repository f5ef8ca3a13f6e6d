"""Build the native parts in-tree.

  libdiaq_gb300.so   csrc/*.cu with nvcc for sm_103a only (-gencode arch=compute_103a,code=sm_103a),
                     one process per translation unit, then linked; cudart static.
  diaq_gpu*.so       host/diaq_gpu.cpp, the pybind11 module (headers bundled with torch),
                     linked against libdiaq_gb300.so with an $ORIGIN rpath.

Run ``python -m diaq_gb300.build`` or call ``build()``.  Outputs land in diaq_gb300/lib/ and
diaq_gb300/ (git-ignored); objects in diaq_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libdiaq_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "diaq_gb300.h"))
    return hs


def build_lib(verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = _headers()
    jobs = []
    for f in srcs:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f[:-3] + ".o")
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout, r.stderr)
    objs = [os.path.join(OBJ, f[:-3] + ".o") for f in srcs]
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs])
    return LIB


def module_path() -> str:
    return os.path.join(PKG, "diaq_gpu" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_module() -> str:
    import torch  # only for the location of its bundled pybind11 headers

    tinc = os.path.join(os.path.dirname(torch.__file__), "include")
    out = module_path()
    src = os.path.join(HOST, "diaq_gpu.cpp")
    if _stale(out, [src, LIB, os.path.join(ROOT, "include", "diaq_gb300.h")]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", src, "-o", out,
              f"-I{tinc}", f"-I{sysconfig.get_paths()['include']}", f"-I{os.path.join(ROOT, 'include')}",
              f"-L{LIBDIR}", "-ldiaq_gb300", "-Wl,-rpath,$ORIGIN/lib"])
    return out


def build(verbose: bool = False):
    lib = build_lib(verbose)
    mod = build_module()
    return lib, mod


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
