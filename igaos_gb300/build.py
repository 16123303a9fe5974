"""Build of the engine's native parts, in-tree (no pip install).

  libigaos_pdhg.so  -- CUDA engine behind the C ABI (include/igaos_pdhg.h)
  igaos             -- CLI with `solve <model.mps> --engine pdhg`
  _core*.so         -- pybind11 module (igaos.solve / read_mps surface)

nvcc compiles for sm_103a only. Translation units build in parallel.
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libigaos_pdhg.so")
CLI = os.path.join(PKG, "igaos")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", INC, "-I", CSRC] + ARCH
CU_SOURCES = ["engine.cu", "capi.cu", "batch.cu", "kkt_noalloc.cu", "unrolled.cu", "host_kkt.cu",
              "calibrate.cu", "certificate.cu", "presolve.cu",
              "crossover.cu"]
# per-file extra nvcc flags
EXTRA_FLAGS = {}
CXX_HOST = ["model.cpp", "pdhg_solve.cpp"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _deps():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hs += [os.path.join(INC, "igaos_pdhg.h")]
    hs += [os.path.join(INC, "igaos", f) for f in os.listdir(os.path.join(INC, "igaos"))]
    return hs


def build_lib(force=False, verbose=False, defines=(), out=None):
    """Builds the engine library; `defines` (e.g. ["IGX_HOT_CTAS=7"]) and `out`
    produce a variant library elsewhere (tuning sweeps)."""
    out = out or LIB
    objdir = BUILD if out == LIB else os.path.join(os.path.dirname(out), "_obj")
    os.makedirs(objdir, exist_ok=True)
    deps = _deps()
    objs = []
    jobs = []
    dflags = [f"-D{d}" for d in defines]
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + deps):
            jobs.append([_nvcc(), *NVFLAGS, *dflags, *EXTRA_FLAGS.get(src, []), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    if force or _newer(out, objs):
        _run([_nvcc(), *ARCH, "-shared", "-o", out, *objs, "-lcudart"])
    return out


def build_cli(force=False):
    srcs = [os.path.join(CSRC, f) for f in ["igaos_cli.cpp", *CXX_HOST]]
    if not all(os.path.exists(s) for s in srcs):
        return None
    if force or _newer(CLI, srcs + _deps() + [LIB]):
        _run(["g++", "-O2", "-std=c++17", "-I", INC, "-I", CSRC, "-o", CLI, *srcs,
              "-L", PKG, "-ligaos_pdhg", "-Wl,-rpath,$ORIGIN"])
    return CLI


def build_pymod(force=False):
    src = os.path.join(CSRC, "py_core.cpp")
    if not os.path.exists(src):
        return None
    import torch.utils.cpp_extension as ce  # only for its pybind11 headers
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(PKG, "_core" + suffix)
    srcs = [src] + [os.path.join(CSRC, f) for f in CXX_HOST]
    if force or _newer(out, srcs + _deps() + [LIB]):
        incs = []
        for d in ce.include_paths():
            incs += ["-I", d]
        pyinc = sysconfig.get_paths()["include"]
        _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", INC, "-I", CSRC, "-I", pyinc,
              *incs, "-o", out, *srcs, "-L", PKG, "-ligaos_pdhg", "-Wl,-rpath,$ORIGIN"])
    return out


def build(force=False, verbose=False):
    build_lib(force, verbose)
    build_cli(force)
    build_pymod(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", LIB)
