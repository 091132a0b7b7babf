"""In-tree build of the native libraries (no setuptools, no cmake).

* ``libtmc_meshgen.so`` - host C++ mesh generator (g++).
* ``libtmcore_gpu.so``  - sm_103a CUDA kernels + host-side mesh preparation +
  the C ABI declared in ``include/tmcore_gpu.h`` (nvcc).

Objects are compiled in parallel; a library is rebuilt only when one of its
sources or headers is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unknown-pragmas"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build tmcore_gb300")
    return cand


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if os.environ.get("TMC_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout)


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    return hs


# (source, compiler, extra flags)
GPU_SOURCES = [
    ("tmc_api.cu", "nvcc", []),
    ("tmc_kernels_f64.cu", "nvcc", ["-fmad=false"]),
    ("tmc_kernels_f32.cu", "nvcc", []),
    ("tmc_noalloc.cu", "nvcc", []),
    ("tmc_ensemble.cu", "nvcc", []),
    ("tmc_mlp.cu", "nvcc", []),
    ("tmc_coarsen.cu", "nvcc", []),
    ("tmc_prep.cpp", "g++", ["-ffp-contract=off"]),
    ("tmc_netcdf.cpp", "g++", []),
]


def _compile(src: str, tool: str, extra: list[str], force: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if not force and not _newer(obj, [path] + _headers()):
        return obj
    if tool == "nvcc":
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
               "-I", INCLUDE, "-I", CSRC, *extra, "-c", path, "-o", obj]
    else:
        cmd = ["g++", *CXXFLAGS, "-I", INCLUDE, "-I", CSRC, *extra, "-c", path, "-o", obj]
    _run(cmd)
    return obj


def build(force: bool = False, verbose: bool = False) -> dict[str, str]:
    """Compile every native library of the package; return {name: path}."""
    os.makedirs(OBJ, exist_ok=True)
    out: dict[str, str] = {}

    # host mesh generator
    mg_src = os.path.join(CSRC, "meshgen.cpp")
    mg_lib = os.path.join(OUT, "libtmc_meshgen.so")
    if force or _newer(mg_lib, [mg_src]):
        _run(["g++", *CXXFLAGS, "-shared", mg_src, "-o", mg_lib])
    out["meshgen"] = mg_lib

    # CUDA library
    gpu_lib = os.path.join(OUT, "libtmcore_gpu.so")
    srcs = [s for s in GPU_SOURCES if os.path.exists(os.path.join(CSRC, s[0]))]
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s[0], s[1], s[2], force), srcs))
    if force or _newer(gpu_lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fopenmp", *objs, "-o", gpu_lib, "-lgomp"])
    out["gpu"] = gpu_lib
    if verbose:
        for k, v in out.items():
            print(f"built {k}: {v}")
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
