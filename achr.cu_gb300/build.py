"""Build the native parts of the GB300 ACHR sampler in-tree.

Outputs (git-ignored, under achr.cu_gb300/_build/):
  libachr_gb300.so   the C-ABI shared library (CUDA kernels + host set-up + I/O)
  ACHRCuda           the drop-in command line, linked against the library

Compiled for sm_103a only.  Translation units build in parallel; no cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["achr_chain_cfg_small.cu", "achr_chain_cfg_mid.cu", "achr_chain_cfg_large.cu", "achr_chain_launch.cu", "achr_capi.cu",
              "achr_noalloc.cu", "achr_tc_gemm.cu", "achr_reproject.cu", "achr_defer.cu", "achr_precond.cu", "achr_rhat.cu"]
CXX_SOURCES = ["achr_io.cpp"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}")


def library_path() -> Path:
    return OUT / "libachr_gb300.so"


def cli_path() -> Path:
    return OUT / "ACHRCuda"


def build(verbose: bool = False, force: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    cxx = os.environ.get("CXX", "g++")
    OUT.mkdir(parents=True, exist_ok=True)
    objs: list[Path] = []
    jobs = []
    inc = ["-I", str(INCLUDE), "-I", str(SRC)]
    for src in CU_SOURCES:
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *inc, "-c", str(SRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        jobs.append([cxx, *CXX_FLAGS, *inc, "-c", str(SRC / src), "-o", str(obj)])
    srcs = [SRC / s for s in CU_SOURCES + CXX_SOURCES + ["achr_main.cpp"]] + list(SRC.glob("*.cuh")) + \
        list(SRC.glob("*.h"))
    srcs.append(INCLUDE / "achr.h")
    lib = library_path()
    newest = max(p.stat().st_mtime for p in srcs)
    if not force and lib.exists() and lib.stat().st_mtime > newest and cli_path().exists():
        return lib
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    libdir = cuda / "lib64"
    if not libdir.exists():
        libdir = cuda / "lib"
    _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-L", str(libdir),
          "-lcusolver", "-lcublas", "-lcudart", "-Xlinker", f"-rpath={libdir}"])
    main_obj = OUT / "achr_main.o"
    _run([cxx, *CXX_FLAGS, "-pthread", *inc, "-I", str(cuda / "include"), "-c", str(SRC / "achr_main.cpp"), "-o",
          str(main_obj)])
    _run([cxx, "-pthread", "-o", str(cli_path()), str(main_obj), "-L", str(OUT), "-lachr_gb300", "-L", str(libdir),
          "-lcudart", f"-Wl,-rpath,{OUT}", f"-Wl,-rpath,{libdir}"])
    if verbose:
        print(f"built {lib} and {cli_path()}")
    return lib


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
