"""Build libflecsale_gb300.so in-tree for sm_103a.

Each translation unit is compiled in parallel; the FP64 kernel file is compiled
with --fmad=false so its arithmetic rounds exactly like the reference's CPU
code.  Outputs: flecsale_gb300/_build/*.o and flecsale_gb300/libflecsale_gb300.so.
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libflecsale_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-Xcompiler", "-fopenmp", "-I", INCLUDE, "-I", CSRC,
                      "--expt-relaxed-constexpr"]
CXX_COMMON = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17",
              "-I", INCLUDE, "-I", CSRC]

# (source, extra flags)
UNITS = [
    ("fvh_mesh.cpp", []),
    ("fvh_problems.cpp", []),
    ("fvh_io.cpp", []),
    ("fvh_plain.cu", ["--fmad=false"]),
    ("fvh_mixed.cu", ["-prec-div=false", "-prec-sqrt=false"]),
    ("fvh_capi.cu", []),
    ("fvh_noalloc.cu", []),
    ("fvh_batch.cu", []),
    ("fvh_lua.cpp", []),
    ("fvh_input.cpp", []),
]
# the command-line driver (apps/hydro's executable), linked against the library
DRIVER_SRC = "fvh_driver.cpp"
DRIVER = os.path.join(PKG, "flecsale_hydro")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build flecsale_gb300")


def _sources_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str, extra: list[str]) -> tuple[str, str]:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if src.endswith(".cu"):
        cmd = [_nvcc(), *NVCC_COMMON, *extra, "-c", path, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_COMMON, *extra, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of libflecsale_gb300.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda u: _compile(*u), UNITS))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static",
           "-Xcompiler", "-fopenmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I", INCLUDE,
           os.path.join(CSRC, DRIVER_SRC), "-o", DRIVER + ".tmp", "-L", PKG, "-lflecsale_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
