"""Builds lucid_gb300/liblucid_gb300.so from csrc/*.cu with nvcc for sm_103a only.

Numerics flags are part of the contract with the CPU oracle: --fmad=false (no FMA
contraction), IEEE division and square root, no flush-to-zero. Translation units compile in
parallel; the object files go to lucid_gb300/_build/ (git-ignored).

`python -m lucid_gb300.build --counters` builds a second library,
liblucid_gb300_counters.so, with the raster kernel's work counters compiled in
(LUCID_RASTER_COUNTERS, read by lucid_gb300/profile_raster.py); the product library is not
touched.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblucid_gb300.so")
COUNTERS_LIB = os.path.join(HERE, "liblucid_gb300_counters.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xptxas", "-warn-spills", "-I", INCLUDE]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in sources() + headers())


def _compile(src: str, extra, build_dir: str = BUILD) -> str:
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False, counters: bool = False) -> str:
    """Compiles every CUDA source and links the shared library. Returns its path."""
    lib = COUNTERS_LIB if counters else LIB
    if not force and not counters and not needs_build():
        return LIB
    build_dir = os.path.join(BUILD, "counters") if counters else BUILD
    os.makedirs(build_dir, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    if counters:
        extra += ["-DLUCID_RASTER_COUNTERS=1"]
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv,
                counters="--counters" in sys.argv))
