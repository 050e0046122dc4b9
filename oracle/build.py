"""Builds the oracle shared library (oracle/liblucid_oracle.so) with g++.

The oracle must use plain IEEE float arithmetic with no FMA contraction so that it matches the
CUDA path bit for bit: -ffp-contract=off (GCC contracts by default on aarch64), no
-ffast-math, no -march=native (the same source builds on x86-64 and aarch64).

The reference's own setup, bin-counter and row-span shader functions are compiled separately
into oracle/_ref by oracle/ref_build.py (the pin of this oracle); its raster passes need a
graphics stack and its host code the libfwk submodule, which is empty.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liblucid_oracle.so")
SRC = [os.path.join(HERE, "lucid_oracle.cpp")]
HDR = [os.path.join(HERE, "lucid_oracle.h"), os.path.join(HERE, "..", "include", "lucid_gb300.h")]


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SRC + HDR)


def build(force: bool = False) -> str:
    if force or needs_build():
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
               "-fno-fast-math", "-Wall", "-o", LIB + ".tmp"] + SRC
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
