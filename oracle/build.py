"""Build the CPU oracle (test infrastructure): oracle/build/libgla_oracle.so.

The reference (GenericLinearAlgebra.jl) is pure Julia with no compiled
sources, so there is no `oracle/_ref` build; the oracle is the C++
restatement in gla_ref.hpp. Compiled with -ffp-contract=off so that x86_64
and aarch64 hosts produce the same bits (no FMA contraction, as in Julia).
No -march=native: the same source must build and give the same results on
the x86_64 build host and the aarch64 (Grace) GPU host, so the flags name no
host-specific instruction set; with contraction off and no -ffast-math the
compiler may not reassociate the reductions anyway, so a native target would
change speed only through wider loads.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "libgla_oracle.so")


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "gla_ref.cpp")]
    hdr = [os.path.join(HERE, "gla_ref.hpp")]
    if not force and os.path.exists(LIB):
        lib_m = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) <= lib_m for f in src + hdr):
            return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", *src, "-o", LIB + ".tmp"]
    if platform.machine() == "x86_64":
        cmd.append("-lquadmath")
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
