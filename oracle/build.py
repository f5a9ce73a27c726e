"""Build the CPU oracle (test infrastructure): oracle/build/libgla_oracle.so.

The reference (GenericLinearAlgebra.jl) is pure Julia with no compiled
sources, so there is no `oracle/_ref` build; the oracle is the C++
restatement in gla_ref.hpp. Compiled with -ffp-contract=off so that x86_64
and aarch64 hosts produce the same bits (no FMA contraction, as in Julia).
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
