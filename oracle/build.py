"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/aeros_oracle.cpp into oracle/_build/libaeros_oracle.so with the
host compiler.  Portable flags only (the library is rebuilt on every machine, x86-64 and aarch64):
no -march=native, no ISA intrinsics.  -ffp-contract=off keeps the arithmetic
free of fused multiply-adds on both x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libaeros_oracle.so")
SRC = os.path.join(HERE, "aeros_oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "aeros_gpu.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
