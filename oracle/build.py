"""Build recipe for the CPU oracle (test infrastructure only).

Compiles with the host compiler, into oracle/_build/:
  libaeros_oracle.so       oracle/aeros_oracle.cpp, the parity build: -O3
                           -ffp-contract=off keeps the arithmetic free of fused
                           multiply-adds on both x86-64 and aarch64;
  libaeros_oracle_fast.so  the same source built for timing (the CPU baseline):
                           -O3 -ffp-contract=fast -funroll-loops, fused
                           multiply-adds allowed, as an optimising Fortran
                           build of the reference would use them;
  libaeros_truth.so        oracle/truth.cpp, the tendency chain in long double.
Portable flags only (the libraries are rebuilt on every machine, x86-64 and
aarch64): no -march=native, no ISA intrinsics.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libaeros_oracle.so")
LIB_FAST = os.path.join(OUT_DIR, "libaeros_oracle_fast.so")
LIB_TRUTH = os.path.join(OUT_DIR, "libaeros_truth.so")
SRC = os.path.join(HERE, "aeros_oracle.cpp")
SRC_TRUTH = os.path.join(HERE, "truth.cpp")
HDR = os.path.join(HERE, "..", "include", "aeros_gpu.h")

_FLAGS = {
    LIB: (SRC, ["-O3", "-ffp-contract=off"]),
    LIB_FAST: (SRC, ["-O3", "-ffp-contract=fast", "-funroll-loops"]),
    LIB_TRUTH: (SRC_TRUTH, ["-O2", "-ffp-contract=off"]),
}


def _build_one(lib, force):
    src, flags = _FLAGS[lib]
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(src), os.path.getmtime(HDR),
                                             os.path.getmtime(__file__))):
        return lib
    cmd = ["g++", "-std=c++17", "-fPIC", "-shared", "-fopenmp"] + flags + [src, "-o", lib + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def build(force: bool = False, variant: str = "parity") -> str:
    """Build (if stale) and return the path of one library: variant "parity"
    (the oracle the tests check against), "fast" (the timed CPU baseline) or
    "truth" (the long double tendency chain)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    return _build_one({"parity": LIB, "fast": LIB_FAST, "truth": LIB_TRUTH}[variant], force)


def build_all(force: bool = False):
    import concurrent.futures as cf
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(3) as ex:
        return list(ex.map(lambda l: _build_one(l, force), [LIB, LIB_FAST, LIB_TRUTH]))


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
