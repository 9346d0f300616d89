"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/oracle_capi.cpp (which includes the header-only restatement
oracle/dio_oracle.hpp) into oracle/_build/liboracle.so.  Flags keep float
arithmetic IEEE and uncontracted (-ffp-contract=off) so the oracle performs
exactly the operations it spells out, on x86_64 and aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
DEPS = SOURCES + [os.path.join(HERE, "dio_oracle.hpp"),
                  os.path.join(HERE, "..", "include", "dio_cuda.h")]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= mtime for d in DEPS):
            return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas",
           "-o", LIB + ".tmp"] + SOURCES
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
