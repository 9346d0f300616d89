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


# build variants of the oracle for tests that measure a rounding choice:
# rotate_tq rotates vectors as v + w t + b x t (t = 2 b x v) instead of glam's
# mul_vec3 form
VARIANTS = {"": [], "rotate_tq": ["-DDIO_ORACLE_ROTATE_TQ"]}


def build(force=False, verbose=False, variant=""):
    os.makedirs(OUT_DIR, exist_ok=True)
    lib = LIB if not variant else os.path.join(OUT_DIR, f"liboracle_{variant}.so")
    if not force and os.path.exists(lib):
        mtime = os.path.getmtime(lib)
        if all(os.path.getmtime(d) <= mtime for d in DEPS):
            return lib
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas"] + VARIANTS[variant] + \
          ["-o", lib + ".tmp"] + SOURCES
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
