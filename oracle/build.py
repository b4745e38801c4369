"""Build recipe for the CPU oracle shared library (test infrastructure only).

Compiles the FP64 C++ restatement of the reference's MPM, DEM and coupling
step into ``oracle/_build/libhg_oracle.so``. ``-ffp-contract=off`` keeps every
multiply and add separately rounded, as the restatement's operation order
assumes. OpenMP is enabled for the threaded CPU-baseline mode.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["mpm_oracle.cpp", "dem_oracle.cpp", "coupling_oracle.cpp", "zones_oracle.cpp"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhg_oracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in ("oracle_common.h", "oracle_state.h")]
    if not force and os.path.exists(LIB):
        lib_mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= lib_mtime for d in deps):
            return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-o", LIB + ".tmp"] + srcs
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
