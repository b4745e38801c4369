"""Builds oracle/_ref/libhg_ref.so from the reference's own sources (test
infrastructure only, never shipped or timed as the product).

Only the reference files that compile standalone are used, from where they
lie in the reference checkout:

* ``hybridgrains2dnew/CircleRectangleIntersection.cpp`` (disk/box area of the
  packing fraction), wrapped by ``oracle/ref_shim.cpp``;
* ``hybridgrains2dnew/random.c`` (MT19937 of the resampling insertion;
  ``seedMT``, ``randomMT``, ``randomMT_i``).

The rest of the reference needs Eigen, RapidXML and HDF5, which are absent.
The checkout is looked up in $HG_REFERENCE_ROOT, else /root/reference; when it
is absent (as on machines that only run the GPU tests), nothing is built and
the tests that need the library are skipped.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libhg_ref.so")


def reference_root():
    return os.environ.get("HG_REFERENCE_ROOT", "/root/reference")


def build(force=False):
    src_dir = os.path.join(reference_root(), "hybridgrains2dnew")
    sources = [os.path.join(src_dir, "CircleRectangleIntersection.cpp"),
               os.path.join(src_dir, "random.c"), os.path.join(HERE, "ref_shim.cpp")]
    if not all(os.path.exists(s) for s in sources[:2]):
        return None
    if not force and os.path.exists(LIB) and \
            all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in sources):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []
    for s in sources:
        obj = os.path.join(OUT_DIR, os.path.basename(s) + ".o")
        cc = "gcc" if s.endswith(".c") else "g++"
        subprocess.run([cc, "-O2", "-fPIC", "-ffp-contract=off", "-I", src_dir, "-c", s,
                        "-o", obj], check=True)
        objs.append(obj)
    subprocess.run(["g++", "-shared", "-o", LIB + ".tmp"] + objs, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
