"""Builds oracle/_ref/libhg_ref.so from the reference's own sources (test
infrastructure only, never shipped or timed as the product).

Only the reference files that compile standalone are used, from where they
lie in the reference checkout:

* ``hybridgrains2dnew/CircleRectangleIntersection.cpp`` (disk/box area of the
  packing fraction), wrapped by ``oracle/ref_shim.cpp``;
* ``hybridgrains2dnew/random.c`` (MT19937 of the resampling insertion;
  ``seedMT``, ``randomMT``, ``randomMT_i``).

The rest of the reference needs Eigen, RapidXML and HDF5, which are absent.
The checkout is the argument (``python oracle/build_ref.py <reference_root>``,
or ``build(root)``), else $HG_REFERENCE_ROOT. Without one, an earlier build
is reused; where none exists (as on machines that only run the GPU tests)
nothing is built and the tests that need the library are skipped.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libhg_ref.so")


def build(root=None, force=False):
    root = root or os.environ.get("HG_REFERENCE_ROOT")
    if not root:
        return LIB if os.path.exists(LIB) else None
    src_dir = os.path.join(root, "hybridgrains2dnew")
    sources = [os.path.join(src_dir, "CircleRectangleIntersection.cpp"),
               os.path.join(src_dir, "random.c"), os.path.join(HERE, "ref_shim.cpp")]
    if not all(os.path.exists(s) for s in sources[:2]):
        return LIB if os.path.exists(LIB) else None
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
    args = [a for a in sys.argv[1:] if a != "--force"]
    print(build(args[0] if args else None, force="--force" in sys.argv))
