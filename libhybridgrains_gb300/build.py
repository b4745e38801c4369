"""Build recipe for libhg_gpu.so (the C-ABI CUDA library), in-tree.

Each translation unit is compiled for sm_103a only, in parallel, and linked
into ``libhybridgrains_gb300/_build/libhg_gpu.so``. Translation units that
restate the reference's FP64 arithmetic are compiled with ``--fmad=false`` so
that every multiply and add rounds separately, matching the operation order of
the reference's expressions; the mixed-precision path keeps FMA contraction.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhg_gpu.so")
# The bounds-checking variant (HG_BOUNDS_CHECK: computed indices checked on
# the device, HG_STATUS_INDEX set and the access skipped), for tests; loaded
# instead of libhg_gpu.so when HG_GPU_VARIANT=bounds.
BOUNDS_DIR = os.path.join(HERE, "_build_bounds")
BOUNDS_LIB = os.path.join(BOUNDS_DIR, "libhg_gpu_bounds.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, exact-FP64 translation unit). The mixed-precision unit is built
# with fast FP32 division and square root: its FP32 results are checked
# against the FP64 oracle with a stated tolerance, not bit for bit.
SOURCES = [
    ("capi.cu", True),
    ("scan.cu", False),
    ("mpm_fp64.cu", True),
    ("mpm_mixed.cu", None),
    ("dem.cu", True),
    ("coupling.cu", True),
    ("zones.cu", True),  # host code (zone labels)
    ("resampling.cu", True),  # host code (resampling)
    ("state.cu", False),  # checkpoint / resume blobs
]
HEADERS = ["hg_internal.cuh", "mpm_basis.cuh", "scan_block.cuh", "zones_internal.cuh"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src, exact, verbose, out_dir=OUT_DIR, defines=()):
    obj = os.path.join(out_dir, src.replace(".cu", ".o"))
    # -ffp-contract=off keeps the host-side seeding and grid set-up rounding
    # identical on x86 and on Arm (where GCC would otherwise fuse a*b+c).
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
           "-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
    for d in defines:
        cmd.insert(1, "-D" + d)
    if exact:
        cmd.insert(1, "--fmad=false")
    elif exact is None:
        cmd.insert(1, "--use_fast_math")
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, s) for s, _ in SOURCES] + [os.path.join(CSRC, h) for h in HEADERS]
    deps.append(os.path.join(INCLUDE, "hg_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, bounds_check=False):
    """Compile and link libhg_gpu.so (or, with bounds_check, the
    bounds-checking libhg_gpu_bounds.so) if any source is newer than it."""
    lib, out_dir = (BOUNDS_LIB, BOUNDS_DIR) if bounds_check else (LIB, OUT_DIR)
    defines = ("HG_BOUNDS_CHECK",) if bounds_check else ()
    if not force and not _stale(lib):
        return lib
    os.makedirs(out_dir, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s[0], s[1], verbose, out_dir, defines),
                              SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                bounds_check="--bounds" in sys.argv))
