"""The reference-side shims of INTEGRATION.md as compilable sources (test
infrastructure).

INTEGRATION.md marks each shim as a C++ code block whose first line is
``// shim: <name>``; ``blocks()`` returns them by name, and ``compile()``
builds one against ``reference_stubs.h`` (stand-ins for the reference's
declarations) and ``include/hg_gpu.h``.
"""
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DOC = os.path.join(ROOT, "INTEGRATION.md")


def blocks():
    with open(DOC) as f:
        text = f.read()
    out = {}
    for m in re.finditer(r"```cpp\n// shim: (\w+)\n(.*?)```", text, re.S):
        out[m.group(1)] = m.group(2)
    return out


def flags():
    # the reference's language level (its CMakeLists use C++14)
    return ["-std=c++14", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
            "-I", os.path.join(ROOT, "include"), "-I", HERE]


def write_unit(tmpdir, name):
    """A translation unit: the stand-in declarations, then the shim."""
    path = os.path.join(str(tmpdir), "%s_shim.cpp" % name)
    with open(path, "w") as f:
        f.write('#include "reference_stubs.h"\n')
        f.write(blocks()[name])
    return path


def syntax_check(tmpdir, name):
    src = write_unit(tmpdir, name)
    return subprocess.run(["g++", *flags(), "-fsyntax-only", src], capture_output=True,
                          text=True)


def build_dem_driver(tmpdir, lib_dir):
    """tests/integration/dem_shim_driver.cpp with the DEM shim, linked
    against libhg_gpu.so in lib_dir."""
    inc = os.path.join(str(tmpdir), "dem_shim.inc")
    with open(inc, "w") as f:
        f.write(blocks()["dem"])
    exe = os.path.join(str(tmpdir), "dem_shim_driver")
    cmd = ["g++", *flags(), "-I", str(tmpdir), os.path.join(HERE, "dem_shim_driver.cpp"),
           "-o", exe, "-L", lib_dir, "-lhg_gpu", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return exe, r
