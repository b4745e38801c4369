"""The C-ABI library builds for sm_103a and exports every declared symbol.

Runs without a GPU: no compute call is made."""
import ctypes
import os
import re

import pytest

from libhybridgrains_gb300 import _capi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _capi.load()


def test_every_declared_symbol_is_exported(lib):
    declared = _capi.declared_symbols()
    assert len(declared) >= 35
    missing = [s for s in declared if not hasattr(lib, s)]
    assert missing == []
    # every declared entry point has a ctypes signature in the binding
    assert sorted(_capi.SIGNATURES) == declared


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "hg_gpu.h"\nint main(void){hg_mpm_desc d; (void)d; return HG_OK;}\n')
    import subprocess
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(tmp_path / "t")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_struct_layouts_match_header(lib):
    # sizes of the descriptor structs seen by ctypes equal the C compiler's
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "s.c")
        with open(src, "w") as f:
            f.write('#include <stdio.h>\n#include "hg_gpu.h"\nint main(void){printf("%zu %zu %zu %zu %zu",'
                    ' sizeof(hg_mpm_desc), sizeof(hg_mpm_plane), sizeof(hg_dem_desc),'
                    ' sizeof(hg_dem_plane), sizeof(hg_dem_drum)); return 0;}\n')
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True).stdout.split()
    sizes = list(map(int, out))
    assert sizes == [ctypes.sizeof(_capi.MpmDesc), ctypes.sizeof(_capi.MpmPlane),
                     ctypes.sizeof(_capi.DemDesc), ctypes.sizeof(_capi.DemPlane),
                     ctypes.sizeof(_capi.DemDrum)]


def test_status_strings(lib):
    assert lib.hg_status_string(0) == b"ok"
    assert lib.hg_status_string(4) == b"capacity exceeded"


def test_no_gpu_fails_loudly(lib):
    """Without a device the context call reports an error instead of falling
    back to the CPU."""
    h = ctypes.c_void_p()
    st = lib.hg_context_create(0, ctypes.byref(h))
    if st == 0:
        lib.hg_context_destroy(h)
        pytest.skip("a GPU is present")
    assert st in (1, 2)
    assert lib.hg_last_error()


def test_tuning_table_round_trip(lib, tmp_path):
    """The launch-shape table (host only): save, merge, clear, and a
    malformed file is refused without touching the table."""
    import libhybridgrains_gb300 as hg
    hg.tune_clear()
    p = tmp_path / "shapes.txt"
    p.write_text("0 152 8192 2097152 2 16\n1 152 0 16777216 3 8\n")
    hg.tune_load(str(p))
    q = tmp_path / "out.txt"
    hg.tune_save(str(q))
    assert q.read_text() == p.read_text()
    bad = tmp_path / "bad.txt"
    bad.write_text("0 152 8192\n")
    with pytest.raises(hg.HGError):
        hg.tune_load(str(bad))
    bad.write_text("0 152 8192 2097152 99 16\n")  # CTAs per SM out of range
    with pytest.raises(hg.HGError):
        hg.tune_load(str(bad))
    hg.tune_save(str(q))
    assert q.read_text() == p.read_text()
    hg.tune_clear()
    hg.tune_save(str(q))
    assert q.read_text() == ""


def test_bounds_variant_builds_and_exports(lib):
    """The bounds-checking variant compiles for sm_103a and exports the same
    entry points (loaded here without a GPU only to list its symbols)."""
    path = build.build(bounds_check=True)
    assert path.endswith("libhg_gpu_bounds.so") and os.path.exists(path)
    other = ctypes.CDLL(path)
    assert all(hasattr(other, s) for s in _capi.declared_symbols())
