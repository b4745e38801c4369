"""The CPU oracle built with AddressSanitizer and UndefinedBehaviorSanitizer
(g++ -fsanitize=address,undefined) runs a small MPM column (linear and
uGIMP), a DEM pile with planes and a fixed body, and the node-node coupling,
in a child process with the sanitizer runtimes preloaded: no memory error
and no undefined behaviour is reported."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import numpy as np
import oracle
from libhybridgrains_gb300 import scenes
cfg = scenes.mpm_column("column_12800")
p = scenes.seed_column_points(cfg)
k = np.arange(0, len(p["m"]), 16)
for basis in (0, 1):
    o = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"], basis=basis,
                   shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                   dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"], gravity=scenes.GRAVITY)
    for (x, n, st, lb) in cfg["planes"]:
        o.add_plane(x, n, st, lb)
    o.set_particles(p["q"][k], p["v"][k], p["m"][k], p["vol"][k], p["hl"][k])
    o.step(cfg["dt"], 5)
sc = scenes.dem_column(n=200, per_row=20)
sc["fixed"][0] = 1
dp = scenes.dem_params()
d = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
               dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
d.add_plane((0.0, 0.0), (0.0, 1.0))
d.step(1e-6, 20)
d.step(1e-6, 5, weighted=True)
h = scenes.hybrid_column(scale=0.01)
hc = h["mpm"]
hp = scenes.seed_column_points(hc)
m = oracle.MPM(hc["grid_min"], hc["grid_max"], hc["h"], basis=1,
               shear_modulus=hc["shear_modulus"], bulk_modulus=hc["bulk_modulus"],
               dp_alpha=hc["dp_alpha"], flip_alpha=hc["flip_alpha"], gravity=scenes.GRAVITY)
for (x, n, st, lb) in hc["planes"]:
    m.add_plane(x, n, st, lb)
m.set_particles(hp["q"], hp["v"], hp["m"], hp["vol"], hp["hl"])
g = h["dem"]
hd = oracle.DEM(g["q"], g["v"], g["r"], g["m"], g["I"], g["fixed"], scenes.GRAVITY,
                dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
c = oracle.Hybrid(m, hd)
c.step(1e-6, 3, homogenize_stress=True, homogenize_velocity=True)
print("sanitized oracle ok")
"""


def runtime(name):
    path = subprocess.run(["g++", "-print-file-name=" + name], capture_output=True,
                          text=True).stdout.strip()
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_oracle_under_asan_and_ubsan(tmp_path):
    asan, ubsan = runtime("libasan.so"), runtime("libubsan.so")
    if not asan or not ubsan:
        pytest.skip("g++ sanitizer runtimes not installed")
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    lib = str(tmp_path / "libhg_oracle_san.so")
    srcs = [os.path.join(ROOT, "oracle", s) for s in ob.SOURCES]
    subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fPIC", "-shared", "-fopenmp",
                    "-ffp-contract=off", "-fno-omit-frame-pointer",
                    "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                    "-o", lib] + srcs, check=True)
    env = dict(os.environ, HG_ORACLE_LIB=lib, LD_PRELOAD=asan + " " + ubsan,
               ASAN_OPTIONS="detect_leaks=0", UBSAN_OPTIONS="print_stacktrace=1",
               PYTHONPATH=ROOT, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-4000:]
    assert "sanitized oracle ok" in r.stdout
