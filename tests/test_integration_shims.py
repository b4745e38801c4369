"""The reference-side shims in INTEGRATION.md compile.

Each shim (the MPM ExplicitIntegrator functions, the DEM ImpactFrictionMap
subclass) is compiled as C++14 with warnings as errors against stand-ins of
the reference's declarations (tests/integration/reference_stubs.h, which
keeps the reference's names and signatures: ImpactFrictionMap.h:41-80,
ExplicitIntegrator.h:8-13, SimulationState.h, RigidBody2DState.h) and the
library's header, so that the recipes stay in step with both. The DEM
shim's behaviour is run on the GPU by tests/test_gpu_integration_shims.py.
"""
import shutil

import pytest

from integration import shims

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


def test_every_shim_is_marked():
    assert set(shims.blocks()) == {"mpm", "dem"}


@pytest.mark.parametrize("name", ["mpm", "dem"])
def test_shim_compiles_against_reference_declarations(tmp_path, name):
    r = shims.syntax_check(tmp_path, name)
    assert r.returncode == 0, r.stderr


def test_dem_driver_links_against_the_library(tmp_path):
    from libhybridgrains_gb300 import build
    lib = build.build()
    exe, r = shims.build_dem_driver(tmp_path, __import__("os").path.dirname(lib))
    assert r.returncode == 0, r.stderr
