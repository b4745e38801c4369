"""The bounds-checking build (libhg_gpu_bounds.so, HG_BOUNDS_CHECK): every
computed grid-node, tile, particle-range, bucket, body and contact index is
checked on the device, and an index outside its array would set
HG_STATUS_INDEX and skip the access. The same small cases (MIXED column
across re-sorts and graph chunks, a batch of three scenes, DEM piles with an
edit, a hybrid column) run through both builds in separate processes: no
status bit is set, the DEM results are identical bit for bit and the MPM
results agree to the order of atomic sums."""
import os
import subprocess
import sys

import numpy as np
import pytest

from libhybridgrains_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def run_cases(tmp_path, variant):
    env = dict(os.environ)
    env.pop("HG_GPU_VARIANT", None)
    if variant:
        env["HG_GPU_VARIANT"] = variant
    out = tmp_path / ("cases_%s.npz" % (variant or "release"))
    subprocess.run([sys.executable, os.path.join(HERE, "bounds_cases.py"), str(out)], env=env,
                   check=True, timeout=600)
    with np.load(out) as f:
        return {k: f[k] for k in f.files}


def test_bounds_checking_build(tmp_path):
    build.build()
    build.build(bounds_check=True)
    a = run_cases(tmp_path, "")
    b = run_cases(tmp_path, "bounds")
    for r in (a, b):
        assert int(r["mixed_status"]) == 0 and int(r["dem_status"]) == 0
        assert not r["batch_status"].any() and not r["hybrid_status"].any()
    assert np.array_equal(a["dem_q"], b["dem_q"]) and np.array_equal(a["dem_v"], b["dem_v"])
    assert np.array_equal(a["dem_contacts"], b["dem_contacts"])
    assert np.abs(a["mixed_q"] - b["mixed_q"]).max() <= 1e-9
    assert np.abs(a["batch_q0"] - b["batch_q0"]).max() <= 1e-9
    assert np.abs(a["hybrid_q"] - b["hybrid_q"]).max() <= 1e-9
