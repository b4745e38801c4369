"""Long-horizon agreement of the GPU paths with the FP64 oracle. Granular flow
is chaotic, so point states diverge; the shape of the collapse must not.

The 12,800-point column (0.2 m x 0.4 m, E = 1e6 Pa, friction angle 30 deg)
collapses for 0.3 s (30,000 steps of 1e-5 s). Compared, against the FP64
oracle's run (``tests/golden/column_12800_30k.json``, made by
``tests/golden/make_long_horizon.py``) and between the MIXED and FP64 GPU
paths:

* run-out length: front position (largest x of the points) minus the
  column's initial right edge, within 2%;
* free-surface height profile: the highest point in each 1 cm strip, within
  2% of the initial height, from x = 5 cm to the front. The first 5 cm are
  excluded: the column's left side slides against the sticking wall at
  x = 0, where points stop at whatever height they touch it. Two FP64 GPU
  runs of the same scene, differing only in the order of atomic sums, end up
  to 9 cm apart there, but within 1.7 mm (0.4%) everywhere from 5 cm on and
  within 0.3% in run-out.
"""
import json
import os

import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu

X_EDGE = 0.3  # initial right edge of the column (m)
H0 = 0.4      # initial height (m)
FIRST = 5     # first compared strip (x >= 5 cm)
STEPS = 30000
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "column_12800_30k.json")


def profile(q, width=0.01, xmax=1.0):
    bins = np.floor(q[:, 0] / width).astype(int)
    prof = np.zeros(int(round(xmax / width)))
    np.maximum.at(prof, np.clip(bins, 0, len(prof) - 1), q[:, 1])
    return prof


def compare(front_a, prof_a, front_b, prof_b):
    ra, rb = front_a - X_EDGE, front_b - X_EDGE
    assert rb > 0.1, rb  # the column has collapsed
    assert abs(ra - rb) <= 0.02 * rb, (ra, rb)
    d = np.abs(prof_a[FIRST:] - prof_b[FIRST:])
    assert d.max() <= 0.02 * H0, (d.max(), int(d.argmax()) + FIRST)


def run(ctx, precision):
    cfg = scenes.mpm_column("column_12800")
    p = scenes.seed_column_points(cfg)
    m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=precision, capacity=len(p["m"]))
    m.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    for _ in range(STEPS // 1000):
        m.flow(cfg["dt"], 1000)
    assert m.status() == 0
    return m.download()["q"]


@pytest.fixture(scope="module")
def finals(ctx):
    return {"mixed": run(ctx, hg.MIXED), "fp64": run(ctx, hg.FP64)}


@pytest.mark.parametrize("path", ["mixed", "fp64"])
def test_collapse_shape_matches_the_oracle_after_30000_steps(finals, path):
    with open(GOLDEN) as f:
        g = json.load(f)
    assert g["steps"] == STEPS
    q = finals[path]
    compare(q[:, 0].max(), profile(q), g["front_x_m"], np.array(g["profile_top_y_m"]))


def test_mixed_collapse_shape_matches_fp64_after_30000_steps(finals):
    a, b = finals["mixed"], finals["fp64"]
    compare(a[:, 0].max(), profile(a), b[:, 0].max(), profile(b))
