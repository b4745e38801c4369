"""Zone labels of the hybrid method (ZoneTools) in libhg_gpu's host code
against the oracle, and the oracle's disk/box area against the reference's
own compiled function (oracle/_ref, built from the reference sources where a
checkout is present).

Everything here is bit-exact: packing fractions, signed distances, level-set
and MPM cell labels, zone lists, deletion lists and weights are FP64 results
that feed threshold tests, so they must agree to the last bit. Inputs are the
reference's column-collapse hybrid scene (tests/golden/column_collapse_*,
made by tests/golden/make_column_collapse_assets.py): 6,694 disks of the
settled column, with and without a block of MPM points, over successive
updates so that the hysteresis on the previous labels is exercised.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def asset():
    with open(os.path.join(GOLDEN, "column_collapse_scene.json")) as f:
        sc = json.load(f)
    d = np.load(os.path.join(GOLDEN, "column_collapse_dem.npz"))
    q = np.stack([d["x"], d["y"], d["theta"]], axis=1)
    return sc, q, d["r"], d["fixed"]


def mpm_grid(sc):
    """PhysicsGrid::setDimensions: cell counts and the centred minimum."""
    m = sc["mpm"]
    lo, hi, h = m["grid_min"], m["grid_max"], m["cell_width"]
    cells = [math.ceil((hi[a] - lo[a]) / h) for a in range(2)]
    gmin = [0.5 * (lo[a] + hi[a]) - 0.5 * (cells[a] * h) for a in range(2)]
    return gmin, h, cells


def pair(sc, allow_direct):
    gmin, h, cells = mpm_grid(sc)
    hy = sc["hybrid"]
    args = (hy["level_set_cell_width"], hy["phi_window_size"], hy["phi_samples_per_cell_side"],
            hy["phi_threshold"], hy["rzone_level_set"], hy["rzone_half_thickness"])
    ours = hg.Zones(gmin, h, cells, *args, allow_direct_transitions=allow_direct)
    ref = oracle.Zones(gmin, h, cells, hy["level_set_cell_width"], allow_direct)
    return ours, ref, hy


def update_both(ours, ref, hy, q, r, fixed, pts):
    ours.update(q, r, fixed, pts)
    ref.update(q, r, fixed, pts, hy["phi_window_size"], hy["phi_samples_per_cell_side"],
               hy["phi_threshold"], hy["rzone_level_set"], hy["rzone_half_thickness"])


def same_fields(ours, ref):
    a, b = ours.fields(), ref.fields()
    for k in ("phi", "dist", "ls", "mpm"):
        assert np.array_equal(a[k], b[k]), k
    return a


def block(x0, x1, y0, y1, h, n=2):
    """Material points on the reference lattice of a rectangle."""
    xs = x0 + h * (np.arange(int(round((x1 - x0) / h)))[:, None] + (np.arange(n) + 0.5) / n)
    ys = y0 + h * (np.arange(int(round((y1 - y0) / h)))[:, None] + (np.arange(n) + 0.5) / n)
    X, Y = np.meshgrid(xs.ravel(), ys.ravel())
    return np.stack([X.ravel(), Y.ravel()], axis=1)


def test_disk_box_area_matches_the_reference_function():
    rng = np.random.default_rng(5)
    cases = [(-1.0, 1.0, -1.0, 1.0, 0.0, 0.0, 0.5), (-0.1, 0.1, -0.1, 0.1, 0.0, 0.0, 1.0),
             (2.0, 3.0, 2.0, 3.0, 0.0, 0.0, 1.0), (0.0, 1.0, 0.0, 1.0, 0.0, 0.0, 1.0),
             (-1.0, 1.0, 0.3, 0.3, 0.0, 0.0, 1.0), (1.0, -1.0, 1.0, -1.0, 0.2, -0.1, 0.7)]
    for _ in range(2000):
        c = rng.uniform(-1, 1, 2)
        x = np.sort(rng.uniform(-1.5, 1.5, 2))
        y = np.sort(rng.uniform(-1.5, 1.5, 2))
        cases.append((x[0], x[1], y[0], y[1], c[0], c[1], rng.uniform(0.01, 1.0)))
    ref = oracle.reference_lib()
    for cs in cases:
        a = hg.disk_box_area(*cs)
        b = oracle.disk_box_area(*cs)
        assert a == b, cs
        if ref is not None:
            assert ref.hgr_circle_rectangle_area(*cs) == b, cs
    # the full disk inside a box
    assert abs(hg.disk_box_area(-2, 2, -2, 2, 0, 0, 1) - math.pi) < 1e-14


@pytest.mark.parametrize("allow_direct", [False, True])
def test_labels_of_the_settled_column_match_the_oracle(asset, allow_direct):
    sc, q, r, fixed = asset
    ours, ref, hy = pair(sc, allow_direct)
    update_both(ours, ref, hy, q, r, fixed, None)
    f = same_fields(ours, ref)
    assert ours.boundary_samples() == ref.samples() > 0
    assert (f["mpm"] == hg.DISCRETE).any() and (f["mpm"] == hg.HYBRID).any()
    # a second update starts from the first one's labels
    update_both(ours, ref, hy, q, r, fixed, None)
    same_fields(ours, ref)


@pytest.mark.parametrize("allow_direct", [False, True])
def test_labels_with_material_points_and_hysteresis(asset, allow_direct):
    sc, q, r, fixed = asset
    ours, ref, hy = pair(sc, allow_direct)
    h = sc["mpm"]["cell_width"]
    seen = set()
    for k, shift in enumerate((0.0, 1.3, 2.9, 4.1)):
        # disks left of x = 7, material points in a block that moves right
        keep = q[:, 0] < 7.0 - 0.5 * shift
        pts = block(6.0 + shift, 14.0 + shift, 0.0, 5.2, h)
        update_both(ours, ref, hy, q[keep], r[keep], fixed[keep], pts)
        f = same_fields(ours, ref)
        seen.update(np.unique(f["mpm"]).tolist())
        for which in range(4):
            ba, ca = ours.zone_list(which)
            bb, cb = ref.zone_list(which)
            assert np.array_equal(ba, bb) and np.array_equal(ca, cb), (k, which)
        assert np.array_equal(ours.to_delete(hg.ZONES_MPM, pts, 2),
                              ref.to_delete(0, pts, 2))
        assert np.array_equal(ours.to_delete(hg.ZONES_DEM, q, 3, fixed),
                              ref.to_delete(1, q, 3, fixed))
        assert np.array_equal(ours.weights(hg.ZONES_MPM, pts, 2), ref.weights(0, pts, 2))
        assert np.array_equal(ours.weights(hg.ZONES_DEM, q, 3), ref.weights(1, q, 3))
    assert seen == {hg.CONTINUUM, hg.DISCRETE, hg.HYBRID}


def test_set_labels_feeds_the_hysteresis(asset):
    sc, q, r, fixed = asset
    ours, ref, hy = pair(sc, False)
    labels = np.full(ours.mpm_cells[0] * ours.mpm_cells[1], hg.CONTINUUM, dtype=np.int32)
    ours.set_labels(labels)
    ref.set_labels(labels)
    update_both(ours, ref, hy, q, r, fixed, None)
    f = same_fields(ours, ref)
    # cells that were continuum cannot turn discrete without passing hybrid
    assert not (f["mpm"] == hg.DISCRETE).any()


def test_coarse_level_set_is_rejected(asset):
    sc, _, _, _ = asset
    gmin, h, cells = mpm_grid(sc)
    with pytest.raises(hg.HGError):
        hg.Zones(gmin, h, cells, 2 * h, 0.25, 1, 0.3, 1.25, 0.1)
