"""Pins the CPU DEM oracle (test infrastructure): the SpatialGrid candidate set
against its definition, a two-disk known answer, the Coulomb cone
(PenaltyImpactFrictionMap.cpp:684, 834) and momentum conservation."""
import math

import numpy as np
import pytest

import oracle
from libhybridgrains_gb300 import scenes


def brute_pairs(mn, mx):
    n = len(mn)
    out = []
    for i in range(n):
        ov = (mx[i, 0] >= mn[i + 1:, 0]) & (mx[i, 1] >= mn[i + 1:, 1]) & \
             (mx[i + 1:, 0] >= mn[i, 0]) & (mx[i + 1:, 1] >= mn[i, 1])
        for j in np.nonzero(ov)[0]:
            out.append((i, i + 1 + j))
    return np.array(out, dtype=np.int32).reshape(-1, 2)


@pytest.mark.parametrize("cell_scale", [0.5, 1.0, 5.5])
def test_spatial_grid_candidates_equal_overlap_set(cell_scale):
    rng = np.random.default_rng(3)
    n = 600
    c = rng.uniform(0, 0.05, size=(n, 2))
    r = rng.uniform(0.9e-3, 1.1e-3, size=n)
    mn, mx = c - r[:, None], c + r[:, None]
    # exact touching boxes exercise the inclusive comparison
    mn[1] = [mx[0, 0], mn[0, 1]]
    mx[1] = mn[1] + 2e-3
    pairs, h, dims, org = oracle.candidate_pairs(mn, mx, cell_scale)
    assert np.array_equal(pairs, brute_pairs(mn, mx))
    assert h > 0 and dims[0] > 0 and dims[1] > 0


def two_disk_system(v_a, v_b, gap):
    r = np.array([1e-3, 1e-3])
    m = 2600 * math.pi * r * r
    q = np.array([[0.0, 0.0, 0.0], [2e-3 + gap, 0.0, 0.0]])
    v = np.array([[v_a, 0.0, 0.0], [v_b, 0.0, 0.0]])
    return q, v, r, m, 0.5 * m * r * r


def test_two_disk_head_on_known_answer():
    q, v, r, m, I = two_disk_system(0.1, -0.1, -1e-5)
    kn, gn = 1e5, 10.0
    d = oracle.DEM(q, v, r, m, I, [0, 0], (0.0, 0.0), kn, 1e4, gn, gn, 0.5, 1.0)
    dt = 1e-6
    d.step(dt)
    Q, V = d.state()
    # circle-circle: depth = |qa - qb| - 2r; n = (qa - qb)/|qa - qb| = (-1, 0);
    # vrel = va - vb; normal force -kn depth n - gamma_n/2 vn; no friction.
    depth = abs(q[0, 0] - q[1, 0]) - 2e-3
    n = -1.0
    vrel = 0.2
    fn = -kn * 1.0 * depth * n - 0.5 * gn * 1.0 * vrel
    va1 = v[0, 0] + (dt * (1.0 / m[0])) * fn
    vb1 = v[1, 0] + (dt * (1.0 / m[1])) * (-fn)
    assert V[0, 0] == pytest.approx(va1, rel=1e-14)
    assert V[1, 0] == pytest.approx(vb1, rel=1e-14)
    assert Q[0, 0] == pytest.approx(q[0, 0] + dt * va1, abs=1e-18)
    rec = d.contacts()
    assert rec.shape[0] == 1 and rec[0, 0] == 1  # one circle-circle contact
    assert rec[0, 3] == pytest.approx(depth, rel=1e-12)


def test_column_cone_and_momentum():
    sc = scenes.dem_column(n=400, per_row=20)
    p = scenes.dem_params()
    # no gravity, no planes: internal pair forces conserve linear momentum
    rng = np.random.default_rng(1)
    v = sc["v"].copy()
    v[:, :2] = rng.normal(scale=0.05, size=(400, 2))
    d = oracle.DEM(sc["q"], v, sc["r"], sc["m"], sc["I"], sc["fixed"], (0.0, 0.0), p["kn"],
                   p["kt"], p["gamman"], p["gammat"], p["mu"], 1.0)
    p0 = (sc["m"][:, None] * v[:, :2]).sum(axis=0)
    d.step(1e-6, 50)
    Q, V = d.state()
    p1 = (sc["m"][:, None] * V[:, :2]).sum(axis=0)
    assert np.allclose(p0, p1, rtol=0, atol=1e-14)
    rec = d.contacts()
    assert len(rec) > 0
    fn = np.hypot(rec[:, 17], rec[:, 18])
    ft = np.hypot(rec[:, 19], rec[:, 20])
    assert (ft <= p["mu"] * fn * (1 + 1e-9) + 1e-12).all()


def test_fixed_bodies_and_planes():
    sc = scenes.dem_column(n=200, per_row=20)
    fixed = np.zeros(200, dtype=np.uint8)
    fixed[:20] = 1  # bottom row is kinematic
    p = scenes.dem_params()
    v = sc["v"].copy()
    v[20:, 1] = -1.0  # fall onto the fixed row
    d = oracle.DEM(sc["q"], v, sc["r"], sc["m"], sc["I"], fixed, scenes.GRAVITY, p["kn"],
                   p["kt"], p["gamman"], p["gammat"], p["mu"], 1.0)
    d.add_plane((0.0, 0.0), (1.0, 0.0))
    q0 = sc["q"].copy()
    d.step(1e-6, 200)
    Q, V = d.state()
    assert np.array_equal(Q[:20], q0[:20])  # fixed bodies do not move
    kinds = d.contacts()[:, 0]
    assert (kinds == 2).any()  # kinematic circle-circle contacts exist


def test_static_drum_contact_known_answer():
    """StaticDrumCircleConstraint (StaticDrumCircleConstraint.cpp:7-159): a
    disk at rest pressed 0.5 mm into the wall of a drum of radius 0.1 m is
    pushed back towards the drum's centre by kn * 0.5 mm; a disk well inside
    the drum and a fixed disk against the wall have no drum contact."""
    kn = 1.0e5
    r = np.array([0.01, 0.01, 0.01])
    q = np.array([[0.0905, 0.0, 0.0], [0.0, 0.02, 0.0], [-0.0905, 0.0, 0.0]])
    v = np.zeros((3, 3))
    m = 2600.0 * math.pi * r * r
    fixed = np.array([0, 0, 1], dtype=np.uint8)
    d = oracle.DEM(q, v, r, m, 0.5 * m * r * r, fixed, (0.0, 0.0), kn, 0.0, 0.0, 0.0, 0.5, 1.0)
    d.add_drum((0.0, 0.0), 0.1)
    dt = 1e-6
    d.step(dt, 1)
    R = d.contacts()
    assert len(R) == 1
    kind, a, b, depth = R[0, :4]
    assert (kind, a, b) == (3, 0, 0)
    assert depth == pytest.approx(-5e-4, rel=1e-9)
    assert R[0, 4:6].tolist() == [-1.0, 0.0]           # towards the drum's centre
    assert R[0, 15:17] == pytest.approx([0.1005, 0.0])  # the disk's far point
    assert R[0, 10:12] == pytest.approx([0.01, 0.0])    # lever arm -r n
    assert R[0, 17:19] == pytest.approx([-kn * 5e-4, 0.0], rel=1e-9)
    q1, v1 = d.state()
    assert v1[0, 0] == pytest.approx(-dt * kn * 5e-4 / m[0], rel=1e-9)
    assert np.array_equal(v1[1:], np.zeros((2, 3)))
