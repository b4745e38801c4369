"""The FP32 bounds of the DEM pair search against the reference's FP64 tests.

The counting and emission passes decide a candidate pair from FP32 offsets of
the centres from their home cells' corners: no contact when the FP32 distance
exceeds ra + rb + tol, a contact when it is below ra + rb - tol (tol = 1e-4 of
the cell width), and the reference's FP64 AABB and c0 tests in between
(SpatialGrid.cpp:14-19, CircleGeometry.cpp:22-30, ballBallCCDCollisionHappens
with q0 == q1). This restates that arithmetic in numpy (float32 operations
rounded one by one, as an upper bound on the kernel's error, which may fuse a
multiply-add) on pairs placed within a few tol of the contact distance, far
from the origin, and checks that neither bound ever disagrees with FP64.
"""
import numpy as np


def fp32_bounds(xa, ya, ra, xb, yb, rb, H):
    Hf, tol = np.float32(H), np.float32(1.0e-4 * H)

    def home(x, y, r):
        cx, cy = np.floor((x - r) / H), np.floor((y - r) / H)
        return cx, cy, np.float32(x - cx * H), np.float32(y - cy * H), np.float32(r)

    cxa, cya, pax, pay, raf = home(xa, ya, ra)
    cxb, cyb, pbx, pby, rbf = home(xb, yb, rb)
    dx, dy = (cxb - cxa).astype(np.float32), (cyb - cya).astype(np.float32)
    ex = dx * Hf + (pbx - pax)
    ey = dy * Hf + (pby - pay)
    d2 = ex * ex + ey * ey
    outer, inner = raf + rbf + tol, raf + rbf - tol
    return d2 > outer * outer, (inner > 0) & (d2 < inner * inner), np.abs(dx) <= 1


def fp64_contact(xa, ya, ra, xb, yb, rb):
    aabb = (xa + ra >= xb - rb) & (ya + ra >= yb - rb) & (xb + rb >= xa - ra) & (yb + rb >= ya - ra)
    ddx, ddy = xa - xb, ya - yb
    c0 = (ddx * ddx + ddy * ddy) - (ra + rb) * (ra + rb)
    return aabb & (c0 <= 0.0)


def test_fp32_bounds_never_contradict_fp64():
    rng = np.random.default_rng(7)
    n = 2_000_000
    H = 2.2e-3
    tol = 1.0e-4 * H
    ra = rng.uniform(0.9e-3, 1.1e-3, n)
    rb = rng.uniform(0.9e-3, 1.1e-3, n)
    xa = rng.uniform(-100.0, 100.0, n)
    ya = rng.uniform(-100.0, 100.0, n)
    # distances within 3 tol of contact, some exactly at the FP32 bounds' slack
    u = rng.uniform(-3.0, 3.0, n)
    u[: n // 10] = rng.choice([-1.0, 1.0], n // 10)
    d = ra + rb + u * tol
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    xb, yb = xa + d * np.cos(phi), ya + d * np.sin(phi)
    reject, accept, adjacent = fp32_bounds(xa, ya, ra, xb, yb, rb, H)
    truth = fp64_contact(xa, ya, ra, xb, yb, rb)
    assert adjacent.all()
    assert not (reject & truth).any()  # the outer bound drops no contact
    assert not (accept & ~truth).any()  # the inner bound adds none
    band = ~reject & ~accept
    # the band is about 2 tol wide: only those pairs take the FP64 tests
    assert 0.2 < band.mean() < 0.45
    assert accept[u < -1.01].all() and reject[u > 1.01].all()


def test_dense_packing_decides_almost_all_in_fp32():
    rng = np.random.default_rng(3)
    n = 200_000
    H = 2.2e-3
    ra = rng.uniform(0.9e-3, 1.1e-3, n)
    rb = rng.uniform(0.9e-3, 1.1e-3, n)
    xa, ya = rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    d = np.full(n, 1.9e-3)  # neighbours of a 1.9 mm hex lattice
    xb, yb = xa + d * np.cos(phi), ya + d * np.sin(phi)
    reject, accept, _ = fp32_bounds(xa, ya, ra, xb, yb, rb, H)
    truth = fp64_contact(xa, ya, ra, xb, yb, rb)
    assert not (accept & ~truth).any() and not (reject & truth).any()
    assert (accept | reject).mean() > 0.998  # the band (2 tol of ra + rb) is rare
