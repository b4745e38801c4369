"""Synthetic scenes with the shapes of the benchmark configurations.

* ``mpm_column``   - granular column on a floor between walls (MPM configs:
                     1.0 x 0.5 m domain at h = 5 mm with a 0.2 x 0.4 m column,
                     12,800 points; or 2048 x 1024 cells at h = 1 mm with a
                     1.0 x 0.5 m column, 2,000,000 points).
* ``dem_column``   - disks on a jittered hex lattice (10,000 disks, radii
                     U[0.9, 1.1] mm, pitch 2.2 mm, 100 per row).

Material constants follow the configuration text: E = 1e6 Pa, nu = 0.3,
rho = 1550 kg/m^3, friction angle 30 deg. The Drucker-Prager coefficient used
for a friction angle phi is alpha = sqrt(2/3) * 2 sin(phi) / (3 - sin(phi))
(the reference takes alpha directly as a material input, so this mapping is a
choice of this project). PIC/FLIP alpha = 0.999 as in the reference assets.
Random numbers come from splitmix64 with the stated seed.
"""
import math

import numpy as np

GRAVITY = (0.0, -9.81)


def elastic_moduli(E, nu):
    """(shear, bulk) moduli of a plane-strain solid."""
    return E / (2.0 * (1.0 + nu)), E / (3.0 * (1.0 - 2.0 * nu))


def dp_alpha(phi_deg):
    s = math.sin(math.radians(phi_deg))
    return math.sqrt(2.0 / 3.0) * 2.0 * s / (3.0 - s)


def splitmix64(seed, n):
    """n uniform doubles in [0, 1) from splitmix64 (53-bit mantissas)."""
    out = np.empty(n, dtype=np.float64)
    x = seed & 0xFFFFFFFFFFFFFFFF
    mask = 0xFFFFFFFFFFFFFFFF
    for i in range(n):
        x = (x + 0x9E3779B97F4A7C15) & mask
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z = z ^ (z >> 31)
        out[i] = (z >> 11) * (1.0 / 9007199254740992.0)
    return out


MPM_CONFIGS = {
    # 12,800 points: 1.0 x 0.5 m domain, h = 5 mm, column 0.2 x 0.4 m at x = 0.1
    "column_12800": dict(grid_min=(0.0, 0.0), grid_max=(1.0, 0.5), h=5.0e-3,
                         rect_min=(0.1, 0.0), rect_max=(0.3, 0.4), dt=1.0e-5, steps=1000),
    # 2,000,000 points: 2048 x 1024 cells at h = 1 mm, column 1.0 x 0.5 m
    "column_2M": dict(grid_min=(0.0, 0.0), grid_max=(2.048, 1.024), h=1.0e-3,
                      rect_min=(0.0, 0.0), rect_max=(1.0, 0.5), dt=2.0e-6, steps=500),
}


def mpm_material(E=1.0e6, nu=0.3, phi_deg=30.0, rho=1550.0):
    mu, kappa = elastic_moduli(E, nu)
    return dict(shear_modulus=mu, bulk_modulus=kappa, dp_alpha=dp_alpha(phi_deg),
                flip_alpha=0.999, rho=rho)


def mpm_planes(grid_min, grid_max):
    """Sticking floor and walls (MPMStaticPlane STICKING)."""
    return [((grid_min[0], grid_min[1]), (0.0, 1.0), True, -np.inf),
            ((grid_min[0], grid_min[1]), (1.0, 0.0), True, -np.inf),
            ((grid_max[0], grid_min[1]), (-1.0, 0.0), True, -np.inf)]


def mpm_column(name="column_12800", **overrides):
    """Configuration dict for an MPM column scene (geometry, material, planes)."""
    cfg = dict(MPM_CONFIGS[name])
    cfg.update(mpm_material())
    cfg.update(overrides)
    cfg["planes"] = mpm_planes(cfg["grid_min"], cfg["grid_max"])
    cfg["samples_per_dim"] = 2
    return cfg


def seed_column_points(cfg):
    """rasterizeRectangle (mpmgrains2d/InitialSimulationState.cpp:48-145) in numpy.

    Same formula and filters as the reference (and as hg_mpm_seed_rectangle),
    for hosts that build scenes without a device.
    """
    gmin, gmax, h = cfg["grid_min"], cfg["grid_max"], cfg["h"]
    # PhysicsGrid::setDimensions
    cx, cy = 0.5 * (gmin[0] + gmax[0]), 0.5 * (gmin[1] + gmax[1])
    nx, ny = math.ceil((gmax[0] - gmin[0]) / h), math.ceil((gmax[1] - gmin[1]) / h)
    g0 = (cx - 0.5 * (nx * h), cy - 0.5 * (ny * h))
    rmin, rmax, npd = cfg["rect_min"], cfg["rect_max"], cfg["samples_per_dim"]
    bx0, by0 = math.floor((rmin[0] - g0[0]) / h), math.floor((rmin[1] - g0[1]) / h)
    bx1, by1 = math.ceil((rmax[0] - g0[0]) / h), math.ceil((rmax[1] - g0[1]) / h)
    gx = np.arange(bx0, bx1, dtype=np.float64)
    gy = np.arange(by0, by1, dtype=np.float64)
    off = (np.arange(npd, dtype=np.float64) + 0.5) / float(npd)
    # loop order gy, gx, cy, cx
    px = g0[0] + h * (gx[None, :, None, None] + off[None, None, None, :])
    py = g0[1] + h * (gy[:, None, None, None] + off[None, None, :, None])
    px, py = np.broadcast_arrays(px, py)
    px, py = px.ravel(), py.ravel()
    keep = (px >= rmin[0]) & (py >= rmin[1]) & (px <= rmax[0]) & (py <= rmax[1])
    for (x, n, _st, lb) in cfg["planes"]:
        nn = math.hypot(n[0], n[1])
        d = (n[0] / nn) * (px - x[0]) + (n[1] / nn) * (py - x[1])
        # pointInsidePlane is evaluated plane by plane with early exits; with
        # -inf lower bounds it reduces to "strictly behind any plane".
        keep &= ~((py >= lb) & (d < 0.0))
    px, py = px[keep], py[keep]
    half = 0.5 * h / float(npd)
    vol = half * half * 4.0
    n = px.size
    return dict(q=np.stack([px, py], axis=1), v=np.zeros((n, 2)),
                m=np.full(n, cfg["rho"] * vol), vol=np.full(n, vol), hl=np.full(n, half))


# ---- DEM ------------------------------------------------------------------------

def dem_column(n=10000, per_row=100, pitch=2.2e-3, rmin=0.9e-3, rmax=1.1e-3, jitter=0.05e-3,
               rho=2600.0, seed=12345, x0=0.0, y0=0.0):
    """Disks on a hex lattice with seeded radius and position jitter.

    Returns q, v as (N, 3), radii, masses (rho pi r^2) and inertias (m r^2 / 2,
    rigidbody2d/CircleGeometry.cpp:44-48).
    """
    u = splitmix64(seed, 3 * n)
    r = rmin + (rmax - rmin) * u[:n]
    k = np.arange(n)
    row, col = k // per_row, k % per_row
    x = x0 + pitch * (col + 0.5 + 0.5 * (row % 2)) + jitter * (2.0 * u[n:2 * n] - 1.0)
    y = y0 + pitch * (0.5 + row * math.sqrt(3.0) / 2.0) + jitter * (2.0 * u[2 * n:] - 1.0)
    q = np.stack([x, y, np.zeros(n)], axis=1)
    v = np.zeros((n, 3))
    m = rho * math.pi * r * r
    I = 0.5 * m * r * r
    return dict(q=q, v=v, r=r, m=m, I=I, fixed=np.zeros(n, dtype=np.uint8))


def dem_packed(n=10000, per_row=100, pitch=1.9e-3, seed=12345):
    """The DEM column's disks (radii U[0.9, 1.1] mm, jitter 0.05 mm, rho 2600)
    on a hex lattice compacted to a pitch below the mean diameter, between a
    floor and two walls: about 2.5 contacts per disk from the first step (the
    loose 2.2 mm lattice has about 0.03). The planes (floor at y = 0, walls
    at x = 0 and x = (per_row + 1/2) pitch) are returned with the bodies; the
    walls keep the lattice compacted across its width while the top relaxes."""
    sc = dem_column(n=n, per_row=per_row, pitch=pitch, seed=seed)
    sc["planes"] = [((0.0, 0.0), (0.0, 1.0)), ((0.0, 0.0), (1.0, 0.0)),
                    (((per_row + 0.5) * pitch, 0.0), (-1.0, 0.0))]
    return sc


def dem_params(kn=1.0e5, mu=0.5, restitution=0.5, r_mean=1.0e-3, rho=2600.0):
    """Penalty parameters: restitution-matched normal damping for the mean disk.

    The reference applies 0.5 * gamma in the force law
    (PenaltyImpactFrictionMap.cpp:641-645), so gamma_n = 2 c with
    c = 2 sqrt(m_eff k) ln(1/e) / sqrt(pi^2 + ln(e)^2), m_eff = m / 2.
    kt = 2/7 kn, gamma_t = gamma_n.
    """
    m = rho * math.pi * r_mean * r_mean
    le = math.log(restitution)
    c = 2.0 * math.sqrt(0.5 * m * kn) * (-le) / math.sqrt(math.pi ** 2 + le * le)
    gn = 2.0 * c
    return dict(kn=kn, kt=2.0 / 7.0 * kn, gamman=gn, gammat=gn, mu=mu)


def serving_column(npoints, aspect, phi_deg, h=5.0e-3):
    """A granular-column collapse of about npoints material points (2 x 2 per
    cell) whose height/width ratio is aspect, on a domain long enough for the
    run-out; friction angle phi_deg. Used for mixes of many small scenes."""
    cells = max(npoints / 4.0, 4.0)
    wc = max(int(round(math.sqrt(cells / aspect))), 2)
    hc = max(int(round(cells / wc)), 2)
    nx, ny = wc + 2 * hc + 8, hc + 8
    cfg = dict(grid_min=(0.0, 0.0), grid_max=(nx * h, ny * h), h=h,
               rect_min=(2 * h, 0.0), rect_max=((2 + wc) * h, hc * h), dt=1.0e-5)
    cfg.update(mpm_material(phi_deg=phi_deg))
    cfg["planes"] = mpm_planes(cfg["grid_min"], cfg["grid_max"])
    cfg["samples_per_dim"] = 2
    return cfg


def hybrid_column(scale=1.0, seed=12345):
    """The hybrid column collapse (MPM bulk under a DEM layer).

    scale=1: 100,000 material points (h = 2.5 mm, 2 x 2 per cell, a column
    0.25 m wide and 0.625 m tall) under 20,000 disks (r U[0.9, 1.1] mm, hex
    pitch 2.2 mm, 113 per row) that start 10 mm (four cells) below the top
    of the bulk, so the coupling band is four cells wide; resampling every
    200 steps, dt = 1e-6 s. The disk count does not fit a 10 mm band on this
    column, so the layer is as tall as the count needs (about 0.34 m). scale
    < 1 shrinks both counts (column and layer widths by sqrt(scale)) for
    tests. Zone settings are the reference's column-collapse ones in units
    of the cell width and mean radius."""
    h = 2.5e-3
    wc = max(int(round(100 * math.sqrt(scale))), 8)
    hc = max(int(round(250 * math.sqrt(scale))), 8)
    # the grid extends four cells past the floor and the left wall: uGIMP
    # stencils of points within half a sample of a wall then stay on the grid
    nx, ny = 404, 404
    cfg = dict(grid_min=(-4 * h, -4 * h), grid_max=(400 * h, 400 * h), h=h,
               rect_min=(0.0, 0.0), rect_max=(wc * h, hc * h), dt=1.0e-6)
    cfg.update(mpm_material())
    cfg["planes"] = [((0.0, 0.0), (0.0, 1.0), True, -np.inf),
                     ((0.0, 0.0), (1.0, 0.0), True, -np.inf),
                     ((396 * h, 0.0), (-1.0, 0.0), True, -np.inf)]
    cfg["samples_per_dim"] = 2
    per_row = max(int((wc * h) / 2.2e-3), 4)
    n_disks = int(round(20000 * scale))
    sc = dem_column(n=n_disks, per_row=per_row, pitch=2.2e-3, seed=seed, x0=0.0,
                    y0=hc * h - 4 * h)
    dp = dem_params()
    zones = dict(level_set_cell_width=h, phi_window_size=4.35e-3, phi_samples_per_cell_side=1,
                 phi_threshold=0.3, rzone_level_set=6.25 * h, rzone_half_thickness=0.5 * h,
                 allow_direct_transitions=False)
    res = dict(dem_r_mean=1.0e-3, dem_r_std=0.1e-3, rho_dem=2600.0, avoid_a_void_freq=200,
               homogenize_stress=True, homogenize_velocity=True,
               newly_inserted_continuum_stress_free=False)
    return dict(mpm=cfg, dem=sc, dem_params=dp, zones=zones, resampling=res)
