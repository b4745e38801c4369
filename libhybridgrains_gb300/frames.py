"""Frame output with the reference's dataset names, as ``.npz`` files.

The reference writes HDF5 frames (HDF5 is not available here): for MPM the
datasets of SimulationState::writeBinaryState (SimulationState.cpp:145-188)
under a prefix, for DEM those of RigidBody2DSim::writeBinaryState
(RigidBody2DSim.cpp:1365-1427) under ``discrete``. Each frame file here
holds the same names (``<prefix>/q``, ...) as arrays in the reference's
matrix shapes (2 x N for MPM positions and velocities, 3N vectors for DEM
generalised coordinates); file names follow generateOutputFileName
(mpmgrains2d_cli.cpp:47-57): ``<stem>_<frame, zero-padded>.npz``.
"""
import os

import numpy as np

from . import reference_format as rf


def frame_path(directory, frame, width=5, stem="config"):
    return os.path.join(directory, "%s_%0*d.npz" % (stem, width, frame))


def mpm_frame(mpm, cfg, m, volume, hl=None, prefix="mpm", hybrid_factors=None):
    """Datasets of one MPM frame from a device object and the host-held
    masses and volumes: npoints, q, v, m, r (the half widths), J, jhf, the
    grid node positions, masses and hybrid factors (zero unless given), and
    the pressure -tr(sigma) / 2 per point. An empty prefix puts them at the
    file's root, as mpmgrains2d_cli does (writeBinaryState with group "")."""
    st = mpm.download()
    G = mpm.grid()
    n = len(st["q"])
    nx, ny = mpm.nx, mpm.ny
    # PhysicsGrid::computeGridPointLocation: node (i, j) at min + h (i, j),
    # nodes numbered with x fastest
    j, i = np.divmod(np.arange((nx + 1) * (ny + 1)), nx + 1)
    h = cfg["h"]
    nodes = np.stack([mpm.grid_min[0] + h * i, mpm.grid_min[1] + h * j], axis=1).reshape(-1)
    sigma = rf.cauchy_stress(st["be"], st["J"], st["jh"], cfg["shear_modulus"],
                             cfg["bulk_modulus"])
    p = -(sigma[:, 0] + sigma[:, 3]) / 2.0
    hl = np.zeros(n) if hl is None else np.asarray(hl, dtype=np.float64)
    out = {"npoints": np.array(n, dtype=np.uint32), "q": st["q"].T.copy(), "v": st["v"].T.copy(),
           "m": np.asarray(m, dtype=np.float64), "r": hl, "J": st["J"], "jhf": st["jh"],
           "grid_node_positions": nodes, "grid_node_masses": G["mass"],
           "grid_node_hybrid_factors": (np.zeros(len(G["mass"])) if hybrid_factors is None
                                        else np.asarray(hybrid_factors, dtype=np.float64)),
           "p": p}
    return {(prefix + "/" if prefix else "") + k: v for k, v in out.items()}


def dem_frame(dem, radius, mass, fixed=None):
    """Datasets of one DEM frame: discrete/q and v (3N), m (mass and inertia
    per body as 3N, the diagonal of M), kinematically_scripted, unique_index
    and the circle radii under discrete/geometry."""
    q, v = dem.download()
    n = len(q)
    fixed = np.zeros(n, dtype=np.uint8) if fixed is None else np.asarray(fixed, np.uint8)
    radius = np.asarray(radius, dtype=np.float64)
    mass = np.asarray(mass, dtype=np.float64)
    inertia = 0.5 * mass * radius * radius
    return {"discrete/q": q.reshape(-1), "discrete/v": v.reshape(-1),
            "discrete/m": np.stack([mass, mass, inertia], axis=1).reshape(-1),
            "discrete/kinematically_scripted": fixed, "discrete/unique_index":
            np.arange(n, dtype=np.uint32), "discrete/geometry/circle_r": radius}


def write(path, *datasets):
    """One frame file from dicts of datasets."""
    merged = {}
    for d in datasets:
        merged.update(d)
    np.savez(path, **merged)


def read(path):
    with np.load(path) as f:
        return {k: f[k] for k in f.files}
