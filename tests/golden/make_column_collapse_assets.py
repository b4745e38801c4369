"""Writes the column-collapse hybrid scene of the reference's assets
(assets/hybridgrains2dnew/column-collapse/{hybrid,mpm,dem}.xml) as test
inputs:

* column_collapse_dem.npz: the 6,694 disks (x, y, theta, r, fixed), in file
  order;
* column_collapse_scene.json: the MPM grid, material, rectangle and planes,
  the DEM penalty parameters and the hybrid (zone / resampling) settings.

Run from the repository root where the reference checkout is available,
naming it as the argument or in $HG_REFERENCE_ROOT:

    python tests/golden/make_column_collapse_assets.py <reference_root>
"""
import json
import os
import sys
import xml.etree.ElementTree as ET

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def nums(s):
    return [float(v) for v in s.split()]


def frac(s):
    # "1 / 1000080" style time steps
    if "/" in s:
        a, b = s.split("/")
        return float(a) / float(b)
    return float(s)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HG_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_column_collapse_assets.py <reference_root> "
                 "(or set HG_REFERENCE_ROOT)")
    d = os.path.join(root, "assets", "hybridgrains2dnew", "column-collapse")
    dem = ET.parse(os.path.join(d, "dem.xml")).getroot()
    geo = [float(g.get("r")) for g in dem.findall("geometry")]
    bodies = dem.findall("rigid_body")
    x = np.array([nums(b.get("x")) for b in bodies])
    theta = np.array([float(b.get("theta")) for b in bodies])
    r = np.array([geo[int(b.get("geo_idx"))] for b in bodies])
    fixed = np.array([int(b.get("fixed")) for b in bodies], dtype=np.uint8)
    rho = np.array([float(b.get("rho")) for b in bodies])
    np.savez_compressed(os.path.join(HERE, "column_collapse_dem.npz"), x=x[:, 0], y=x[:, 1],
                        theta=theta, r=r, fixed=fixed, rho=rho)
    mpm = ET.parse(os.path.join(d, "mpm.xml")).getroot()
    hyb = ET.parse(os.path.join(d, "hybrid.xml")).getroot()
    grid = mpm.find("grid")
    mat = mpm.find("material")
    rect = mpm.find("rectangle")
    integ = mpm.find("integrator")
    pen = dem.find("penalty_impact_map")
    cf = hyb.find("coupling_force")
    scene = {
        "mpm": {"grid_min": nums(grid.get("min")), "grid_max": nums(grid.get("max")),
                "cell_width": float(grid.get("cell_width")),
                "shear_modulus": float(mat.get("shear_modulus")),
                "bulk_modulus": float(mat.get("bulk_modulus")), "dp_alpha": float(mat.get("alpha")),
                "flip_alpha": float(integ.get("alpha")), "basis": integ.get("shape_function_category"),
                "rect_min": nums(rect.get("min")), "rect_max": nums(rect.get("max")),
                "density": float(rect.get("density")),
                "samples_per_dim": int(rect.get("cell_samples_per_dim")),
                "gravity": nums(mpm.find("near_earth_gravity").get("f")),
                "planes": [{"x": nums(p.get("x")), "n": nums(p.get("n")),
                            "sticking": p.get("boundary_behavior") == "sticking"}
                           for p in mpm.findall("static_plane")]},
        "dem": {"kn": float(pen.get("kn")), "kt": float(pen.get("kt")),
                "gamman": float(pen.get("gamman")), "gammat": float(pen.get("gammat")),
                "mu": float(pen.get("mu")), "dt": frac(pen.get("dt")),
                "cell_scale": float(dem.find("collision_detection").get("cell_scale")),
                "gravity": nums(dem.find("near_earth_gravity").get("f")),
                "planes": [{"x": nums(p.get("x")), "n": nums(p.get("n"))}
                           for p in dem.findall("static_plane")]},
        "hybrid": {"dt": frac(hyb.find("time_step").get("dt")),
                   "rzone_half_thickness": float(cf.get("rzoneHalfThickness")),
                   "dem_r_mean": float(cf.get("demRMean")), "dem_r_std": float(cf.get("demRStd")),
                   "avoid_a_void_freq": int(cf.get("avoidAVoidFreq")),
                   "phi_threshold": float(cf.get("phiThreshold")),
                   "rzone_level_set": float(cf.get("rzoneLevelSet")),
                   "phi_window_size": float(cf.get("phi_window_size")),
                   "phi_samples_per_cell_side": int(cf.get("phi_samples_per_cell_side")),
                   "level_set_cell_width": float(cf.get("level_set_cell_width")),
                   "rho_dem": float(cf.get("rho_dem")),
                   "homogenize_stress": int(cf.get("homogenize_stress", "0")) != 0,
                   "homogenize_velocity": int(cf.get("homogenize_velocity", "0")) != 0,
                   "end_time": float(hyb.find("end_time").get("t"))},
    }
    with open(os.path.join(HERE, "column_collapse_scene.json"), "w") as f:
        json.dump(scene, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
