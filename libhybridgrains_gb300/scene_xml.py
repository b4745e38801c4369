"""The reference's scene files (XML), read into this library's objects.

Three readers follow the reference's parsers for the elements on the
per-step path:

* ``read_mpm``: ``<mpmgrains2d>`` (mpmgrains2dutils/MPMGrains2DParser.cpp):
  grid, integrator (dt as a rational, PIC/FLIP alpha, basis order and
  category), material, rectangles of material points, static planes,
  gravity and the end time;
* ``read_dem``: ``<rigidbody2d_scene>`` with circle bodies and the penalty
  impact-friction map (rigidbody2dutils/RigidBody2DSceneParser.cpp):
  geometry, rigid bodies, static planes, gravity, collision detection and
  the end time;
* ``read_hybrid``: ``<hybridgrains2d_scene>``
  (hybridgrains2dnewutils/HybridGrains2DSceneParser.cpp): the two files
  above, the time step and the coupling_force (zone and resampling)
  settings, as the scene dict ``hybrid.HybridSim`` takes.

Numbers are read the way the reference reads them: the first token of an
attribute for a scalar (``std::stringstream >> x``), exactly n tokens for a
list, ``inf``/``-inf`` accepted in lists, and time steps as exact rationals
("1 / 1000080", "0.000001") converted by one division. Elements that only
drive the reference's viewers (camera, cairo_settings) or its Python hooks
(scripting) are ignored. Features outside this library's path (box and
annulus bodies, portals, cubic basis functions, other hybrid
integrator styles) raise ``SceneError`` naming the element, where the
reference's parser would accept them.

``make_mpm``, ``make_dem`` build and upload the device objects; material
points are seeded from the rectangles by ``seed_points``
(InitialSimulationState.cpp:33-145).
"""
import math
import os
import re
import xml.etree.ElementTree as ET
from fractions import Fraction

import numpy as np


class SceneError(ValueError):
    """A scene file that the reference's parser rejects, or that uses a
    feature outside this library's path."""


def _root(source, tag):
    """Parses a path or XML text and checks the root element's tag."""
    text = source
    if not source.lstrip().startswith("<"):
        with open(source, "r") as f:
            text = f.read()
    try:
        root = ET.fromstring(text)
    except ET.ParseError as e:
        raise SceneError("malformed XML: %s" % e) from None
    if root.tag != tag:
        raise SceneError("root node %s not found (found %s)" % (tag, root.tag))
    return root


def _attr(node, name, required=True):
    v = node.get(name)
    if v is None and required:
        raise SceneError("%s: attribute %s missing" % (node.tag, name))
    return v


def _scalar(node, name, required=True, default=None):
    """StringUtilities::extractFromString: the first token as a scalar."""
    v = _attr(node, name, required)
    if v is None:
        return default
    tok = v.split()
    try:
        return float(tok[0])
    except (IndexError, ValueError):
        raise SceneError("%s: %s must be a scalar (got %r)" % (node.tag, name, v)) from None


def _int(node, name, required=True, default=None):
    """The first token as an integer (a stream reads the integer prefix)."""
    v = _attr(node, name, required)
    if v is None:
        return default
    tok = v.split()
    digits = ""
    if tok:
        t = tok[0]
        k = 1 if t[:1] in "+-" else 0
        while k < len(t) and t[k].isdigit():
            k += 1
        digits = t[:k]
    try:
        return int(digits)
    except ValueError:
        raise SceneError("%s: %s must be an integer (got %r)" % (node.tag, name, v)) from None


def _list(node, name, n, required=True):
    """StringUtilities::readScalarList: exactly n scalars."""
    v = _attr(node, name, required)
    if v is None:
        return None
    tok = v.split()
    if len(tok) != n:
        raise SceneError("%s: %s must hold %d scalars (got %r)" % (node.tag, name, n, v))
    try:
        return tuple(float(t) for t in tok)
    except ValueError:
        raise SceneError("%s: %s must hold %d scalars (got %r)" % (node.tag, name, n, v)) from None


_FRACTION = re.compile(r"^\s*([+-]?\d+)\s*/\s*([+-]?\d+)\s*$")
_DECIMAL = re.compile(r"^\s*([+-]?)(\d*)(?:\.(\d*))?\s*$")


def rational(text):
    """RationalTools::extractFromString (scisim/Math/Rational.h): "a / b",
    a decimal or an integer as an exact fraction. Forms that parser would
    misread (exponents: "1e-06" reads as 1) are rejected."""
    m = _FRACTION.match(text)
    if m:
        if int(m.group(2)) == 0:
            raise SceneError("not a rational number: %r" % text)
        return Fraction(int(m.group(1)), int(m.group(2)))
    m = _DECIMAL.match(text)
    if not m or not (m.group(2) or m.group(3)):
        raise SceneError("not a rational number: %r" % text)
    whole, frac_digits = m.group(2) or "0", m.group(3) or ""
    r = Fraction(int(whole + frac_digits), 10 ** len(frac_digits))
    return -r if m.group(1) == "-" else r


def _time(node, name):
    """A positive rational attribute and its double value (numerator /
    denominator in one division, as scalar(Rational) does)."""
    r = rational(_attr(node, name))
    if r <= 0:
        raise SceneError("%s: %s must be positive" % (node.tag, name))
    return r, float(r.numerator) / float(r.denominator)


# ---- mpmgrains2d ------------------------------------------------------------------

def read_mpm(source):
    """MPMGrains2DParser::readXMLFile (MPMGrains2DParser.cpp:660-683).

    Returns the scene as a dict: grid_min, grid_max, h; shear_modulus,
    bulk_modulus, dp_alpha; flip_alpha, dt (and dt_rational, dt_string),
    basis ("linear" or "ugimp"); rectangles (min, max, density,
    samples_per_dim, vel, omega per region, in file order); planes as
    (x, n, sticking, lower_bound); gravity; end_time (inf when absent).
    The first rectangle's geometry is also given as rect_min, rect_max, rho
    and samples_per_dim, the keys of the library's column scenes.
    """
    root = _root(source, "mpmgrains2d")
    cfg = {}
    # loadMaterialPointRectangles (:225-346)
    rects = []
    for nd in root.findall("rectangle"):
        lo, hi = _list(nd, "min", 2), _list(nd, "max", 2)
        if lo[0] >= hi[0] or lo[1] >= hi[1]:
            raise SceneError("rectangle: max must be greater than min")
        rho = _scalar(nd, "density")
        if not rho > 0.0:
            raise SceneError("rectangle: density must be positive")
        spd = _int(nd, "cell_samples_per_dim")
        if spd < 0:
            raise SceneError("rectangle: cell_samples_per_dim must be non-negative")
        rects.append(dict(min=lo, max=hi, density=rho, samples_per_dim=spd,
                          vel=_list(nd, "vel", 2), omega=_scalar(nd, "omega")))
    # loadMaterialSettings (:438-527)
    mat = root.find("material")
    if mat is None:
        raise SceneError("material node missing")
    for key, name in (("shear_modulus", "shear_modulus"), ("bulk_modulus", "bulk_modulus"),
                      ("dp_alpha", "alpha")):
        cfg[key] = _scalar(mat, name)
        if cfg[key] < 0.0:
            raise SceneError("material: %s must be non-negative" % name)
    # loadGridSettings (:529-600)
    grid = root.find("grid")
    if grid is None:
        raise SceneError("grid node missing")
    gmin, gmax = _list(grid, "min", 2), _list(grid, "max", 2)
    h = _scalar(grid, "cell_width")
    if not h > 0.0:
        raise SceneError("grid: cell_width must be positive")
    if gmax[0] <= gmin[0] or gmax[1] <= gmin[1]:
        raise SceneError("grid: minimum must be less than maximum")
    cfg.update(grid_min=gmin, grid_max=gmax, h=h)
    # loadIntegrator (:80-200)
    integ = root.find("integrator")
    if integ is None:
        raise SceneError("integrator node missing")
    dt_r, dt = _time(integ, "dt")
    alpha = _scalar(integ, "alpha")
    if not 0.0 <= alpha <= 1.0:
        raise SceneError("integrator: alpha must lie in [0, 1]")
    order = _int(integ, "shape_function_order")
    if order not in (1, 3):
        raise SceneError("integrator: shape_function_order must be 1 or 3")
    category = _attr(integ, "shape_function_category", required=False) or "Standard"
    if category not in ("Standard", "uGIMP"):
        raise SceneError("integrator: shape_function_category must be uGIMP or Standard")
    if order == 3:
        raise SceneError("integrator: third-order basis functions are outside this library")
    cfg.update(dt=dt, dt_rational=dt_r, dt_string=integ.get("dt"), flip_alpha=alpha,
               basis="ugimp" if category == "uGIMP" else "linear")
    # loadStaticPlanes (:351-436)
    planes = []
    for nd in root.findall("static_plane"):
        x, n = _list(nd, "x", 2), _list(nd, "n", 2)
        beh = _attr(nd, "boundary_behavior")
        if beh not in ("sticking", "sliding"):
            raise SceneError("static_plane: boundary_behavior must be sticking or sliding")
        lb = nd.get("lower_bound")
        lower = -math.inf if lb is None else _scalar(nd, "lower_bound")
        planes.append((x, n, beh == "sticking", lower))
    cfg["planes"] = planes
    # loadGravityForce (:55-78): the last one wins, zero without any
    g = (0.0, 0.0)
    for nd in root.findall("near_earth_gravity"):
        g = _list(nd, "f", 2)
    cfg["gravity"] = g
    et = root.find("end_time")
    cfg["end_time"] = math.inf if et is None else _scalar(et, "t")
    if not cfg["end_time"] > 0.0:
        raise SceneError("end_time: t must be positive")
    cfg["rectangles"] = rects
    if not rects:
        # InitialSimulationState::generateSimulationState (:201-204)
        raise SceneError("provide at least one rectangle region")
    r0 = rects[0]
    cfg.update(rect_min=r0["min"], rect_max=r0["max"], rho=r0["density"],
               samples_per_dim=r0["samples_per_dim"])
    return cfg


def grid_origin(cfg):
    """PhysicsGrid::setDimensions: the grid is centred on the requested box
    with ceil(extent / h) cells per axis; returns the origin and the cell
    counts."""
    gmin, gmax, h = cfg["grid_min"], cfg["grid_max"], cfg["h"]
    nx = math.ceil((gmax[0] - gmin[0]) / h)
    ny = math.ceil((gmax[1] - gmin[1]) / h)
    cx, cy = 0.5 * (gmin[0] + gmax[0]), 0.5 * (gmin[1] + gmax[1])
    return (cx - 0.5 * (nx * h), cy - 0.5 * (ny * h)), (nx, ny)


def _inside_planes(planes, px, py):
    """pointInsidePlane (InitialSimulationState.cpp:33-44): planes in order;
    a point below a plane's lower bound ends the test with "outside", a
    point strictly behind a plane ends it with "inside"."""
    inside = np.zeros(px.shape, dtype=bool)
    open_ = np.ones(px.shape, dtype=bool)  # not yet decided
    for (x, n, _st, lb) in planes:
        nn = math.hypot(n[0], n[1])
        below = open_ & (py < lb)
        open_ &= ~below
        d = (n[0] / nn) * (px - x[0]) + (n[1] / nn) * (py - x[1])
        hit = open_ & (d < 0.0)
        inside |= hit
        open_ &= ~hit
    return inside


def seed_points(cfg):
    """InitialSimulationState::generateSimulationState with rasterizeRectangle
    (InitialSimulationState.cpp:46-145): every rectangle's samples in file
    order (cells y-major, then samples y-major), those outside the rectangle
    or behind a plane skipped; velocity vel + omega (-(y - yc), x - xc);
    mass density x (2 hl)^2 with hl = h / (2 samples per dimension)."""
    (g0x, g0y), _ = grid_origin(cfg)
    h = cfg["h"]
    gmax = (g0x + h * math.ceil((cfg["grid_max"][0] - cfg["grid_min"][0]) / h),
            g0y + h * math.ceil((cfg["grid_max"][1] - cfg["grid_min"][1]) / h))
    out = dict(q=[], v=[], m=[], vol=[], hl=[])
    for r in cfg["rectangles"]:
        rmin, rmax, npd = r["min"], r["max"], r["samples_per_dim"]
        if rmin[0] < g0x or rmin[1] < g0y:
            raise SceneError("initial rectangle region is below the simulation grid")
        if rmax[0] > gmax[0] or rmax[1] > gmax[1]:
            raise SceneError("initial rectangle region is above the simulation grid")
        bx0, by0 = math.floor((rmin[0] - g0x) / h), math.floor((rmin[1] - g0y) / h)
        bx1, by1 = math.ceil((rmax[0] - g0x) / h), math.ceil((rmax[1] - g0y) / h)
        if npd == 0 or bx1 <= bx0 or by1 <= by0:
            continue
        gx = np.arange(bx0, bx1, dtype=np.float64)
        gy = np.arange(by0, by1, dtype=np.float64)
        off = (np.arange(npd, dtype=np.float64) + 0.5) / float(npd)
        px = g0x + h * (gx[None, :, None, None] + off[None, None, None, :])
        py = g0y + h * (gy[:, None, None, None] + off[None, None, :, None])
        px, py = np.broadcast_arrays(px, py)
        px, py = px.ravel(), py.ravel()
        keep = (px >= rmin[0]) & (py >= rmin[1]) & (px <= rmax[0]) & (py <= rmax[1])
        keep &= ~_inside_planes(cfg["planes"], px, py)
        px, py = px[keep], py[keep]
        xc, yc = 0.5 * (rmin[0] + rmax[0]), 0.5 * (rmin[1] + rmax[1])
        w = r["omega"]
        v = np.stack([r["vel"][0] + w * -(py - yc), r["vel"][1] + w * (px - xc)], axis=1)
        hl = 0.5 * h / float(npd)
        vol = hl * hl * 4.0
        out["q"].append(np.stack([px, py], axis=1))
        out["v"].append(v)
        out["m"].append(np.full(px.size, r["density"] * vol))
        out["vol"].append(np.full(px.size, vol))
        out["hl"].append(np.full(px.size, hl))
    return {k: (np.concatenate(a) if a else np.zeros((0, 2) if k in ("q", "v") else 0))
            for k, a in out.items()}


def make_mpm(ctx, cfg, precision=None, capacity=0, points=None):
    """The scene's MPM object with its material points uploaded (seeded
    from the rectangles unless ``points`` is given)."""
    from . import MPM, LINEAR, UGIMP, MIXED
    p = seed_points(cfg) if points is None else points
    n = len(p["m"])
    obj = MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
              cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], cfg["gravity"],
              cfg["planes"], basis=UGIMP if cfg["basis"] == "ugimp" else LINEAR,
              precision=MIXED if precision is None else precision,
              capacity=max(int(capacity), n))
    obj.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    return obj


# ---- rigidbody2d ------------------------------------------------------------------

_DEM_UNSUPPORTED = ("planar_portal", "lees_edwards_portal")


def read_dem(source):
    """RigidBody2DSceneParser::parseXMLSceneFile (RigidBody2DSceneParser.cpp:
    1136-1330) for circle bodies under the penalty impact-friction map.

    Returns a dict: q, v as (N, 3) (x, y, theta); r, m, I (m = rho pi r^2,
    I = m r^2 / 2, CircleGeometry.cpp:44-48); fixed (uint8); rho; the
    penalty parameters kn, kt, gamman, gammat, mu and dt (with dt_rational,
    dt_string); cell_scale; gravity (the sum of the near_earth_gravity
    forces); planes as (x, n); end_time (inf when absent).
    """
    root = _root(source, "rigidbody2d_scene")
    for tag in _DEM_UNSUPPORTED:
        if root.find(tag) is not None:
            raise SceneError("%s: not supported by this library" % tag)
    d = {}
    et = root.find("end_time")
    d["end_time"] = math.inf if et is None else _scalar(et, "t")
    # loadPenaltyImpactFrictionMap (:975-1125): the DEM step's contact law
    pen = root.find("penalty_impact_map")
    if pen is None:
        raise SceneError("penalty_impact_map node missing (the only impact map of this path)")
    d["dt_rational"], d["dt"] = _time(pen, "dt")
    d["dt_string"] = pen.get("dt")
    for key in ("kn", "kt", "gamman", "gammat", "mu"):
        d[key] = _scalar(pen, key)
        if d[key] < 0.0:
            raise SceneError("penalty_impact_map: %s must be non-negative" % key)
    # loadCollisionDetection (:905-970)
    cd = root.find("collision_detection")
    if cd is None:
        raise SceneError("collision_detection node missing")
    if _attr(cd, "broadphase") != "spatial_grid":
        raise SceneError("collision_detection: broadphase must be spatial_grid")
    d["cell_scale"] = _scalar(cd, "cell_scale")
    if not d["cell_scale"] > 0.0:
        raise SceneError("collision_detection: cell_scale must be positive")
    if _attr(cd, "bandwidth_reduction") not in ("none", "cuthill_mckee"):
        raise SceneError("collision_detection: bandwidth_reduction must be none or cuthill_mckee")
    # loadGravityForce (:586-608): one force per node; their sum acts
    g = [0.0, 0.0]
    for nd in root.findall("near_earth_gravity"):
        f = _list(nd, "f", 2)
        g[0] += f[0]
        g[1] += f[1]
    d["gravity"] = tuple(g)
    # loadStaticPlanes (:219-270)
    d["planes"] = [(_list(nd, "x", 2), _list(nd, "n", 2)) for nd in root.findall("static_plane")]
    # loadStaticDrums (:541-585): centre x and a positive radius r
    d["drums"] = []
    for nd in root.findall("static_drum"):
        x = _list(nd, "x", 2)
        r = _scalar(nd, "r")
        if not r > 0.0:
            raise SceneError("static_drum: r must be a positive scalar")
        d["drums"].append((x, r))
    # loadGeometry (:610-725)
    geo = []
    for nd in root.findall("geometry"):
        kind = _attr(nd, "type")
        if kind == "circle":
            r = _scalar(nd, "r")
            if not r > 0.0:
                raise SceneError("geometry: circle radius must be positive")
            geo.append(r)
        elif kind in ("box", "annulus"):
            geo.append(kind)  # an error only if a body uses it
        else:
            raise SceneError("geometry: unknown type %r" % kind)
    # loadBodies (:727-900)
    bodies = root.findall("rigid_body")
    n = len(bodies)
    q, v = np.zeros((n, 3)), np.zeros((n, 3))
    r, rho = np.zeros(n), np.zeros(n)
    fixed = np.zeros(n, dtype=np.uint8)
    for k, nd in enumerate(bodies):
        x = _list(nd, "x", 2)
        q[k] = (x[0], x[1], _scalar(nd, "theta"))
        vb = _list(nd, "v", 2)
        v[k] = (vb[0], vb[1], _scalar(nd, "omega"))
        rho[k] = _scalar(nd, "rho")
        if not rho[k] > 0.0:
            raise SceneError("rigid_body: rho must be positive")
        gi = _int(nd, "geo_idx")
        if gi < 0 or gi >= len(geo):
            raise SceneError("rigid_body: geo_idx %d out of range" % gi)
        if not isinstance(geo[gi], float):
            raise SceneError("rigid_body: %s bodies are not supported by this library" % geo[gi])
        r[k] = geo[gi]
        fv = nd.get("fixed")
        if fv is not None:
            fi = _int(nd, "fixed")
            if fi not in (0, 1):
                raise SceneError("rigid_body: fixed must be a boolean")
            fixed[k] = fi
    m = rho * math.pi * r * r
    d.update(q=q, v=v, r=r, m=m, I=0.5 * m * r * r, fixed=fixed, rho=rho)
    return d


def make_dem(ctx, d, precision=None, capacity=0, contact_capacity=0):
    """The scene's DEM object with its bodies uploaded."""
    from . import DEM, FP64
    n = len(d["r"])
    obj = DEM(ctx, d["gravity"], d["kn"], d["kt"], d["gamman"], d["gammat"], d["mu"],
              d["planes"], cell_scale=d["cell_scale"], capacity=max(int(capacity), n),
              contact_capacity=contact_capacity, precision=FP64 if precision is None else precision,
              drums=d.get("drums", ()))
    obj.upload(d["q"], d["v"], d["r"], d["m"], d["I"], d["fixed"])
    return obj


# ---- hybridgrains2d --------------------------------------------------------------

def read_hybrid(path):
    """HybridGrains2DSceneParser (HybridGrains2DSceneParser.cpp): the
    discrete and continuum files (relative to this one), the time step and
    the coupling_force settings with the parser's defaults for absent
    attributes. Returns the scene dict of ``hybrid.HybridSim``: mpm (the
    continuum scene, with dt the hybrid time step), dem (the bodies),
    dem_params, zones and resampling, plus dt, dt_rational and end_time."""
    root = _root(path, "hybridgrains2d_scene")
    base = os.path.dirname(os.path.abspath(path))

    def sub(tag):
        nd = root.find(tag)
        if nd is None:
            raise SceneError("%s node missing" % tag)
        return os.path.join(base, _attr(nd, "file_name"))

    dem = read_dem(sub("discrete_sim"))
    mpm = read_mpm(sub("continuum_sim"))
    ts = root.find("time_step")
    if ts is None:
        raise SceneError("time_step node missing")
    dt_r, dt = _time(ts, "dt")
    et = root.find("end_time")
    if et is None:
        raise SceneError("end_time node missing")
    end_r, _ = _time(et, "t")
    style = root.find("integrator_style")
    if style is None:
        raise SceneError("integrator_style node missing")
    if _attr(style, "style") != "prediction_correction_advection_node_node":
        raise SceneError("integrator_style: only prediction_correction_advection_node_node "
                         "(the node-node step) is supported by this library")
    cf = root.find("coupling_force")
    if cf is None:
        raise SceneError("coupling_force node missing (the resampling interval needs it)")

    def opt(name, default, conv=_scalar):
        return default if cf.get(name) is None else conv(cf, name)

    def flag(name):
        return cf.get(name) is not None and _int(cf, name) != 0

    # loadHybridIntegratorSettings (:150-350) defaults for absent attributes
    zones = dict(level_set_cell_width=opt("level_set_cell_width", -1.0),
                 phi_window_size=opt("phi_window_size", -1.0),
                 phi_samples_per_cell_side=opt("phi_samples_per_cell_side", -1, _int),
                 phi_threshold=opt("phiThreshold", 0.5),
                 rzone_level_set=opt("rzoneLevelSet", 0.0),
                 rzone_half_thickness=opt("rzoneHalfThickness", 0.0),
                 allow_direct_transitions=flag(
                     "allow_direct_transitions_between_discrete_and_continuum"))
    res = dict(dem_r_mean=opt("demRMean", -1.0), dem_r_std=opt("demRStd", 0.0),
               rho_dem=opt("rho_dem", 0.96), avoid_a_void_freq=opt("avoidAVoidFreq", 20, _int),
               homogenize_stress=flag("homogenize_stress"),
               homogenize_velocity=flag("homogenize_velocity"),
               newly_inserted_continuum_stress_free=flag("newly_converted_continuum_stress_free"))
    mpm = dict(mpm, dt=dt)
    dem_params = {k: dem[k] for k in ("kn", "kt", "gamman", "gammat", "mu", "gravity",
                                       "cell_scale", "planes")}
    return dict(mpm=mpm, dem=dem, dem_params=dem_params, zones=zones, resampling=res, dt=dt,
                dt_rational=dt_r, end_time=float(end_r))
