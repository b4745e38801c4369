"""The reference's on-disk formats for the MPM path, written and read here.

Snapshot (``serial.bin``, mpmgrains2d_cli ``-s`` / ``-r``): the byte layout of
the reference's serialize chain on a 64-bit little-endian build, restated
field by field:

* mpmgrains2d_cli.cpp:163-188: uint32 magic 9035768, the git revision as a
  string, SimulationState, uint32 iteration, the time step as a rational
  (int64 numerator, int64 denominator), double end time, [the output
  directory as a string, in builds with HDF5 only], uint32 steps per save,
  uint32 output frame, uint32 time-string precision, uint32 save-number width,
  bool serialize snapshots, bool overwrite snapshots;
* SimulationState.cpp:119-129: MaterialPoints, PhysicsGrid, the static
  planes, doubles shear modulus, bulk modulus, Drucker-Prager alpha, the
  gravity (2 doubles), PIC/FLIP alpha, and the basis type (int32: linear 0,
  third order 1, uGIMP 2, BasisFunctions.h:13);
* MaterialPoints.cpp:35-53: uint32 point count, q0, q, v (2 x N matrices:
  int64 column count, then column-major doubles), m, volume, m0, volume0,
  weight, hl (vectors: int64 length, doubles), be_bar (uint64 count, 2 x 2
  column-major doubles each), J, sigma, vel_grad (as be_bar),
  just_homogenized (int64 length, int32), always_fixed and
  kinematically_scripted (uint64 length, one byte per flag);
* PhysicsGrid.cpp:118-131: min, max (2 doubles each), cell width, cell count
  (2 uint32), the rasterized mass (vector), momentum, new momentum, force,
  velocity, acceleration (2 x N matrices), homog_factor (vector), hybridized
  (int64 length, int32);
* StaticPlane.cpp:22-27 (the planes, after a uint64 count): x and n (2
  doubles each), the boundary behaviour (int32: sliding 0, sticking 1) and the
  lower bound (double).

Strings are a uint64 length and the bytes (StringUtilities.cpp:21-26).
"""
import struct

import numpy as np

MPM_MAGIC = 9035768
BASIS_LINEAR, BASIS_THIRD_ORDER, BASIS_UGIMP = 0, 1, 2
SLIDING, STICKING = 0, 1

POINT_VECTORS = ("m", "volume", "m0", "volume0", "weight", "hl")
GRID_MATRICES = ("momentum", "momentum_new", "force", "velocity", "acceleration")


class _Writer:
    def __init__(self):
        self.parts = []

    def pack(self, fmt, *v):
        self.parts.append(struct.pack("<" + fmt, *v))

    def raw(self, a, dtype):
        self.parts.append(np.ascontiguousarray(a, dtype=dtype).tobytes())

    def string(self, s):
        b = s.encode()
        self.pack("Q", len(b))
        self.parts.append(b)

    def matrix2x(self, a):  # (N, 2) rows -> 2 x N column-major
        a = np.asarray(a, dtype=np.float64).reshape(-1, 2)
        self.pack("q", len(a))
        self.raw(a, "<f8")

    def vector(self, a, dtype="<f8"):
        a = np.asarray(a).reshape(-1)
        self.pack("q", len(a))
        self.raw(a, dtype)

    def mat22_list(self, a):  # (N, 4) column-major 2 x 2 blocks
        a = np.asarray(a, dtype=np.float64).reshape(-1, 4)
        self.pack("Q", len(a))
        self.raw(a, "<f8")

    def flags(self, a):
        a = np.asarray(a, dtype=bool).reshape(-1)
        self.pack("Q", len(a))
        self.raw(a, "u1")

    def bytes(self):
        return b"".join(self.parts)


class _Reader:
    def __init__(self, data):
        self.d, self.o = data, 0

    def unpack(self, fmt):
        fmt = "<" + fmt
        n = struct.calcsize(fmt)
        if self.o + n > len(self.d):
            raise ValueError("truncated snapshot")
        v = struct.unpack_from(fmt, self.d, self.o)
        self.o += n
        return v if len(v) > 1 else v[0]

    def raw(self, count, dtype):
        dt = np.dtype(dtype)
        n = count * dt.itemsize
        if count < 0 or self.o + n > len(self.d):
            raise ValueError("truncated snapshot")
        a = np.frombuffer(self.d, dtype=dt, count=count, offset=self.o).copy()
        self.o += n
        return a

    def string(self):
        n = self.unpack("Q")
        if self.o + n > len(self.d):
            raise ValueError("truncated snapshot")
        s = self.d[self.o:self.o + n].decode()
        self.o += n
        return s

    def matrix2x(self):
        n = self.unpack("q")
        return self.raw(2 * n, "<f8").reshape(n, 2)

    def vector(self, dtype="<f8"):
        return self.raw(self.unpack("q"), dtype)

    def mat22_list(self):
        n = self.unpack("Q")
        return self.raw(4 * n, "<f8").reshape(n, 4)

    def flags(self):
        return self.raw(self.unpack("Q"), "u1").astype(bool)


def _points_defaults(p):
    n = len(p["q"])
    out = dict(p)
    out.setdefault("q0", p["q"])
    out.setdefault("m0", p["m"])
    out.setdefault("volume0", p["volume"])
    out.setdefault("weight", np.ones(n))
    out.setdefault("hl", np.zeros(n))
    out.setdefault("sigma", np.zeros((n, 4)))
    out.setdefault("vel_grad", np.zeros((n, 4)))
    out.setdefault("just_homogenized", np.zeros(n, dtype=np.int32))
    out.setdefault("always_fixed", np.zeros(n, dtype=bool))
    out.setdefault("kinematically_scripted", np.zeros(n, dtype=bool))
    return out


def encode_mpm_snapshot(state, run, with_output_dir=False):
    """Bytes of a reference MPM snapshot. ``state``: dict with ``points``
    (q, v, m, volume, be_bar, J and optionally the other MaterialPoints
    fields), ``grid`` (min, max, cell_width, cell_count and the node fields;
    missing node fields are written as zeros), ``planes`` (list of (x, n,
    behaviour, lower_bound)), ``shear_modulus``, ``bulk_modulus``,
    ``dp_alpha``, ``gravity``, ``flip_alpha``, ``basis``. ``run``: dict with
    ``iteration``, ``dt`` (numerator, denominator), ``end_time`` and
    optionally ``git_revision``, ``output_dir``, ``steps_per_save``,
    ``output_frame``, ``dt_string_precision``, ``save_number_width``,
    ``serialize_snapshots``, ``overwrite_snapshots``."""
    p = _points_defaults(state["points"])
    g = state["grid"]
    n = len(p["q"])
    nn = int((g["cell_count"][0] + 1) * (g["cell_count"][1] + 1))
    w = _Writer()
    w.pack("I", MPM_MAGIC)
    w.string(run.get("git_revision", ""))
    # MaterialPoints
    w.pack("I", n)
    for k in ("q0", "q", "v"):
        w.matrix2x(p[k])
    for k in POINT_VECTORS:
        w.vector(p[k])
    w.mat22_list(p["be_bar"])
    w.vector(p["J"])
    w.mat22_list(p["sigma"])
    w.mat22_list(p["vel_grad"])
    w.vector(p["just_homogenized"], "<i4")
    w.flags(p["always_fixed"])
    w.flags(p["kinematically_scripted"])
    # PhysicsGrid
    w.pack("2d", *map(float, g["min"]))
    w.pack("2d", *map(float, g["max"]))
    w.pack("d", float(g["cell_width"]))
    w.pack("2I", *map(int, g["cell_count"]))
    w.vector(g.get("mass", np.zeros(nn)))
    for k in GRID_MATRICES:
        w.matrix2x(g.get(k, np.zeros((nn, 2))))
    w.vector(g.get("homog_factor", np.zeros(nn)))
    w.vector(g.get("hybridized", np.zeros(nn, dtype=np.int32)), "<i4")
    # static planes
    w.pack("Q", len(state["planes"]))
    for (x, nrm, behaviour, lower) in state["planes"]:
        w.pack("2d", *map(float, x))
        w.pack("2d", *map(float, nrm))
        w.pack("i", int(behaviour))
        w.pack("d", float(lower))
    w.pack("3d", float(state["shear_modulus"]), float(state["bulk_modulus"]),
           float(state["dp_alpha"]))
    w.pack("2d", *map(float, state["gravity"]))
    w.pack("d", float(state["flip_alpha"]))
    w.pack("i", int(state["basis"]))
    # the CLI's run state
    w.pack("I", int(run["iteration"]))
    w.pack("2q", int(run["dt"][0]), int(run["dt"][1]))
    w.pack("d", float(run["end_time"]))
    if with_output_dir:
        w.string(run.get("output_dir", ""))
    w.pack("4I", int(run.get("steps_per_save", 0)), int(run.get("output_frame", 0)),
           int(run.get("dt_string_precision", 0)), int(run.get("save_number_width", 0)))
    w.pack("2?", bool(run.get("serialize_snapshots", True)),
           bool(run.get("overwrite_snapshots", False)))
    return w.bytes()


def decode_mpm_snapshot(data, with_output_dir=False):
    """(state, run) of a reference MPM snapshot (see encode_mpm_snapshot)."""
    r = _Reader(data)
    if r.unpack("I") != MPM_MAGIC:
        raise ValueError("not a serialized 2D MPM simulation")
    run = dict(git_revision=r.string())
    n = r.unpack("I")
    p = {}
    for k in ("q0", "q", "v"):
        p[k] = r.matrix2x()
    for k in POINT_VECTORS:
        p[k] = r.vector()
    p["be_bar"] = r.mat22_list()
    p["J"] = r.vector()
    p["sigma"] = r.mat22_list()
    p["vel_grad"] = r.mat22_list()
    p["just_homogenized"] = r.vector("<i4")
    p["always_fixed"] = r.flags()
    p["kinematically_scripted"] = r.flags()
    if any(len(p[k]) != n for k in ("q", "v", "m", "J", "be_bar")):
        raise ValueError("inconsistent point count")
    g = dict(min=r.unpack("2d"), max=r.unpack("2d"), cell_width=r.unpack("d"),
             cell_count=r.unpack("2I"))
    g["mass"] = r.vector()
    for k in GRID_MATRICES:
        g[k] = r.matrix2x()
    g["homog_factor"] = r.vector()
    g["hybridized"] = r.vector("<i4")
    planes = []
    for _ in range(r.unpack("Q")):
        x, nrm = r.unpack("2d"), r.unpack("2d")
        planes.append((x, nrm, r.unpack("i"), r.unpack("d")))
    mu, kappa, alpha = r.unpack("3d")
    state = dict(points=p, grid=g, planes=planes, shear_modulus=mu, bulk_modulus=kappa,
                 dp_alpha=alpha, gravity=r.unpack("2d"), flip_alpha=r.unpack("d"),
                 basis=r.unpack("i"))
    run["iteration"] = r.unpack("I")
    run["dt"] = r.unpack("2q")
    run["end_time"] = r.unpack("d")
    if with_output_dir:
        run["output_dir"] = r.string()
    (run["steps_per_save"], run["output_frame"], run["dt_string_precision"],
     run["save_number_width"]) = r.unpack("4I")
    run["serialize_snapshots"], run["overwrite_snapshots"] = r.unpack("2?")
    if r.o != len(data):
        raise ValueError("trailing bytes after the snapshot")
    return state, run


def cauchy_stress(be, J, jh, shear_modulus, bulk_modulus):
    """MaterialPoints::computeHyperelasticCauchyStress with
    ConstitutiveModel::computeTau (MaterialPoints.cpp:183-202,
    ConstitutiveModel.cpp:83-97): for J <= 1 and no just-homogenised flag,
    tau = kappa (J + 1)(J - 1) / 2 I + mu dev(b_e / sqrt(det b_e)) with
    b_e = be_bar J; sigma = tau / J; else 0. Column-major 2 x 2 per row."""
    be = np.asarray(be, dtype=np.float64).reshape(-1, 4)
    J = np.asarray(J, dtype=np.float64)
    b = be * J[:, None]
    det = b[:, 0] * b[:, 3] - b[:, 1] * b[:, 2]
    s = np.sqrt(np.where(det > 0, det, 1.0))  # the J of computeTau
    bn = b / s[:, None]
    tr = 0.5 * (bn[:, 0] + bn[:, 3])
    dev = bn.copy()
    dev[:, 0] -= tr
    dev[:, 3] -= tr
    tau = shear_modulus * dev
    pr = bulk_modulus * 0.5 * (s + 1.0) * (s - 1.0)
    tau[:, 0] += pr
    tau[:, 3] += pr
    sigma = tau / J[:, None]
    live = (J <= 1.0) & (np.asarray(jh) == 0)
    return np.where(live[:, None], sigma, 0.0)


def _gravity():
    from . import scenes
    return scenes.GRAVITY


def snapshot_from_device(mpm, cfg, m, volume, hl=None, q0=None):
    """The reference snapshot's SimulationState for a device MPM object:
    its points and grid, plus the host-held masses and volumes (and, when
    given, half widths and reference positions). sigma is evaluated from the
    downloaded be_bar and J; vel_grad, a per-step temporary, is zero."""
    st = mpm.download()
    G = mpm.grid()
    nn = mpm.nnodes
    grid = dict(min=mpm.grid_min, max=mpm.grid_max, cell_width=cfg["h"],
                cell_count=(mpm.nx, mpm.ny), mass=G["mass"], velocity=G["vel"],
                acceleration=G["acc"], homog_factor=np.zeros(nn))
    for k_ref, k_here in (("momentum", "mom"), ("momentum_new", "mom_new"), ("force", "force")):
        if k_here in G:
            grid[k_ref] = G[k_here]
    n = len(st["q"])
    pts = dict(q=st["q"], v=st["v"], m=m, volume=volume, be_bar=st["be"], J=st["J"],
               just_homogenized=st["jh"],
               sigma=cauchy_stress(st["be"], st["J"], st["jh"], cfg["shear_modulus"],
                                   cfg["bulk_modulus"]))
    if hl is not None:
        pts["hl"] = hl
    if q0 is not None:
        pts["q0"] = q0
    planes = [(x, nrm, STICKING if sticking else SLIDING, lower)
              for (x, nrm, sticking, lower) in cfg["planes"]]
    assert n == len(m) == len(volume)
    return dict(points=pts, grid=grid, planes=planes, shear_modulus=cfg["shear_modulus"],
                bulk_modulus=cfg["bulk_modulus"], dp_alpha=cfg["dp_alpha"],
                gravity=cfg.get("gravity", _gravity()), flip_alpha=cfg["flip_alpha"],
                basis=BASIS_UGIMP if getattr(mpm, "basis", 0) == 1 else BASIS_LINEAR)


def device_from_snapshot(ctx, state, precision=None, capacity=None):
    """A device MPM object with the snapshot's grid, material, planes and
    points (the grid fields are rasterised again by the next step)."""
    import libhybridgrains_gb300 as hg
    g, p = state["grid"], state["points"]
    planes = [(x, nrm, behaviour == STICKING, lower)
              for (x, nrm, behaviour, lower) in state["planes"]]
    basis = 1 if state["basis"] == BASIS_UGIMP else 0
    if state["basis"] == BASIS_THIRD_ORDER:
        raise ValueError("the cubic basis is not supported")
    m = hg.MPM(ctx, tuple(g["min"]), tuple(g["max"]), g["cell_width"], state["shear_modulus"],
               state["bulk_modulus"], state["dp_alpha"], state["flip_alpha"],
               tuple(state["gravity"]), planes, basis=basis,
               precision=hg.FP64 if precision is None else precision,
               capacity=capacity or len(p["q"]))
    kin = np.asarray(p["kinematically_scripted"], dtype=np.uint8)
    m.upload(p["q"], p["v"], p["m"], p["volume"], p["hl"], p["be_bar"], p["J"],
             p["just_homogenized"], kin)
    return m


def write_mpm_snapshot(path, state, run, with_output_dir=False):
    with open(path, "wb") as f:
        f.write(encode_mpm_snapshot(state, run, with_output_dir))


def read_mpm_snapshot(path, with_output_dir=False):
    with open(path, "rb") as f:
        return decode_mpm_snapshot(f.read(), with_output_dir)
