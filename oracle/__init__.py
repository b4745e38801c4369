"""CPU oracle for the hybridgrains-gb300 tests (test infrastructure only).

An FP64 C++ restatement of the reference's per-step MPM, penalty-DEM and
node-node coupling code, loaded through ctypes. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it,
always as the reference the GPU results are compared with or as the timed CPU
baseline, never as the product path.

Parity with the reference binary is unpinned: the reference needs Eigen 3.3.3
and RapidXML 1.13, which are absent, and its own tests hold no golden vectors
for this path. The oracle is pinned instead by the reference's in-code
postconditions (tests/test_oracle_*.py) and by hand-derived known answers.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_U32 = ctypes.POINTER(ctypes.c_uint)
_P = ctypes.c_void_p


def _sig(lib):
    f = lib
    f.hgo_mpm_create.restype = _P
    f.hgo_mpm_create.argtypes = [_D, _D, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, _D]
    f.hgo_mpm_destroy.argtypes = [_P]
    f.hgo_mpm_set_threads.argtypes = [_P, ctypes.c_int]
    f.hgo_mpm_add_plane.argtypes = [_P, _D, _D, ctypes.c_int, ctypes.c_double]
    f.hgo_mpm_grid_info.argtypes = [_P, _D, _D, _U32]
    f.hgo_mpm_set_particles.argtypes = [_P, ctypes.c_int, _D, _D, _D, _D, _D, _D, _D, _I, _U8]
    f.hgo_mpm_get_particles.argtypes = [_P, _D, _D, _D, _D, _I, _D]
    f.hgo_mpm_get_grid.argtypes = [_P, _D, _D, _D, _D, _D, _D]
    f.hgo_mpm_set_grid_coupling.argtypes = [_P, _I, _D]
    f.hgo_mpm_set_mom_new.argtypes = [_P, _D]
    f.hgo_mpm_phase0.argtypes = [_P]
    f.hgo_mpm_phase1.argtypes = [_P, ctypes.c_double]
    f.hgo_mpm_phase2.argtypes = [_P, ctypes.c_double]
    f.hgo_mpm_step.argtypes = [_P, ctypes.c_double, ctypes.c_int]
    f.hgo_mpm_seed_rectangle.restype = ctypes.c_int
    f.hgo_mpm_seed_rectangle.argtypes = [_P, _D, _D, ctypes.c_double, ctypes.c_int, _D,
                                         ctypes.c_double, ctypes.c_int, _D, _D, _D, _D, _D]
    f.hgo_dem_create.restype = _P
    f.hgo_dem_create.argtypes = [ctypes.c_int, _D, _D, _D, _D, _D, _U8, _D, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double]
    f.hgo_dem_destroy.argtypes = [_P]
    f.hgo_dem_add_plane.argtypes = [_P, _D, _D]
    f.hgo_dem_add_drum.argtypes = [_P, _D, ctypes.c_double]
    f.hgo_dem_set_weights.argtypes = [_P, _D]
    f.hgo_dem_set_state.argtypes = [_P, _D, _D]
    f.hgo_dem_step.argtypes = [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    f.hgo_dem_get_state.argtypes = [_P, _D, _D]
    f.hgo_dem_record_width.restype = ctypes.c_int
    f.hgo_dem_get_contacts.restype = ctypes.c_int
    f.hgo_dem_get_contacts.argtypes = [_P, ctypes.c_int, _D]
    f.hgo_dem_candidate_pairs.restype = ctypes.c_int
    f.hgo_dem_candidate_pairs.argtypes = [ctypes.c_int, _D, _D, ctypes.c_double, ctypes.c_int,
                                          _I, _D, _U32, _D]
    f.hgo_hybrid_create.restype = _P
    f.hgo_hybrid_create.argtypes = [_P, _P]
    f.hgo_hybrid_destroy.argtypes = [_P]
    f.hgo_hybrid_step.argtypes = [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    f.hgo_hybrid_clear_homogenized.argtypes = [_P]
    f.hgo_hybrid_num_packed.restype = ctypes.c_int
    f.hgo_hybrid_num_packed.argtypes = [_P, ctypes.c_int]
    f.hgo_hybrid_get.argtypes = [_P, _I, _I, _D, _D, _D, _D, _D, _D, _D]


def _zones_sig(f):
    f.hgo_zones_create.restype = _P
    f.hgo_zones_create.argtypes = [_D, ctypes.c_double, _I, ctypes.c_double, ctypes.c_int]
    f.hgo_zones_destroy.argtypes = [_P]
    f.hgo_zones_packing.argtypes = [_P, ctypes.c_int, _D, _D, _U8, ctypes.c_int, _D,
                                    ctypes.c_double, ctypes.c_int]
    f.hgo_zones_distance.argtypes = [_P, ctypes.c_double]
    f.hgo_zones_labels.argtypes = [_P, ctypes.c_double, ctypes.c_double]
    f.hgo_zones_get.argtypes = [_P, _D, _D, _I, _I]
    f.hgo_zones_nsamples.restype = ctypes.c_int
    f.hgo_zones_nsamples.argtypes = [_P]
    f.hgo_zones_list.restype = ctypes.c_int
    f.hgo_zones_list.argtypes = [_P, ctypes.c_int, _D, _I]
    f.hgo_zones_to_delete.restype = ctypes.c_int
    f.hgo_zones_to_delete.argtypes = [_P, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, _U8, _I]
    f.hgo_zones_weights.argtypes = [_P, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, _D]
    f.hgo_zones_set_labels.argtypes = [_P, _I]
    f.hgo_disk_box_area.restype = ctypes.c_double
    f.hgo_disk_box_area.argtypes = [ctypes.c_double] * 7


def lib():
    global _lib
    if _lib is None:
        # HG_ORACLE_LIB: a separately built copy (the sanitizer test's build)
        path = os.environ.get("HG_ORACLE_LIB") or _build.build()
        _lib = ctypes.CDLL(path)
        _sig(_lib)
        _zones_sig(_lib)
    return _lib


_ref = None


def reference_lib():
    """The reference's own standalone sources (circle/box area, MT19937)
    built by oracle/build_ref.py, or None where the reference checkout is
    absent."""
    global _ref
    if _ref is None:
        from . import build_ref
        path = build_ref.build()
        if path is None:
            return None
        _ref = ctypes.CDLL(path)
        _ref.hgr_circle_rectangle_area.restype = ctypes.c_double
        _ref.hgr_circle_rectangle_area.argtypes = [ctypes.c_double] * 7
        _ref.seedMT.argtypes = [ctypes.c_uint32]
        _ref.randomMT.restype = ctypes.c_float
        _ref.randomMT_i.restype = ctypes.c_uint32
    return _ref


def _d(a):
    return a.ctypes.data_as(_D) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_I) if a is not None else None


def _u8(a):
    return a.ctypes.data_as(_U8) if a is not None else None


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


class MPM:
    """ExplicitIntegrator + SimulationState (mpmgrains2d) on the CPU."""

    def __init__(self, grid_min, grid_max, h, basis=0, shear_modulus=1.0, bulk_modulus=1.0,
                 dp_alpha=0.0, flip_alpha=0.999, gravity=(0.0, -9.81), threads=1):
        L = lib()
        self._h = L.hgo_mpm_create(_d(_f64(grid_min)), _d(_f64(grid_max)), float(h), int(basis),
                                   float(shear_modulus), float(bulk_modulus), float(dp_alpha),
                                   float(flip_alpha), _d(_f64(gravity)))
        L.hgo_mpm_set_threads(self._h, int(threads))
        gmin = np.zeros(2)
        gmax = np.zeros(2)
        nxny = np.zeros(2, dtype=np.uint32)
        L.hgo_mpm_grid_info(self._h, _d(gmin), _d(gmax), nxny.ctypes.data_as(_U32))
        self.grid_min, self.grid_max = gmin, gmax
        self.nx, self.ny = int(nxny[0]), int(nxny[1])
        self.nnodes = (self.nx + 1) * (self.ny + 1)
        self.np = 0

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.hgo_mpm_destroy(self._h)
            self._h = None

    def set_threads(self, n):
        lib().hgo_mpm_set_threads(self._h, int(n))

    def add_plane(self, x, n, sticking, lower_bound=-np.inf):
        lib().hgo_mpm_add_plane(self._h, _d(_f64(x)), _d(_f64(n)), int(sticking), float(lower_bound))

    def seed_rectangle(self, rmin, rmax, rho, npd, vel=(0.0, 0.0), omega=0.0):
        L = lib()
        cnt = L.hgo_mpm_seed_rectangle(self._h, _d(_f64(rmin)), _d(_f64(rmax)), float(rho),
                                       int(npd), _d(_f64(vel)), float(omega), 0,
                                       None, None, None, None, None)
        q = np.zeros(2 * cnt)
        v = np.zeros(2 * cnt)
        m = np.zeros(cnt)
        vol = np.zeros(cnt)
        hl = np.zeros(cnt)
        L.hgo_mpm_seed_rectangle(self._h, _d(_f64(rmin)), _d(_f64(rmax)), float(rho), int(npd),
                                 _d(_f64(vel)), float(omega), cnt, _d(q), _d(v), _d(m), _d(vol),
                                 _d(hl))
        return dict(q=q.reshape(-1, 2), v=v.reshape(-1, 2), m=m, vol=vol, hl=hl)

    def set_particles(self, q, v, m, vol, hl, be=None, J=None, jh=None, kin=None):
        n = len(m)
        be = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), n) if be is None else _f64(be).ravel()
        J = np.ones(n) if J is None else _f64(J)
        jh = np.zeros(n, dtype=np.int32) if jh is None else np.ascontiguousarray(jh, dtype=np.int32)
        kin = np.zeros(n, dtype=np.uint8) if kin is None else np.ascontiguousarray(kin, dtype=np.uint8)
        self._keep = [_f64(q).ravel(), _f64(v).ravel(), _f64(m), _f64(vol), _f64(hl), be, J, jh, kin]
        a = self._keep
        lib().hgo_mpm_set_particles(self._h, n, _d(a[0]), _d(a[1]), _d(a[2]), _d(a[3]), _d(a[4]),
                                    _d(a[5]), _d(a[6]), _i(a[7]), _u8(a[8]))
        self.np = n

    def particles(self):
        n = self.np
        q = np.zeros(2 * n)
        v = np.zeros(2 * n)
        be = np.zeros(4 * n)
        J = np.zeros(n)
        jh = np.zeros(n, dtype=np.int32)
        sg = np.zeros(4 * n)
        lib().hgo_mpm_get_particles(self._h, _d(q), _d(v), _d(be), _d(J), _i(jh), _d(sg))
        return dict(q=q.reshape(-1, 2), v=v.reshape(-1, 2), be=be.reshape(-1, 4), J=J, jh=jh,
                    sigma=sg.reshape(-1, 4))

    def grid(self):
        n = self.nnodes
        out = {k: np.zeros(2 * n) for k in ("mom", "mom_new", "force", "vel", "acc")}
        mass = np.zeros(n)
        lib().hgo_mpm_get_grid(self._h, _d(mass), _d(out["mom"]), _d(out["mom_new"]),
                               _d(out["force"]), _d(out["vel"]), _d(out["acc"]))
        res = {k: v.reshape(-1, 2) for k, v in out.items()}
        res["mass"] = mass
        return res

    def set_grid_coupling(self, hybridized=None, coupling_force=None):
        hy = None if hybridized is None else np.ascontiguousarray(hybridized, dtype=np.int32)
        cf = None if coupling_force is None else _f64(coupling_force).ravel()
        lib().hgo_mpm_set_grid_coupling(self._h, _i(hy), _d(cf))

    def phase0(self):
        lib().hgo_mpm_phase0(self._h)

    def phase1(self, dt):
        lib().hgo_mpm_phase1(self._h, float(dt))

    def phase2(self, dt):
        lib().hgo_mpm_phase2(self._h, float(dt))

    def step(self, dt, nsteps=1):
        lib().hgo_mpm_step(self._h, float(dt), int(nsteps))


class DEM:
    """RigidBody2DSim + PenaltyImpactFrictionMap (rigidbody2d) on the CPU."""

    def __init__(self, q, v, r, m, I, fixed, gravity, kn, kt, gamman, gammat, mu, cell_scale):
        self.n = len(r)
        q = _f64(q).ravel()
        v = _f64(v).ravel()
        fx = np.ascontiguousarray(fixed, dtype=np.uint8)
        self._h = lib().hgo_dem_create(self.n, _d(q), _d(v), _d(_f64(r)), _d(_f64(m)), _d(_f64(I)),
                                       _u8(fx), _d(_f64(gravity)), float(kn), float(kt),
                                       float(gamman), float(gammat), float(mu), float(cell_scale))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.hgo_dem_destroy(self._h)
            self._h = None

    def add_plane(self, x, n):
        lib().hgo_dem_add_plane(self._h, _d(_f64(x)), _d(_f64(n)))

    def add_drum(self, x, r):
        lib().hgo_dem_add_drum(self._h, _d(_f64(x)), float(r))

    def set_weights(self, w):
        lib().hgo_dem_set_weights(self._h, _d(_f64(w)))

    def set_state(self, q=None, v=None):
        qq = None if q is None else _f64(q).ravel()
        vv = None if v is None else _f64(v).ravel()
        lib().hgo_dem_set_state(self._h, _d(qq), _d(vv))

    def step(self, dt, nsteps=1, weighted=False):
        lib().hgo_dem_step(self._h, float(dt), int(nsteps), int(bool(weighted)))

    def state(self):
        q = np.zeros(3 * self.n)
        v = np.zeros(3 * self.n)
        lib().hgo_dem_get_state(self._h, _d(q), _d(v))
        return q.reshape(-1, 3), v.reshape(-1, 3)

    def contacts(self):
        L = lib()
        w = L.hgo_dem_record_width()
        cnt = L.hgo_dem_get_contacts(self._h, 0, None)
        buf = np.zeros(max(cnt, 1) * w)
        L.hgo_dem_get_contacts(self._h, cnt, _d(buf))
        return buf[: cnt * w].reshape(cnt, w)


def candidate_pairs(aabb_min, aabb_max, cell_scale):
    """SpatialGrid::getPotentialOverlaps: sorted (i, j), i < j, plus h/dims/origin."""
    L = lib()
    mn = _f64(aabb_min).ravel()
    mx = _f64(aabb_max).ravel()
    n = len(mn) // 2
    h = np.zeros(1)
    dims = np.zeros(2, dtype=np.uint32)
    org = np.zeros(2)
    cnt = L.hgo_dem_candidate_pairs(n, _d(mn), _d(mx), float(cell_scale), 0, None, _d(h),
                                    dims.ctypes.data_as(_U32), _d(org))
    pairs = np.zeros(2 * max(cnt, 1), dtype=np.int32)
    L.hgo_dem_candidate_pairs(n, _d(mn), _d(mx), float(cell_scale), cnt, _i(pairs), _d(h),
                              dims.ctypes.data_as(_U32), _d(org))
    return pairs[: 2 * cnt].reshape(cnt, 2), float(h[0]), dims.copy(), org


class Hybrid:
    """HybridGrains2DSim node-node step over an MPM and a DEM oracle."""

    def __init__(self, mpm, dem):
        self.mpm, self.dem = mpm, dem
        self._h = lib().hgo_hybrid_create(mpm._h, dem._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.hgo_hybrid_destroy(self._h)
            self._h = None

    def step(self, dt, nsteps=1, homogenize_stress=False, homogenize_velocity=False):
        flags = (1 if homogenize_stress else 0) | (2 if homogenize_velocity else 0)
        lib().hgo_hybrid_step(self._h, float(dt), int(nsteps), flags)

    def clear_homogenized(self):
        lib().hgo_hybrid_clear_homogenized(self._h)

    def coupling(self):
        L = lib()
        nd = L.hgo_hybrid_num_packed(self._h, 0)
        nm = L.hgo_hybrid_num_packed(self._h, 1)
        nn = self.mpm.nnodes
        pd = np.zeros(max(nd, 1), dtype=np.int32)
        pm = np.zeros(max(nm, 1), dtype=np.int32)
        dm = np.zeros(nn)
        dp = np.zeros(2 * nn)
        va = np.zeros(2 * nn)
        aa = np.zeros(2 * nn)
        hf = np.zeros(nn)
        hs = np.zeros(4 * nn)
        hv = np.zeros(2 * nn)
        L.hgo_hybrid_get(self._h, _i(pd), _i(pm), _d(dm), _d(dp), _d(va), _d(aa), _d(hf), _d(hs),
                         _d(hv))
        return dict(packed_dem=pd[:nd], packed_mpm=pm[:nm], dem_mass_grid=dm,
                    dem_mom_grid=dp.reshape(-1, 2), v_after=va.reshape(-1, 2),
                    at_after=aa.reshape(-1, 2), homog_factor=hf, homog_stress=hs.reshape(-1, 4),
                    homog_velocity=hv.reshape(-1, 2))


class Zones:
    """ZoneTools restated (zones_oracle.cpp)."""

    def __init__(self, mpm_min, mpm_cell_width, mpm_cells, level_set_cell_width,
                 allow_direct=False):
        self.cells = (int(mpm_cells[0]), int(mpm_cells[1]))
        self.N = tuple(int(np.ceil(c * mpm_cell_width / level_set_cell_width)) for c in mpm_cells)
        self._h = lib().hgo_zones_create(_d(_f64(mpm_min)), float(mpm_cell_width),
                                         (ctypes.c_int * 2)(*self.cells),
                                         float(level_set_cell_width), int(allow_direct))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hgo_zones_destroy(self._h)
            self._h = None

    def update(self, q3, r, fixed, points, window, samples, threshold, level, half):
        q3 = _f64(q3)
        r = _f64(r)
        fixed = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        points = _f64(points) if points is not None else None
        L = lib()
        L.hgo_zones_packing(self._h, len(r), _d(q3), _d(r),
                            None if fixed is None else fixed.ctypes.data_as(_U8),
                            0 if points is None else len(points), _d(points), float(window),
                            int(samples))
        L.hgo_zones_distance(self._h, float(threshold))
        L.hgo_zones_labels(self._h, float(level), float(half))

    def fields(self):
        nx, ny = self.N
        pf = np.zeros(nx * ny)
        dist = np.zeros((nx + 1) * (ny + 1))
        ls = np.zeros(nx * ny, dtype=np.int32)
        mpm = np.zeros(self.cells[0] * self.cells[1], dtype=np.int32)
        lib().hgo_zones_get(self._h, _d(pf), _d(dist), _i(ls), _i(mpm))
        return dict(phi=pf, dist=dist, ls=ls, mpm=mpm)

    def samples(self):
        return lib().hgo_zones_nsamples(self._h)

    def zone_list(self, which):
        n = lib().hgo_zones_list(self._h, int(which), None, None)
        boxes = np.zeros((n, 4))
        cells = np.zeros((n, 2), dtype=np.int32)
        lib().hgo_zones_list(self._h, int(which), _d(boxes), _i(cells))
        return boxes, cells

    def to_delete(self, kind, x, stride, fixed=None):
        x = _f64(x)
        n = len(x.reshape(-1)) // stride
        ids = np.zeros(max(n, 1), dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        c = lib().hgo_zones_to_delete(self._h, int(kind), n, _d(x), int(stride),
                                      None if fx is None else fx.ctypes.data_as(_U8), _i(ids))
        return ids[:c]

    def weights(self, kind, x, stride):
        x = _f64(x)
        n = len(x.reshape(-1)) // stride
        w = np.zeros(n)
        lib().hgo_zones_weights(self._h, int(kind), n, _d(x), int(stride), _d(w))
        return w

    def set_labels(self, mpm):
        mpm = np.ascontiguousarray(mpm, dtype=np.int32)
        lib().hgo_zones_set_labels(self._h, _i(mpm))


def disk_box_area(x0, x1, y0, y1, cx, cy, r):
    return lib().hgo_disk_box_area(x0, x1, y0, y1, cx, cy, r)
