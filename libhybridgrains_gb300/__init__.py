"""GB300-native per-timestep core of libHybridGrains (Python host binding).

The compute lives in ``libhg_gpu.so`` (hand-written sm_103a CUDA behind the C
ABI of ``include/hg_gpu.h``). This module binds that ABI with ctypes and numpy
and mirrors the reference's integrator surface:

* ``MPM``     - SimulationState + ExplicitIntegrator (mpmgrains2d):
                ``flow(dt)``, ``flow_zero_phase()``, ``flow_first_phase(dt)``,
                ``flow_second_phase(dt)``.
* ``DEM``     - RigidBody2DSim + PenaltyImpactFrictionMap (rigidbody2d):
                ``flow(dt)``, ``flow_with_weights(dt)``.
* ``Hybrid``  - HybridGrains2DSim node-node step (hybridgrains2dnew).

There is no CPU fallback: constructing any object loads the CUDA library and
raises if it is missing or no GPU is present.
"""
import ctypes
import os
import weakref

import numpy as np

from . import _capi
from ._capi import HGError, check, load  # noqa: F401

__all__ = ["Context", "MPM", "DEM", "Hybrid", "Batch", "HGError", "load",
           "kernel_launch_count", "pinned"]

LINEAR, UGIMP = 0, 1
FP64, MIXED = 0, 1


def _d(a):
    return None if a is None else a.ctypes.data_as(_capi._D)


def _i32(a):
    return None if a is None else a.ctypes.data_as(_capi._I32)


def _u8(a):
    return None if a is None else a.ctypes.data_as(_capi._U8)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def pinned(shape, dtype=np.float64):
    """A numpy array in page-locked host memory (hg_host_alloc), freed when
    the array is garbage collected. Asynchronous copies to and from it
    overlap with queued device work."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    nbytes = max(count * dt.itemsize, 1)
    p = ctypes.c_void_p()
    check("hg_host_alloc", nbytes, ctypes.byref(p))
    buf = (ctypes.c_char * nbytes).from_address(p.value)
    arr = np.frombuffer(buf, dtype=dt, count=count).reshape(shape)
    weakref.finalize(buf, _capi.load().hg_host_free, ctypes.c_void_p(p.value))
    return arr


def _save_blob(prefix, h):
    """The object's state blob (hg_*_state_save) as a uint8 array."""
    n = ctypes.c_int64()
    check(prefix + "_bytes", h, ctypes.byref(n))
    buf = np.zeros(n.value, dtype=np.uint8)
    check(prefix + "_save", h, buf.ctypes.data_as(ctypes.c_void_p), n.value)
    return buf


def _load_blob(prefix, h, blob):
    blob = np.ascontiguousarray(blob, dtype=np.uint8)
    check(prefix + "_load", h, blob.ctypes.data_as(ctypes.c_void_p), len(blob))


def _report(r):
    k = r.candidates
    return dict(tried=[(r.tried[i].fused_ctas_per_sm, r.tried[i].update_ctas_per_sm)
                       for i in range(k)],
                fused_ms=[r.fused_ms[i] for i in range(k)],
                update_ms=[r.update_ms[i] for i in range(k)],
                step_ms=[[r.step_ms[i][j] for j in range(k)] for i in range(k)],
                steps=r.steps,
                chosen=(r.chosen.fused_ctas_per_sm, r.chosen.update_ctas_per_sm))


def tune_save(path):
    """Writes the process-wide launch-shape table (hg_tune_save)."""
    check("hg_tune_save", os.fsencode(path))


def tune_load(path):
    """Merges a saved launch-shape table (hg_tune_load)."""
    check("hg_tune_load", os.fsencode(path))


def tune_clear():
    check("hg_tune_clear")


def kernel_launch_count():
    """Kernels launched by libhg_gpu in this process so far."""
    return int(load().hg_kernel_launch_count())


def set_host_threads(n):
    """Host threads of the library's host loops (zone update, resampling),
    process-wide; 0 restores the default. Results do not depend on it."""
    check("hg_set_host_threads", int(n))


class Context:
    """A device and the CUDA stream all objects of the context run on."""

    def __init__(self, device=0):
        load()
        h = ctypes.c_void_p()
        check("hg_context_create", int(device), ctypes.byref(h))
        self._h = h
        self.device = device

    def synchronize(self):
        check("hg_context_synchronize", self._h)

    def timer_begin(self):
        check("hg_context_timer_begin", self._h)

    def timer_end(self):
        """Milliseconds on the context stream since timer_begin (synchronises)."""
        ms = ctypes.c_double()
        check("hg_context_timer_end", self._h, ctypes.byref(ms))
        return ms.value

    def fence(self):
        """Marks the calls queued so far; see fence_done / fence_wait."""
        f = ctypes.c_int64()
        check("hg_context_fence", self._h, ctypes.byref(f))
        return f.value

    def fence_done(self, fence):
        d = ctypes.c_int32()
        check("hg_context_fence_done", self._h, int(fence), ctypes.byref(d))
        return bool(d.value)

    def fence_wait(self, fence):
        check("hg_context_fence_wait", self._h, int(fence))

    def device_bytes(self):
        b = ctypes.c_int64()
        check("hg_context_device_bytes", self._h, ctypes.byref(b))
        return b.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _mpm_desc(grid_min, grid_max, cell_width, shear_modulus, bulk_modulus, dp_alpha,
              flip_alpha, gravity, planes, basis, precision, capacity):
    d = _capi.MpmDesc()
    d.grid_min[:] = list(map(float, grid_min))
    d.grid_max[:] = list(map(float, grid_max))
    d.cell_width = float(cell_width)
    d.basis = int(basis)
    d.precision = int(precision)
    d.shear_modulus = float(shear_modulus)
    d.bulk_modulus = float(bulk_modulus)
    d.dp_alpha = float(dp_alpha)
    d.flip_alpha = float(flip_alpha)
    d.gravity[:] = list(map(float, gravity))
    planes = list(planes)
    d.num_planes = len(planes)
    for k, pl in enumerate(planes):
        x, n = pl[0], pl[1]
        st = pl[2] if len(pl) > 2 else True
        lb = pl[3] if len(pl) > 3 else -np.inf
        d.planes[k].x[:] = list(map(float, x))
        d.planes[k].n[:] = list(map(float, n))
        d.planes[k].sticking = 1 if st else 0
        d.planes[k].lower_bound = float(lb)
    d.capacity = int(capacity)
    return d


def mpm_estimate_bytes(grid_min, grid_max, cell_width, capacity, precision=MIXED,
                       basis=LINEAR):
    """Device bytes an MPM object of this size holds (hg_mpm_estimate_bytes)."""
    d = _mpm_desc(grid_min, grid_max, cell_width, 1.0, 1.0, 0.0, 1.0, (0.0, 0.0), (), basis,
                  precision, capacity)
    b = ctypes.c_int64()
    check("hg_mpm_estimate_bytes", ctypes.byref(d), ctypes.byref(b))
    return b.value


class MPM:
    """Material points + physics grid on the device (mpmgrains2d SimulationState).

    planes: iterable of (x[2], n[2], sticking: bool, lower_bound) like
    MPMStaticPlane. precision: MIXED (FP64 positions, FP32 elsewhere) or FP64.
    """

    def __init__(self, ctx, grid_min, grid_max, cell_width, shear_modulus, bulk_modulus,
                 dp_alpha, flip_alpha, gravity=(0.0, -9.81), planes=(), basis=LINEAR,
                 precision=MIXED, capacity=0):
        self.ctx = ctx
        d = _mpm_desc(grid_min, grid_max, cell_width, shear_modulus, bulk_modulus, dp_alpha,
                      flip_alpha, gravity, planes, basis, precision, capacity)
        h = ctypes.c_void_p()
        check("hg_mpm_create", ctx._h, ctypes.byref(d), ctypes.byref(h))
        self._h = h
        self.precision = precision
        self.basis = basis
        gmin = np.zeros(2)
        gmax = np.zeros(2)
        cc = np.zeros(2, dtype=np.int32)
        check("hg_mpm_grid_info", h, _d(gmin), _d(gmax), _i32(cc))
        self.grid_min, self.grid_max = gmin, gmax
        self.nx, self.ny = int(cc[0]), int(cc[1])
        self.nnodes = (self.nx + 1) * (self.ny + 1)
        self.n = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_mpm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def seed_rectangle(self, rmin, rmax, density, samples_per_dim, vel=(0.0, 0.0), omega=0.0):
        """InitialSimulationState rasterizeRectangle: returns particle arrays."""
        cnt = ctypes.c_int64()
        rmin, rmax, vel = _f64(rmin), _f64(rmax), _f64(vel)
        check("hg_mpm_seed_rectangle", self._h, _d(rmin), _d(rmax), float(density),
              int(samples_per_dim), _d(vel), float(omega), 0, None, None, None, None, None,
              ctypes.byref(cnt))
        n = cnt.value
        q, v = np.zeros((n, 2)), np.zeros((n, 2))
        m, vol, hl = np.zeros(n), np.zeros(n), np.zeros(n)
        check("hg_mpm_seed_rectangle", self._h, _d(rmin), _d(rmax), float(density),
              int(samples_per_dim), _d(vel), float(omega), n, _d(q), _d(v), _d(m), _d(vol),
              _d(hl), ctypes.byref(cnt))
        return dict(q=q, v=v, m=m, vol=vol, hl=hl)

    def seed_rectangle_device(self, rmin, rmax, density, samples_per_dim, vel=(0.0, 0.0),
                              omega=0.0):
        """seed_rectangle + upload with the points generated on the device
        (hg_mpm_seed_rectangle_device); returns the point count."""
        cnt = ctypes.c_int64()
        rmin, rmax, vel = _f64(rmin), _f64(rmax), _f64(vel)
        check("hg_mpm_seed_rectangle_device", self._h, _d(rmin), _d(rmax), float(density),
              int(samples_per_dim), _d(vel), float(omega), ctypes.byref(cnt))
        self.n = cnt.value
        return self.n

    def upload(self, q, v, m, vol, hl=None, be=None, J=None, jh=None, kin=None):
        """MaterialPoints::setPoints. q, v: (N, 2); be: (N, 4) column-major."""
        q, v, m, vol = _f64(q), _f64(v), _f64(m), _f64(vol)
        hl, be, J = _f64(hl), _f64(be), _f64(J)
        jh = None if jh is None else np.ascontiguousarray(jh, dtype=np.int32)
        kin = None if kin is None else np.ascontiguousarray(kin, dtype=np.uint8)
        n = len(m)
        check("hg_mpm_upload", self._h, n, _d(q), _d(v), _d(m), _d(vol), _d(hl), _d(be), _d(J),
              _i32(jh), _u8(kin))
        self.n = n

    def upload_async(self, q, v, m, vol, hl=None):
        """hg_mpm_upload_async: the arrays (float64, C order; page-locked for
        the copy to overlap) must stay alive and unchanged until a fence
        taken after this call is done."""
        for a in (q, v, m, vol) + (() if hl is None else (hl,)):
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("upload_async takes C-contiguous float64 arrays")
        n = len(m)
        check("hg_mpm_upload_async", self._h, n, _d(q), _d(v), _d(m), _d(vol), _d(hl), None,
              None, None, None)
        self.n = n

    def frame_async(self, q=None, v=None):
        """Queue a copy of positions / velocities ((N, 2) float64 arrays) to
        the host; valid once a later fence is done."""
        check("hg_mpm_frame_async", self._h, _d(q), _d(v))

    def download(self):
        n = self.n
        q, v, be = np.zeros((n, 2)), np.zeros((n, 2)), np.zeros((n, 4))
        J = np.zeros(n)
        jh = np.zeros(n, dtype=np.int32)
        check("hg_mpm_download", self._h, _d(q), _d(v), _d(be), _d(J), _i32(jh))
        return dict(q=q, v=v, be=be, J=J, jh=jh)

    def download_into(self, q=None, v=None, be=None, J=None, jh=None):
        """Download into caller-provided (e.g. pinned) buffers."""
        check("hg_mpm_download", self._h, _d(q), _d(v), _d(be), _d(J), _i32(jh))

    def grid(self):
        nn = self.nnodes
        mass = np.zeros(nn)
        vel, acc = np.zeros((nn, 2)), np.zeros((nn, 2))
        if self.precision == FP64:
            mom, mom_new, force = np.zeros((nn, 2)), np.zeros((nn, 2)), np.zeros((nn, 2))
            check("hg_mpm_download_grid", self._h, _d(mass), _d(mom), _d(mom_new), _d(force),
                  _d(vel), _d(acc))
            return dict(mass=mass, mom=mom, mom_new=mom_new, force=force, vel=vel, acc=acc)
        check("hg_mpm_download_grid", self._h, _d(mass), None, None, None, _d(vel), _d(acc))
        return dict(mass=mass, vel=vel, acc=acc)

    def cell_index(self):
        cells = np.zeros((self.n, 2), dtype=np.int32)
        check("hg_mpm_cell_index", self._h, _i32(cells))
        return cells

    # ExplicitIntegrator surface (mpmgrains2d/ExplicitIntegrator.h:8-20)
    def flow(self, dt, nsteps=1):
        check("hg_mpm_step", self._h, float(dt), int(nsteps))

    step = flow

    def flow_zero_phase(self):
        check("hg_mpm_phase0", self._h)

    def flow_first_phase(self, dt):
        check("hg_mpm_phase1", self._h, float(dt))

    def flow_second_phase(self, dt):
        check("hg_mpm_phase2", self._h, float(dt))

    def status(self):
        w = ctypes.c_uint32()
        check("hg_mpm_status", self._h, ctypes.byref(w))
        return w.value

    def clear_status(self):
        check("hg_mpm_clear_status", self._h)

    def profile(self, enable=True):
        check("hg_mpm_profile", self._h, 1 if enable else 0)

    def profile_read(self):
        """(fused G2P/P2G ms, grid-update ms, steps) summed since profile(True)."""
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        check("hg_mpm_profile_read", self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n))
        return a.value, b.value, n.value

    def rebin_count(self):
        c = ctypes.c_int64()
        check("hg_mpm_rebin_count", self._h, ctypes.byref(c))
        return c.value

    def state(self):
        """The device state as a blob (hg_mpm_state_save) for checkpoints."""
        return _save_blob("hg_mpm_state", self._h)

    def load_state(self, blob):
        """Restores a blob saved from an object with the same grid."""
        _load_blob("hg_mpm_state", self._h, blob)
        c = ctypes.c_int64()
        check("hg_mpm_num_particles", self._h, ctypes.byref(c))
        self.n = c.value

    def autotune(self, dt, steps_per_candidate=20):
        """hg_mpm_autotune: times the candidate launch shapes on this scene
        (which advances by all the timed steps) and keeps the fastest."""
        r = _capi.TuneReport()
        check("hg_mpm_autotune", self._h, float(dt), int(steps_per_candidate), ctypes.byref(r))
        return _report(r)

    def launch_shape(self):
        s = _capi.LaunchShape()
        check("hg_mpm_launch_shape", self._h, ctypes.byref(s))
        return s.fused_ctas_per_sm, s.update_ctas_per_sm

    def set_launch_shape(self, fused_ctas_per_sm, update_ctas_per_sm):
        s = _capi.LaunchShape(int(fused_ctas_per_sm), int(update_ctas_per_sm))
        check("hg_mpm_set_launch_shape", self._h, ctypes.byref(s))


class DEM:
    """Circle bodies with the penalty impact-friction map (rigidbody2d)."""

    def __init__(self, ctx, gravity, kn, kt, gamman, gammat, mu, planes=(), cell_scale=1.0,
                 capacity=0, contact_capacity=0, precision=0, drums=()):
        """planes: ((x, y), (nx, ny)) static half-planes; drums: ((x, y), r)
        static drums (RigidBody2DStaticDrum) holding the disks inside."""
        self.ctx = ctx
        d = _capi.DemDesc()
        d.gravity[:] = list(map(float, gravity))
        d.kn, d.kt, d.gamman, d.gammat, d.mu = map(float, (kn, kt, gamman, gammat, mu))
        d.cell_scale = float(cell_scale)
        planes = list(planes)
        d.num_planes = len(planes)
        for k, (x, n) in enumerate(planes):
            d.planes[k].x[:] = list(map(float, x))
            d.planes[k].n[:] = list(map(float, n))
        drums = list(drums)
        if len(drums) > _capi.HG_MAX_DRUMS:
            raise HGError("at most %d drums" % _capi.HG_MAX_DRUMS)
        d.num_drums = len(drums)
        for k, (x, r) in enumerate(drums):
            d.drums[k].x[:] = list(map(float, x))
            d.drums[k].r = float(r)
        d.capacity = int(capacity)
        d.contact_capacity = int(contact_capacity or 8 * max(capacity, 1))
        d.precision = int(precision)
        self.precision = int(precision)
        h = ctypes.c_void_p()
        check("hg_dem_create", ctx._h, ctypes.byref(d), ctypes.byref(h))
        self._h = h
        self.n = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_dem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, q, v, r, m, I, fixed=None):
        """q, v: (N, 3) as (x, y, theta); m = rho pi r^2, I = m r^2 / 2."""
        q, v, r, m, I = map(_f64, (q, v, r, m, I))
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        n = len(r)
        check("hg_dem_upload", self._h, n, _d(q), _d(v), _d(r), _d(m), _d(I), _u8(fx))
        self.n = n

    def upload_relabel(self, q, v, r, m, I, fixed, old_to_new):
        """Upload after a resampling step, keeping the contact history
        renumbered by old_to_new (-1 for removed bodies)."""
        q, v, r, m, I = _f64(q), _f64(v), _f64(r), _f64(m), _f64(I)
        fx = np.ascontiguousarray(fixed, dtype=np.uint8)
        mp = np.ascontiguousarray(old_to_new, dtype=np.int32)
        check("hg_dem_upload_relabel", self._h, len(r), _d(q), _d(v), _d(r), _d(m), _d(I),
              _u8(fx), len(mp), _i32(mp))
        self.n = len(r)

    def edit_async(self, old_to_new, q=None, v=None, r=None, m=None, I=None, fixed=None):
        """hg_dem_edit_async: arrays (float64 C order, page-locked for overlap)
        must stay alive until a later fence is done."""
        mp = np.ascontiguousarray(old_to_new, dtype=np.int32)
        n_add = 0 if r is None else len(r)
        q, v, r, m, I = (None if a is None else _f64(a) for a in (q, v, r, m, I))
        if fixed is not None:
            fixed = np.ascontiguousarray(fixed, dtype=np.uint8)
        check("hg_dem_edit_async", self._h, len(mp), _i32(mp), n_add, _d(q), _d(v), _d(r),
              _d(m), _d(I), _u8(fixed))
        c = ctypes.c_int64()
        check("hg_dem_num_bodies", self._h, ctypes.byref(c))
        self.n = c.value
        return mp

    def frame_async(self, q=None, v=None):
        check("hg_dem_frame_async", self._h, _d(q), _d(v))

    def set_concurrent(self, on=True):
        """hg_dem_set_concurrent: run on a stream of its own."""
        check("hg_dem_set_concurrent", self._h, 1 if on else 0)

    def wait_context(self):
        check("hg_dem_wait_context", self._h)

    def join(self):
        check("hg_dem_join", self._h)

    def state(self):
        """Bodies and contact history as a blob (hg_dem_state_save)."""
        return _save_blob("hg_dem_state", self._h)

    def load_state(self, blob):
        _load_blob("hg_dem_state", self._h, blob)
        c = ctypes.c_int64()
        check("hg_dem_num_bodies", self._h, ctypes.byref(c))
        self.n = c.value

    def set_weights(self, w):
        check("hg_dem_set_weights", self._h, _d(_f64(w)))

    def set_state(self, q=None, v=None):
        check("hg_dem_set_state", self._h, _d(_f64(q)), _d(_f64(v)))

    def download(self):
        q, v = np.zeros((self.n, 3)), np.zeros((self.n, 3))
        check("hg_dem_download", self._h, _d(q), _d(v))
        return q, v

    def download_into(self, q=None, v=None):
        """Download into caller-provided (N, 3) float64 arrays (e.g. pinned)."""
        check("hg_dem_download", self._h, _d(q), _d(v))

    def flow(self, dt, nsteps=1):
        check("hg_dem_step", self._h, float(dt), int(nsteps), 0)

    def flow_with_weights(self, dt, nsteps=1):
        check("hg_dem_step", self._h, float(dt), int(nsteps), 1)

    def num_contacts(self):
        n = ctypes.c_int64()
        check("hg_dem_num_contacts", self._h, ctypes.byref(n))
        return n.value

    def contacts(self):
        cnt = ctypes.c_int64()
        check("hg_dem_download_contacts", self._h, 0, None, ctypes.byref(cnt))
        rec = np.zeros((max(cnt.value, 1), _capi.HG_DEM_RECORD_WIDTH))
        check("hg_dem_download_contacts", self._h, cnt.value, _d(rec), ctypes.byref(cnt))
        return rec[: cnt.value]

    def status(self):
        w = ctypes.c_uint32()
        check("hg_dem_status", self._h, ctypes.byref(w))
        return w.value


def candidate_pairs(ctx, aabb_min, aabb_max):
    """SpatialGrid::getPotentialOverlaps on the device: sorted (i, j), i < j."""
    mn, mx = _f64(aabb_min), _f64(aabb_max)
    n = mn.shape[0]
    cnt = ctypes.c_int64()
    check("hg_dem_candidate_pairs", ctx._h, n, _d(mn), _d(mx), 0, None, ctypes.byref(cnt))
    pairs = np.zeros((max(cnt.value, 1), 2), dtype=np.int32)
    check("hg_dem_candidate_pairs", ctx._h, n, _d(mn), _d(mx), cnt.value, _i32(pairs),
          ctypes.byref(cnt))
    return pairs[: cnt.value]


class Hybrid:
    """HybridGrains2DSim node-node step over an FP64 MPM and a DEM object."""

    HOMOGENIZE_STRESS = 1
    HOMOGENIZE_VELOCITY = 2

    def __init__(self, ctx, mpm, dem):
        self.ctx, self.mpm, self.dem = ctx, mpm, dem
        h = ctypes.c_void_p()
        check("hg_hybrid_create", ctx._h, mpm._h, dem._h, ctypes.byref(h))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_hybrid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt, nsteps=1, homogenize_stress=False, homogenize_velocity=False):
        flags = (1 if homogenize_stress else 0) | (2 if homogenize_velocity else 0)
        check("hg_hybrid_step", self._h, float(dt), int(nsteps), flags)

    def state(self):
        """Homogenised accumulators of the interval (hg_hybrid_state_save)."""
        return _save_blob("hg_hybrid_state", self._h)

    def load_state(self, blob):
        _load_blob("hg_hybrid_state", self._h, blob)

    def clear_homogenized(self):
        check("hg_hybrid_clear_homogenized", self._h)

    def homogenized_into(self, stress, velocity):
        """The interval's homogenised stress (nn, 4) and velocity (nn, 2)
        sums into caller-provided float64 arrays (e.g. pinned)."""
        check("hg_hybrid_download", self._h, None, None, None, None, None, None, None,
              _d(stress), _d(velocity))

    def coupling(self):
        ng, nn_ = ctypes.c_int64(), ctypes.c_int64()
        check("hg_hybrid_num_packed", self._h, ctypes.byref(ng), ctypes.byref(nn_))
        nn = self.mpm.nnodes
        pg = np.zeros(max(ng.value, 1), dtype=np.int32)
        pn = np.zeros(max(nn_.value, 1), dtype=np.int32)
        dm, dp = np.zeros(nn), np.zeros((nn, 2))
        va, aa = np.zeros((nn, 2)), np.zeros((nn, 2))
        hf, hs, hv = np.zeros(nn), np.zeros((nn, 4)), np.zeros((nn, 2))
        check("hg_hybrid_download", self._h, _i32(pg), _i32(pn), _d(dm), _d(dp), _d(va), _d(aa),
              _d(hf), _d(hs), _d(hv))
        return dict(packed_dem=pg[: ng.value], packed_mpm=pn[: nn_.value], dem_mass_grid=dm,
                    dem_mom_grid=dp, v_after=va, at_after=aa, homog_factor=hf, homog_stress=hs,
                    homog_velocity=hv)


class Batch:
    """Independent MIXED MPM scenes stepped together: one grid-update and one
    fused G2P/P2G launch per step for all members (no counterpart in the
    reference, which runs one scene per process)."""

    def __init__(self, ctx, max_members=64):
        self.ctx = ctx
        h = ctypes.c_void_p()
        check("hg_batch_create", ctx._h, int(max_members), ctypes.byref(h))
        self._h = h
        self._members = {}

    def add(self, mpm, dt):
        check("hg_batch_add", self._h, mpm._h, float(dt))
        self._members[id(mpm)] = mpm

    def remove(self, mpm):
        check("hg_batch_remove", self._h, mpm._h)
        self._members.pop(id(mpm), None)

    def __len__(self):
        n = ctypes.c_int32()
        check("hg_batch_size", self._h, ctypes.byref(n))
        return n.value

    def step(self, nsteps=1):
        check("hg_batch_step", self._h, int(nsteps))

    def stats(self):
        """(member-steps, re-sorts, batch steps, host ms inside hg_batch_step,
        of which ms waiting for the device)."""
        a, r, s = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        h, w = ctypes.c_double(), ctypes.c_double()
        check("hg_batch_stats", self._h, ctypes.byref(a), ctypes.byref(r), ctypes.byref(s),
              ctypes.byref(h), ctypes.byref(w))
        return a.value, r.value, s.value, h.value, w.value

    def profile(self, enable=True):
        check("hg_batch_profile", self._h, 1 if enable else 0)

    def autotune(self, steps_per_candidate=20):
        """hg_batch_autotune: times the candidate launch shapes on the
        current members (which advance) and records the fastest."""
        r = _capi.TuneReport()
        check("hg_batch_autotune", self._h, int(steps_per_candidate), ctypes.byref(r))
        return _report(r)

    def launch_shape(self):
        s = _capi.LaunchShape()
        check("hg_batch_launch_shape", self._h, ctypes.byref(s))
        return s.fused_ctas_per_sm, s.update_ctas_per_sm

    def profile_read(self):
        """dict of summed ms per phase (resort, table, update, fused) and steps."""
        v = [ctypes.c_double() for _ in range(4)]
        n = ctypes.c_int64()
        check("hg_batch_profile_read", self._h, *[ctypes.byref(x) for x in v], ctypes.byref(n))
        return dict(resort_ms=v[0].value, table_ms=v[1].value, update_ms=v[2].value,
                    fused_ms=v[3].value, steps=n.value)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_batch_destroy(self._h)
            self._h = None
        self._members = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


CONTINUUM, DISCRETE, HYBRID = 0, 1, 2
(ZONES_RECONCILIATION, ZONES_DIRECT_TRANSITION, ZONES_INNER_CONTINUUM,
 ZONES_INNER_CONTINUUM_EXCLUDING_DIRECT, ZONES_LEVEL_SET_HYBRID) = range(5)
ZONES_MPM, ZONES_DEM = 0, 1


class Zones:
    """Zone labels of the hybrid method (ZoneTools), host code of libhg_gpu
    run at the resampling interval on positions copied from the device."""

    def __init__(self, mpm_grid_min, mpm_cell_width, mpm_cells, level_set_cell_width,
                 phi_window_size, phi_samples_per_cell_side, phi_threshold, rzone_level_set,
                 rzone_half_thickness, allow_direct_transitions=False):
        d = _capi.ZonesDesc()
        d.mpm_grid_min[:] = list(map(float, mpm_grid_min))
        d.mpm_cell_width = float(mpm_cell_width)
        d.mpm_cells[:] = [int(mpm_cells[0]), int(mpm_cells[1])]
        d.level_set_cell_width = float(level_set_cell_width)
        d.allow_direct_transitions = 1 if allow_direct_transitions else 0
        d.phi_samples_per_cell_side = int(phi_samples_per_cell_side)
        d.phi_window_size = float(phi_window_size)
        d.phi_threshold = float(phi_threshold)
        d.rzone_level_set = float(rzone_level_set)
        d.rzone_half_thickness = float(rzone_half_thickness)
        h = ctypes.c_void_p()
        check("hg_zones_create", ctypes.byref(d), ctypes.byref(h))
        self._h = h
        ls, mc = np.zeros(2, dtype=np.int32), np.zeros(2, dtype=np.int32)
        check("hg_zones_grid_info", h, _i32(ls), _i32(mc))
        self.level_set_cells = (int(ls[0]), int(ls[1]))
        self.mpm_cells = (int(mc[0]), int(mc[1]))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_zones_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, q, radius, fixed=None, points=None):
        """q: (n, 3) disk states (x, y, theta); points: (m, 2) MPM positions."""
        q, radius = _f64(q), _f64(radius)
        fixed = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        points = None if points is None else _f64(points)
        check("hg_zones_update", self._h, len(radius), _d(q), _d(radius), _u8(fixed),
              0 if points is None else len(points), _d(points))

    def fields(self):
        nx, ny = self.level_set_cells
        phi, dist = np.zeros(nx * ny), np.zeros((nx + 1) * (ny + 1))
        ls = np.zeros(nx * ny, dtype=np.int32)
        mpm = np.zeros(self.mpm_cells[0] * self.mpm_cells[1], dtype=np.int32)
        check("hg_zones_fields", self._h, _d(phi), _d(dist), _i32(ls), _i32(mpm))
        return dict(phi=phi, dist=dist, ls=ls, mpm=mpm)

    def set_labels(self, mpm):
        check("hg_zones_set_labels", self._h, _i32(np.ascontiguousarray(mpm, dtype=np.int32)))

    def zone_list(self, which):
        n = ctypes.c_int64()
        check("hg_zones_list", self._h, int(which), 0, None, None, ctypes.byref(n))
        boxes, cells = np.zeros((n.value, 4)), np.zeros((n.value, 2), dtype=np.int32)
        check("hg_zones_list", self._h, int(which), n.value, _d(boxes), _i32(cells),
              ctypes.byref(n))
        return boxes, cells

    def to_delete(self, kind, x, stride, fixed=None):
        x = _f64(x)
        n = x.size // stride
        ids = np.zeros(max(n, 1), dtype=np.int32)
        c = ctypes.c_int64()
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        check("hg_zones_to_delete", self._h, int(kind), n, _d(x), int(stride), _u8(fx), n,
              _i32(ids), ctypes.byref(c))
        return ids[:c.value]

    def weights(self, kind, x, stride):
        x = _f64(x)
        n = x.size // stride
        w = np.zeros(n)
        check("hg_zones_weights", self._h, int(kind), n, _d(x), int(stride), _d(w))
        return w

    def boundary_samples(self):
        c = ctypes.c_int64()
        check("hg_zones_boundary_samples", self._h, ctypes.byref(c))
        return c.value


def disk_box_area(x0, x1, y0, y1, cx, cy, r):
    """Area of a disk inside an axis-aligned box (hg_zones_disk_box_area)."""
    return _capi.load().hg_zones_disk_box_area(x0, x1, y0, y1, cx, cy, r)


class Resampler:
    """The hybrid method's resampling step (ResamplingTools), host code of
    libhg_gpu run at the resampling interval after Zones.update."""

    def __init__(self, zones_desc_args, mpm_grid_max, basis, initial_particle_size,
                 material_density, dem_r_mean, dem_r_std, rho_dem, kappa, mu,
                 newly_inserted_continuum_stress_free=False, homogenize_stress=False,
                 homogenize_velocity=False):
        d = _capi.ResamplerDesc()
        z = d.zones
        (gmin, cw, cells, ls_cw, window, samples, thr, level, half, direct) = zones_desc_args
        z.mpm_grid_min[:] = list(map(float, gmin))
        z.mpm_cell_width = float(cw)
        z.mpm_cells[:] = [int(cells[0]), int(cells[1])]
        z.level_set_cell_width = float(ls_cw)
        z.phi_window_size = float(window)
        z.phi_samples_per_cell_side = int(samples)
        z.phi_threshold = float(thr)
        z.rzone_level_set = float(level)
        z.rzone_half_thickness = float(half)
        z.allow_direct_transitions = 1 if direct else 0
        d.mpm_grid_max[:] = list(map(float, mpm_grid_max))
        d.basis = int(basis)
        d.newly_inserted_continuum_stress_free = 1 if newly_inserted_continuum_stress_free else 0
        d.initial_particle_size = float(initial_particle_size)
        d.material_density = float(material_density)
        d.dem_r_mean, d.dem_r_std, d.rho_dem = float(dem_r_mean), float(dem_r_std), float(rho_dem)
        d.kappa, d.mu = float(kappa), float(mu)
        d.homogenize_stress = 1 if homogenize_stress else 0
        d.homogenize_velocity = 1 if homogenize_velocity else 0
        h = ctypes.c_void_p()
        check("hg_resampler_create", ctypes.byref(d), ctypes.byref(h))
        self._h = h
        self.nodes = (int(cells[0]) + 1) * (int(cells[1]) + 1)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().hg_resampler_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_points(self, q0, q, v, m, vol, m0, vol0, hl, be, J, jh=None, kin=None):
        a = [_f64(x) for x in (q0, q, v, m, vol, m0, vol0, hl, be, J)]
        jh = None if jh is None else np.ascontiguousarray(jh, dtype=np.int32)
        kin = None if kin is None else np.ascontiguousarray(kin, dtype=np.uint8)
        check("hg_resampler_set_points", self._h, len(a[3]), *[_d(x) for x in a], _i32(jh),
              _u8(kin))

    def set_grains(self, q0, q, v, radius, M0, fixed=None):
        a = [_f64(x) for x in (q0, q, v, radius, M0)]
        fixed = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        check("hg_resampler_set_grains", self._h, len(a[3]), *[_d(x) for x in a], _u8(fixed))

    def set_homogenized(self, stress=None, velocity=None):
        check("hg_resampler_set_homogenized", self._h, _d(_f64(stress) if stress is not None else None),
              _d(_f64(velocity) if velocity is not None else None))

    def run(self, zones):
        check("hg_resampler_run", self._h, zones._h)

    def stats(self):
        n, g = ctypes.c_int64(), ctypes.c_int64()
        s = _capi.ResamplerStats()
        check("hg_resampler_counts", self._h, ctypes.byref(n), ctypes.byref(g), ctypes.byref(s))
        return n.value, g.value, dict(points_inserted=s.points_inserted,
                                      grains_inserted=s.grains_inserted,
                                      points_deleted=s.points_deleted,
                                      grains_deleted=s.grains_deleted,
                                      ms_insert_grains=s.ms_insert_grains,
                                      ms_insert_points=s.ms_insert_points,
                                      ms_point_grids=s.ms_point_grids,
                                      ms_quantities=s.ms_quantities,
                                      ms_delete=s.ms_delete)

    def points(self, alloc=np.empty):
        """The points after the step; alloc(shape, dtype) makes the arrays
        (e.g. ``pinned``); every element is written by the call."""
        n, _, _ = self.stats()
        f = lambda shape, dtype=np.float64: alloc(shape, dtype=dtype)  # noqa: E731
        out = dict(q0=f((n, 2)), q=f((n, 2)), v=f((n, 2)), m=f(n), vol=f(n), m0=f(n),
                   vol0=f(n), w=f(n), hl=f(n), be=f((n, 4)), J=f(n),
                   jh=f(n, dtype=np.int32), kin=f(n, dtype=np.uint8))
        check("hg_resampler_get_points", self._h, *[_d(out[k]) for k in
              ("q0", "q", "v", "m", "vol", "m0", "vol0", "w", "hl", "be", "J")],
              _i32(out["jh"]), _u8(out["kin"]))
        return out

    def grains(self):
        _, g, _ = self.stats()
        k = ctypes.c_int64()
        check("hg_resampler_dem_map_size", self._h, ctypes.byref(k))
        out = dict(q0=np.zeros((g, 3)), q=np.zeros((g, 3)), v=np.zeros((g, 3)), r=np.zeros(g),
                   M0=np.zeros((g, 3)), w=np.zeros(g), fixed=np.zeros(g, dtype=np.uint8),
                   old_to_new=np.zeros(k.value, dtype=np.int32))
        check("hg_resampler_get_grains", self._h, *[_d(out[x]) for x in
              ("q0", "q", "v", "r", "M0", "w")], _u8(out["fixed"]), _i32(out["old_to_new"]))
        return out

    def rng_state(self):
        """The random streams' state (hg_resampler_rng_save)."""
        return _save_blob("hg_resampler_rng", self._h)

    def load_rng_state(self, blob):
        _load_blob("hg_resampler_rng", self._h, blob)

    def random_u32(self):
        return _capi.load().hg_resampler_random_u32(self._h)

    def random_f32(self):
        return _capi.load().hg_resampler_random_f32(self._h)

    def random_radius(self):
        return _capi.load().hg_resampler_random_radius(self._h)
