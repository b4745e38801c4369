"""Hybrid MPM/DEM simulation with the resampling interval (HybridGrains2DSim).

The node-node step runs on the device (``Hybrid.step``); the zone labels and
the resampling step run on the host every ``avoid_a_void_freq + 1`` steps on
state copied from the device, and the result is copied back
(HybridGrains2DSim.cpp:116-227 and 301-559):

* before the first step, the resampling runs once (the reference calls its
  update twice; the second call only counts), from labels seeded by where
  the material points are (see _seed_labels);
* after every step the counter advances; when it wraps, the device
  accumulation of the homogenised stress and velocity is finalised (1/freq),
  the zones and the resampling step run, points and grains are uploaded (the
  DEM contact history renumbered), and the accumulators are cleared.

``precision=MIXED`` runs the MPM bulk in FP32 with FP64 positions (the
coupling exchange is still formed in FP64) and, unless ``dem_precision`` says
otherwise, the DEM contact law in FP32 with FP64 positions and pairwise
differences; the default is the FP64 step of both, the reference's
arithmetic.

Host copies kept between intervals: reference positions q0, initial masses
and volumes (m0, volume0) and half widths of the points; reference
positions, radii and initial masses of the grains.

The homogenised fields are accumulated once per device step, so at a
resampling step the finalised field has one term less than the reference's,
which accumulates the current step a second time inside the branch.
"""
import threading
import time

import numpy as np

from . import DEM, FP64, MPM, Hybrid, Resampler, Zones, pinned, scene_xml, scenes


class HybridSim:
    def __init__(self, ctx, scene, basis=None, point_headroom=2.0, grain_headroom=3.0,
                 precision=FP64, dem_precision=None):
        cfg, sc, dp = scene["mpm"], scene["dem"], scene["dem_params"]
        zs, rs = scene["zones"], scene["resampling"]
        self.ctx, self.cfg, self.dt = ctx, cfg, cfg["dt"]
        if basis is None:  # the continuum scene's basis, uGIMP where it names none
            basis = 0 if cfg.get("basis") == "linear" else 1
        # scenes read from the reference's files seed every rectangle with its
        # velocity; the library's column scenes seed one at rest
        p = scene_xml.seed_points(cfg) if "rectangles" in cfg else scenes.seed_column_points(cfg)
        n, nd = len(p["m"]), len(sc["r"])
        gravity = cfg.get("gravity", scenes.GRAVITY)
        self._cap = dict(points=int(point_headroom * n) + 1024,
                         grains=int(grain_headroom * nd) + 1024)
        self.mpm = MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                       cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], gravity,
                       cfg["planes"], basis=basis, precision=precision,
                       capacity=self._cap["points"])
        self.mpm.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
        # the discrete scene's planes, else the continuum's walls for the grains too
        planes = dp.get("planes") or [(pl[0], pl[1]) for pl in cfg["planes"]]
        # (the spatial grid's cell is one mean diameter in hybrid runs, whatever
        # the discrete scene's cell_scale)
        self.dem = DEM(ctx, dp.get("gravity", gravity), dp["kn"], dp["kt"], dp["gamman"],
                       dp["gammat"], dp["mu"], planes, capacity=self._cap["grains"],
                       precision=precision if dem_precision is None else dem_precision)
        self.dem.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
        self.hyb = Hybrid(ctx, self.mpm, self.dem)
        g = self.mpm
        zargs = (g.grid_min, cfg["h"], (g.nx, g.ny), zs["level_set_cell_width"],
                 zs["phi_window_size"], zs["phi_samples_per_cell_side"], zs["phi_threshold"],
                 zs["rzone_level_set"], zs["rzone_half_thickness"],
                 zs["allow_direct_transitions"])
        self.zones = Zones(*zargs[:-1], allow_direct_transitions=zargs[-1])
        self.res = Resampler(zargs, g.grid_max, basis, cfg["h"] / cfg["samples_per_dim"],
                             cfg["rho"], rs["dem_r_mean"], rs["dem_r_std"], rs["rho_dem"],
                             cfg["bulk_modulus"], cfg["shear_modulus"],
                             rs["newly_inserted_continuum_stress_free"],
                             rs["homogenize_stress"], rs["homogenize_velocity"])
        self.freq = rs["avoid_a_void_freq"]
        self.hom = (rs["homogenize_stress"], rs["homogenize_velocity"])
        # host-side state kept between intervals
        self.P = dict(q0=p["q"].copy(), m0=p["m"].copy(), vol0=p["vol"].copy(), hl=p["hl"].copy(),
                      w=np.ones(n))
        self.G = dict(q0=sc["q"].copy(), r=sc["r"].copy(),
                      M0=np.stack([sc["m"], sc["m"], sc["I"]], axis=1), fixed=sc["fixed"].copy(),
                      w=np.ones(nd))
        self.counter = 0
        self.started = False
        self.resamplings = 0
        self.steps = 0
        self.stats = []
        # host seconds of the resampling intervals by phase: device->host
        # copies, zone update (with the resampler's inputs set alongside),
        # resampling proper, host->device uploads
        self.host_s = dict(download=0.0, zones=0.0, resampling=0.0, upload=0.0)
        # page-locked host arrays of the interval's transfers, sized for the
        # objects' capacities and kept for the simulation's life (the
        # library's kernels read and write them in place)
        self._cap["nodes"] = self.mpm.nnodes
        self._pin = {}
        # (all allocated here: page-locking is slow and would land in an
        # interval otherwise)
        for key, w, dt_ in (("pq", 2, np.float64), ("pv", 2, np.float64),
                            ("pbe", 4, np.float64), ("pJ", 1, np.float64),
                            ("pjh", 1, np.int32), ("gq", 3, np.float64), ("gv", 3, np.float64),
                            ("nhs", 4, np.float64), ("nhv", 2, np.float64), ("pmw", 1, np.float64),
                            ("pvw", 1, np.float64)):
            self._pinned(key, (1, w), dt_)
        for parity in (0, 1):
            for k, (w, dt_) in enumerate(((2, np.float64),) * 3 + ((1, np.float64),) * 6 +
                                         ((4, np.float64), (1, np.float64), (1, np.int32),
                                          (1, np.uint8))):
                self._pinned("p%d_%d" % (parity, k), (1, w), dt_)

    def _pinned(self, key, shape, dtype=np.float64):
        """A page-locked host array of this shape, a view of the key's buffer
        (allocated once, for the capacity of the rows' kind: key's first
        letter p, g or n for points, grains or nodes)."""
        shape = (shape,) if np.isscalar(shape) else tuple(shape)
        n = int(np.prod(shape))
        b = self._pin.get(key)
        if b is None or b.size < n or b.dtype != np.dtype(dtype):
            per_row = n // shape[0] if shape[0] else 1
            kind = {"p": "points", "g": "grains", "n": "nodes"}[key[0]]
            b = pinned(max(n, per_row * self._cap[kind], 1), dtype)
            self._pin[key] = b
        return b[:n].reshape(shape)

    def _resample(self):
        clock = time.perf_counter
        t0 = clock()
        n, nd = self.mpm.n, self.dem.n
        st = dict(q=self._pinned("pq", (n, 2)), v=self._pinned("pv", (n, 2)),
                  be=self._pinned("pbe", (n, 4)), J=self._pinned("pJ", n),
                  jh=self._pinned("pjh", n, np.int32))
        self.mpm.download_into(st["q"], st["v"], st["be"], st["J"], st["jh"])
        q3, v3 = self._pinned("gq", (nd, 3)), self._pinned("gv", (nd, 3))
        self.dem.download_into(q3, v3)
        P, G = self.P, self.G
        nn = self.mpm.nnodes
        t1 = clock()
        # the zone update (positions only) runs on a second host thread
        # while this one reads the homogenised fields and hands the
        # interval's arrays to the resampler (the two meet at run)
        failed = []

        def zone_update():
            try:
                self.zones.update(q3, G["r"], G["fixed"], st["q"])
            except Exception as e:  # re-raised on this thread below
                failed.append(e)
        zt = threading.Thread(target=zone_update)
        zt.start()
        try:
            hs, hv = np.zeros((nn, 4)), np.zeros((nn, 2))
            if self.hom[0] or self.hom[1]:
                hs, hv = self._pinned("nhs", (nn, 4)), self._pinned("nhv", (nn, 2))
                self.hyb.homogenized_into(hs, hv)
                np.divide(hs, self.freq, out=hs)
                np.divide(hv, self.freq, out=hv)
            mw, vw = self._pinned("pmw", n), self._pinned("pvw", n)
            np.multiply(P["m0"], P["w"], out=mw)
            np.multiply(P["vol0"], P["w"], out=vw)
            self.res.set_points(P["q0"], st["q"], st["v"], mw, vw,
                                P["m0"], P["vol0"], P["hl"], st["be"], st["J"], st["jh"])
            self.res.set_grains(G["q0"], q3, v3, G["r"], G["M0"], G["fixed"])
            self.res.set_homogenized(hs, hv)
        finally:
            zt.join()
        if failed:
            raise failed[0]
        t2 = clock()
        self.res.run(self.zones)
        # the new points in page-locked arrays, two sets used in turn (the
        # previous interval's stay valid until this one has read them)
        order = iter(range(64))
        parity = self.resamplings % 2
        a = self.res.points(lambda shape, dtype=np.float64: self._pinned(
            "p%d_%d" % (parity, next(order)), shape, dtype))
        # (points beyond the MPM capacity fail at the upload below; their
        # arrays are then sized as requested)
        b = self.res.grains()
        t3 = clock()
        self.mpm.upload(a["q"], a["v"], a["m"], a["vol"], a["hl"], a["be"], a["J"], a["jh"])
        self.dem.upload_relabel(b["q"], b["v"], b["r"], b["M0"][:, 0], b["M0"][:, 2], b["fixed"],
                                b["old_to_new"])
        self.dem.set_weights(b["w"])
        t4 = clock()
        for k, dt_ in (("download", t1 - t0), ("zones", t2 - t1), ("resampling", t3 - t2),
                       ("upload", t4 - t3)):
            self.host_s[k] += dt_
        self.P = dict(q0=a["q0"], m0=a["m0"], vol0=a["vol0"], hl=a["hl"], w=a["w"])
        self.G = dict(q0=b["q0"], r=b["r"], M0=b["M0"], fixed=b["fixed"], w=b["w"])
        self.hyb.clear_homogenized()
        self.resamplings += 1
        self.stats.append(self.res.stats()[2])

    def _update(self):
        """updateHybridStates_poorman's counter (HybridGrains2DSim.cpp:301-559)."""
        if self.counter == 0:
            self._resample()
        elif self.counter >= self.freq:
            self.counter = -1
        self.counter += 1

    def _seed_labels(self):
        """Both methods are seeded (the reference discards the material
        points at initialisation and grows the continuum from the grains by
        resampling, HybridGrains2DSim.cpp:55): cells holding material points
        start as continuum and the others as discrete, so the first update's
        hysteresis keeps the bulk continuous and the grains discrete."""
        from . import CONTINUUM, DISCRETE
        g = self.mpm
        q = g.download()["q"]
        i = np.floor((q[:, 0] - g.grid_min[0]) / self.cfg["h"]).astype(np.int64)
        j = np.floor((q[:, 1] - g.grid_min[1]) / self.cfg["h"]).astype(np.int64)
        ok = (i >= 0) & (j >= 0) & (i < g.nx) & (j < g.ny)
        labels = np.full(g.nx * g.ny, DISCRETE, dtype=np.int32)
        labels[j[ok] * g.nx + i[ok]] = CONTINUUM
        self.zones.set_labels(labels)

    def step(self, nsteps):
        if not self.started:  # the initial resampling (HybridGrains2DSim.cpp:120-128)
            self._seed_labels()
            self._update()
            self._update()
            self.started = True
        done = 0
        while done < nsteps:
            # device steps up to the next resampling call
            run = 1 if self.counter == 0 else min(nsteps - done, self.freq + 1 - self.counter)
            run = max(run, 1)
            self.hyb.step(self.dt, run, *self.hom)
            for _ in range(run - 1):
                self.counter += 1  # calls that only count
            self._update()
            done += run
            self.steps += run

    def counts(self):
        return self.mpm.n, self.dem.n

    def save(self, path):
        """Checkpoint: the device objects' state, the zone labels, the
        resampler's random streams and the host arrays of the interval."""
        from . import checkpoint
        arrays = dict(mpm=self.mpm.state(), dem=self.dem.state(), hybrid=self.hyb.state(),
                      rng=self.res.rng_state(), labels=self.zones.fields()["mpm"])
        for k, v in self.P.items():
            arrays["P." + k] = v
        for k, v in self.G.items():
            arrays["G." + k] = v
        meta = dict(counter=self.counter, started=self.started, resamplings=self.resamplings,
                    steps=self.steps, stats=self.stats)
        checkpoint.write(path, arrays, meta)

    def restore(self, path):
        """Resumes from ``save`` into a simulation built from the same scene."""
        from . import checkpoint
        arrays, meta = checkpoint.read(path)
        self.mpm.load_state(arrays["mpm"])
        self.dem.load_state(arrays["dem"])
        self.hyb.load_state(arrays["hybrid"])
        self.res.load_rng_state(arrays["rng"])
        self.zones.set_labels(arrays["labels"])
        self.P = {k[2:]: v for k, v in arrays.items() if k.startswith("P.")}
        self.G = {k[2:]: v for k, v in arrays.items() if k.startswith("G.")}
        self.counter = meta["counter"]
        self.started = meta["started"]
        self.resamplings = meta["resamplings"]
        self.steps = meta["steps"]
        self.stats = list(meta["stats"])
