"""Serving loop: many column-collapse requests on one GPU, continuously batched.

No counterpart in the reference (its CLIs run one scene per process). A
request is a granular-column scene that runs ``steps`` MPM steps and returns
a frame every ``frame_every`` steps. The loop

* admits arrived requests first come, first served while their device
  footprint (``hg_mpm_estimate_bytes``) fits the budget and a batch slot is
  free; a request that does not fit waits at the head of the queue;
* creates each admitted scene on the device from its geometry (no host
  point data) and keeps it resident;
* steps all resident scenes together
  (``hg_batch_step``: one grid-update and one fused G2P/P2G launch per step);
* admits new requests at chunk boundaries (every ``frame_every`` steps), at
  most ``admit_per_chunk`` per chunk, so work that arrives while others run
  joins the running batch;
* queues each frame's copy to page-locked host memory and a fence behind the
  chunk, and hands frames over once the fence is done, keeping at most
  ``depth`` chunks queued on the device;
* records for each request its arrival, admission and completion times.

A request may carry a DEM pile (disks of the rigidbody2d penalty map) beside
its MPM column. The piles of all resident requests share one DEM object, each
in its own lane (shifted LANE metres along x, so that piles never meet and the
broadphase hash keeps them apart); a request's disks are a contiguous range of
bodies. Piles join and leave at chunk boundaries through one edit of the DEM
object per chunk (stable compaction of the remaining bodies, which renumbers
their contact history, then the new piles appended), and the whole body array
is copied once per chunk for the frames.

The scheduling is separate from the device (``Backend``) so that admission
and ordering can be tested without a GPU.
"""
import collections
import math
import time

import numpy as np

from . import scenes


class Request:
    __slots__ = ("rid", "arrival", "cfg", "npoints", "steps", "frame_every", "dt",
                 "admitted", "finished", "frames", "footprint", "issued", "ndisks", "aspect")

    def __init__(self, rid, arrival, cfg, npoints, steps=2000, frame_every=100, dt=1.0e-5,
                 ndisks=0, aspect=1.0):
        self.rid = rid
        self.arrival = arrival
        self.cfg = cfg
        self.npoints = npoints
        self.steps = steps
        self.frame_every = frame_every
        self.dt = dt
        self.admitted = None
        self.finished = None
        # per frame: (step, (front x of the column, front x of the pile in its
        # lane or None without disks))
        self.frames = []
        self.footprint = 0
        self.issued = 0   # frames queued on the device
        self.ndisks = ndisks  # disks of the request's DEM pile
        self.aspect = aspect

    def copy(self, arrival=None):
        """A fresh request for the same scene (no frames or times)."""
        return Request(self.rid, self.arrival if arrival is None else arrival, self.cfg,
                       self.npoints, self.steps, self.frame_every, self.dt, self.ndisks,
                       self.aspect)

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def column_requests(n=256, rate=50.0, seed=2024, steps=2000, frame_every=100,
                    nmin=2.0e3, nmax=2.0e5, dem_max=0.2):
    """Seeded request stream: exponential inter-arrival gaps at ``rate``/s,
    aspect ratio U[0.5, 4], point count log-uniform in [nmin, nmax],
    friction angle U[20, 40] degrees, and a DEM pile of U[0, dem_max] times
    the point count in disks."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(n):
        aspect = rng.uniform(0.5, 4.0)
        npts = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        phi = rng.uniform(20.0, 40.0)
        frac = rng.uniform(0.0, dem_max)
        cfg = scenes.serving_column(npts, aspect, phi)
        npoints = len(scenes.seed_column_points(cfg)["m"])
        out.append(Request(i, float(arrivals[i]), cfg, npoints, steps, frame_every,
                           cfg["dt"], int(round(frac * npoints)), aspect))
    return out


LANE = 10.0  # m between the DEM piles of the scenes sharing one DEM object


def dem_pile(req, lane):
    """The request's DEM pile (the DEM column's disks: r U[0.9, 1.1] mm, hex
    pitch 2.2 mm, rho 2600) on the floor with the request's aspect ratio,
    shifted to its lane."""
    per_row = max(4, int(round(math.sqrt(max(req.ndisks, 1) / req.aspect))))
    return scenes.dem_column(n=req.ndisks, per_row=per_row, seed=1000 + req.rid,
                             x0=lane * LANE)


def dem_for_piles(ctx, capacity, precision=None):
    """A DEM object for piles: the penalty parameters of the DEM column and
    the floor (y = 0) as the only plane; the contact law in mixed precision
    (FP32 with FP64 positions and pair differences) unless precision says
    otherwise."""
    from . import DEM, MIXED
    p = scenes.dem_params()
    return DEM(ctx, scenes.GRAVITY, p["kn"], p["kt"], p["gamman"], p["gammat"], p["mu"],
               [((0.0, 0.0), (0.0, 1.0))], capacity=capacity,
               contact_capacity=4 * max(capacity, 1),
               precision=MIXED if precision is None else precision)


def frame_diff(a, b):
    """Largest difference of the fronts of two frames (column and pile)."""
    (ma, da), (mb, db) = a, b
    d = abs(ma - mb)
    if da is not None or db is not None:
        d = max(d, abs(da - db))
    return d


class Backend:
    """Device operations the loop needs (implemented by DeviceBackend)."""

    def footprint(self, req):
        raise NotImplementedError

    def can_open(self, req):  # room for the request besides its footprint
        return True

    def open(self, req):  # create the scene and join the batch
        raise NotImplementedError

    def step(self, nsteps):
        raise NotImplementedError

    def frame(self, req, slot):  # queue a frame copy into slot
        raise NotImplementedError

    def leave(self, req):  # leave the batch (state stays until close)
        raise NotImplementedError

    def fence(self):
        raise NotImplementedError

    def fence_done(self, f):
        raise NotImplementedError

    def fence_wait(self, f):
        raise NotImplementedError

    def read_frame(self, req, slot):  # after the fence: the frame's summary
        raise NotImplementedError

    def close(self, req):  # release device state and host buffers
        raise NotImplementedError


class Server:
    def __init__(self, backend, budget_bytes, max_members=256, depth=3, admit_per_chunk=16,
                 clock=time.perf_counter, sleep=time.sleep):
        self.b = backend
        self.budget = int(budget_bytes)
        self.max_members = max_members
        self.depth = depth
        # scenes created per chunk: creation overlaps with the chunks queued
        # on the device instead of delaying the first one
        self.admit_per_chunk = admit_per_chunk
        self.clock = clock
        self.sleep = sleep
        self.resident = 0
        self.peak_resident = 0
        self.peak_members = 0
        self.chunks = 0

    def run(self, requests):
        """Serve ``requests`` (arrival times in seconds from the start);
        returns them with admission/completion times and frames filled in."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        pending.reverse()  # pop() gives the earliest
        waiting = collections.deque()
        active = []        # admitted, still stepping
        inflight = collections.deque()  # (fence, [(req, frame_no, step)], finished reqs)
        closing = []       # (fence, req): left the batch, closed once fence done
        t0 = self.clock()
        for r in requests:
            r.footprint = self.b.footprint(r)
            if r.footprint > self.budget:
                raise ValueError(f"request {r.rid} needs {r.footprint} bytes, "
                                 f"over the budget of {self.budget}")
        chunk = None
        while pending or waiting or active or inflight:
            now = self.clock() - t0
            while pending and pending[-1].arrival <= now:
                waiting.append(pending.pop())
            # admission: FIFO, by footprint and free slots
            admitted = 0
            while waiting and len(active) < self.max_members and admitted < self.admit_per_chunk \
                    and self.resident + waiting[0].footprint <= self.budget \
                    and self.b.can_open(waiting[0]):
                admitted += 1
                r = waiting.popleft()
                self.b.open(r)
                r.admitted = self.clock() - t0
                active.append(r)
                self.resident += r.footprint
            self.peak_resident = max(self.peak_resident, self.resident)
            self.peak_members = max(self.peak_members, len(active))
            if active:
                fe = active[0].frame_every
                if chunk is None:
                    chunk = fe
                # keep at most depth chunks queued on the device
                while len(inflight) >= self.depth:
                    self._retire(inflight.popleft(), t0, closing, wait=True)
                self.b.step(chunk)
                self.chunks += 1
                frames, done = [], []
                for r in active:
                    k = r.issued
                    r.issued += 1
                    step = (k + 1) * chunk
                    self.b.frame(r, k % (self.depth + 1))
                    frames.append((r, k, step))
                    if step >= r.steps:
                        done.append(r)
                for r in done:
                    active.remove(r)
                    self.b.leave(r)
                f = self.b.fence()
                inflight.append((f, frames, done))
            # hand over every chunk the device has finished
            while inflight and (self.b.fence_done(inflight[0][0]) or not active):
                self._retire(inflight.popleft(), t0, closing, wait=True)
            self._close_finished(closing)
            if not active and not inflight and not waiting and pending:
                gap = pending[-1].arrival - (self.clock() - t0)
                if gap > 0:
                    self.sleep(gap)
        for f, r in closing:
            self.b.fence_wait(f)
            self.b.close(r)
        self.makespan = self.clock() - t0
        return requests

    def _retire(self, item, t0, closing, wait):
        f, frames, done = item
        if wait:
            self.b.fence_wait(f)
        for (r, k, step) in frames:
            r.frames.append((step, self.b.read_frame(r, k % (self.depth + 1))))
        now = self.clock() - t0
        for r in done:
            r.finished = now
            self.resident -= r.footprint
            closing.append((f, r))

    def _close_finished(self, closing):
        keep = []
        for f, r in closing:
            if self.b.fence_done(f):
                self.b.close(r)
            else:
                keep.append((f, r))
        closing[:] = keep


def shard_requests(requests, rank, world):
    """The requests rank serves out of world ranks, one GPU each: every
    world-th request in arrival order (scenes are independent, so the ranks
    exchange nothing while they serve)."""
    ordered = sorted(requests, key=lambda r: (r.arrival, r.rid))
    return ordered[rank::world]


def summary_parts(requests, makespan):
    """The raw figures of one rank's run, for summary_of_parts."""
    return dict(latencies=[float(r.latency) for r in requests],
                waits=[float(r.admitted - r.arrival) for r in requests],
                particle_steps=float(sum(r.npoints * r.steps for r in requests)),
                disk_steps=float(sum(r.ndisks * r.steps for r in requests)),
                makespan_s=float(makespan))


def summary_of_parts(parts):
    """Latency percentiles over all ranks' requests; throughput over the
    slowest rank's makespan."""
    lat = np.array([x for p in parts for x in p["latencies"]])
    wait = np.array([x for p in parts for x in p["waits"]])
    psteps = sum(p["particle_steps"] for p in parts)
    dsteps = sum(p["disk_steps"] for p in parts)
    makespan = max(p["makespan_s"] for p in parts)
    return dict(requests=len(lat), p50_latency_s=float(np.percentile(lat, 50)),
                p99_latency_s=float(np.percentile(lat, 99)),
                max_latency_s=float(lat.max()),
                p50_admission_wait_s=float(np.percentile(wait, 50)),
                p99_admission_wait_s=float(np.percentile(wait, 99)),
                makespan_s=makespan, particle_steps=psteps,
                particle_steps_per_s=psteps / makespan,
                disk_steps=dsteps, disk_steps_per_s=dsteps / makespan,
                requests_per_s=len(lat) / makespan)


def summary(requests, makespan):
    return summary_of_parts([summary_parts(requests, makespan)])


class DeviceBackend(Backend):
    """The loop on one GPU: MIXED MPM scenes in one hg_batch, and their DEM
    piles in one DEM object of ``dem_capacity`` bodies (a fixed pool outside
    the HBM budget; a request waits while its pile does not fit)."""

    def __init__(self, ctx, max_members=256, depth=3, dem_capacity=1 << 21, dem_precision=None):
        from . import Batch  # noqa: WPS433 (package import cycle)
        self.ctx = ctx
        self.batch = Batch(ctx, max_members)
        self.depth = depth
        self.state = {}
        self.pool = collections.defaultdict(list)  # page-locked buffers by size class
        self.owner = {}
        # DEM piles
        self.dem = None
        self.dem_capacity = int(dem_capacity)
        self.dem_precision = dem_precision
        self.dem_dt = None
        self.free_lanes = list(range(max_members - 1, -1, -1))  # pop() gives the lowest
        self.order = []        # requests with disks in the DEM object, in body order
        self.adds = []         # piles opened since the last step
        self.drops = set()     # rids of piles that leave at the next step
        self.disks = 0         # disks in the DEM object and opened since
        self.staging = []      # (fence, page-locked buffer) of edits in flight
        self.chunk = 0
        self.dem_frames = {}   # chunk -> [buffer, {rid: (start, count, x0)}, readers]

    def _buf(self, shape):
        """A page-locked view of the given shape, from a pool of buffers whose
        row counts are powers of two (scenes of similar size share them)."""
        from . import pinned
        rows = shape[0]
        cls = 1 << max(rows - 1, 1).bit_length()
        key = (cls,) + tuple(shape[1:])
        free = self.pool[key]
        base = free.pop() if free else pinned(key)
        view = base[:rows]
        self.owner[id(view)] = (key, base)
        return view

    def _give(self, view):
        key, base = self.owner.pop(id(view))
        self.pool[key].append(base)

    def footprint(self, req):
        from . import mpm_estimate_bytes
        if req.ndisks > self.dem_capacity:
            raise ValueError(f"request {req.rid} has {req.ndisks} disks, over the DEM "
                             f"capacity of {self.dem_capacity}")
        c = req.cfg
        return mpm_estimate_bytes(c["grid_min"], c["grid_max"], c["h"], req.npoints)

    def can_open(self, req):
        return self.disks + req.ndisks <= self.dem_capacity

    def open(self, req):
        from . import MPM
        c = req.cfg
        m = MPM(self.ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], scenes.GRAVITY,
                c["planes"], capacity=req.npoints)
        # points generated on the device from the request's geometry
        m.seed_rectangle_device(c["rect_min"], c["rect_max"], c["rho"], c["samples_per_dim"])
        frames = [self._buf((req.npoints, 2)) for _ in range(self.depth + 1)]
        self.batch.add(m, req.dt)
        st = dict(m=m, frames=frames, dem_chunk=[None] * (self.depth + 1))
        if req.ndisks > 0:
            if self.dem_dt is None:
                self.dem_dt = req.dt
            elif req.dt != self.dem_dt:
                raise ValueError("the DEM piles of one backend share a time step")
            st["lane"] = self.free_lanes.pop()
            self.adds.append((req, dem_pile(req, st["lane"])))
            self.disks += req.ndisks
        self.state[req.rid] = st

    def _edit_piles(self):
        """One DEM edit: drop the piles that left, append the opened ones."""
        if self.dem is None:
            self.dem = dem_for_piles(self.ctx, self.dem_capacity, self.dem_precision)
            # the piles step on a stream of their own, beside the MPM batch
            self.dem.set_concurrent(True)
        n_old = sum(r.ndisks for r in self.order)
        old_to_new = np.full(n_old, -1, dtype=np.int32)
        keep, o, k = [], 0, 0
        for r in self.order:
            if r.rid not in self.drops:
                old_to_new[o:o + r.ndisks] = np.arange(k, k + r.ndisks, dtype=np.int32)
                k += r.ndisks
                keep.append(r)
            o += r.ndisks
        n_add = sum(r.ndisks for r, _ in self.adds)
        arrays = {}
        if n_add:
            # one page-locked staging buffer: q, v (3 per disk), radius, mass, inertia
            buf = self._buf((9 * n_add,))
            names = (("q", 3), ("v", 3), ("r", 1), ("m", 1), ("I", 1))
            o = 0
            for name, w in names:
                a = buf[o:o + w * n_add]
                arrays[name] = a.reshape(n_add, w) if w > 1 else a
                o += w * n_add
            o = 0
            for r, pile in self.adds:
                for name, _ in names:
                    arrays[name][o:o + r.ndisks] = pile[name]
                o += r.ndisks
        self.dem.edit_async(old_to_new, **arrays)
        if n_add:
            self.staging.append((self.fence(), buf))
        self.order = keep + [r for r, _ in self.adds]
        self.adds, self.drops = [], set()

    def step(self, nsteps):
        while self.staging and self.ctx.fence_done(self.staging[0][0]):
            self._give(self.staging.pop(0)[1])
        if self.adds or self.drops:
            self._edit_piles()
        self.batch.step(nsteps)  # on the context's stream
        if self.dem is not None and self.dem.n > 0:
            self.dem.flow(self.dem_dt, nsteps)  # on the DEM's stream, concurrently
        self.chunk += 1

    def frame(self, req, slot):
        s = self.state[req.rid]
        s["m"].frame_async(s["frames"][slot], None)
        if req.ndisks > 0:
            fr = self.dem_frames.get(self.chunk)
            if fr is None:  # the chunk's first frame copies all bodies
                buf = self._buf((self.dem.n, 3))
                self.dem.frame_async(buf)
                ranges, o = {}, 0
                for r in self.order:
                    ranges[r.rid] = (o, r.ndisks, self.state[r.rid]["lane"] * LANE)
                    o += r.ndisks
                fr = self.dem_frames[self.chunk] = [buf, ranges, 0]
            fr[2] += 1
            s["dem_chunk"][slot] = self.chunk

    def leave(self, req):
        self.batch.remove(self.state[req.rid]["m"])
        if req.ndisks > 0:
            self.drops.add(req.rid)

    def fence(self):
        if self.dem is not None:
            self.dem.join()  # the fence covers the DEM's steps, edits and frames
        return self.ctx.fence()

    def fence_done(self, f):
        return self.ctx.fence_done(f)

    def fence_wait(self, f):
        self.ctx.fence_wait(f)

    def read_frame(self, req, slot):
        s = self.state[req.rid]
        q = s["frames"][slot]
        pile = None
        if req.ndisks > 0:
            c = s["dem_chunk"][slot]
            fr = self.dem_frames[c]
            o, n, x0 = fr[1][req.rid]
            pile = float(fr[0][o:o + n, 0].max() - x0)
            fr[2] -= 1
            if fr[2] == 0:
                self._give(fr[0])
                del self.dem_frames[c]
        return float(q[:, 0].max()), pile  # run-outs: front positions

    def close(self, req):
        s = self.state.pop(req.rid)
        s["m"].close()
        for a in s["frames"]:
            self._give(a)
        if req.ndisks > 0:
            self.free_lanes.append(s["lane"])
            self.free_lanes.sort(reverse=True)
            self.disks -= req.ndisks

    def shutdown(self):
        self.batch.close()
        if self.dem is not None:
            self.dem.close()


def run_one_at_a_time(ctx, requests, dem_precision=None):
    """The same requests served one after another, each scene alone
    (hg_mpm_step and, with disks, hg_dem_step of its own DEM object per frame
    interval, frames read synchronously); returns wall seconds."""
    from . import MPM
    t0 = time.perf_counter()
    for r in requests:
        c = r.cfg
        m = MPM(ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], scenes.GRAVITY,
                c["planes"], capacity=r.npoints)
        m.seed_rectangle_device(c["rect_min"], c["rect_max"], c["rho"], c["samples_per_dim"])
        d = None
        if r.ndisks > 0:
            p = dem_pile(r, 0)
            d = dem_for_piles(ctx, r.ndisks, dem_precision)
            d.upload(p["q"], p["v"], p["r"], p["m"], p["I"], p["fixed"])
        q = np.zeros((r.npoints, 2))
        for k in range(r.steps // r.frame_every):
            m.flow(r.dt, r.frame_every)
            if d is not None:
                d.flow(r.dt, r.frame_every)
            m.download_into(q=q)
            pile = None if d is None else float(d.download()[0][:, 0].max())
            r.frames.append(((k + 1) * r.frame_every, (float(q[:, 0].max()), pile)))
        m.close()
        if d is not None:
            d.close()
    return time.perf_counter() - t0
