"""Continuous-batching service for excitation-sweep requests.

Each request is a sphere scene (SPHERE particles in a box of OBSTACLE
triangles), a number of steps and a base excitation evaluated on the device.
The server keeps one pooled session resident in HBM: its arrays hold every
admitted scene in its own ranges, with its own grid, triangles, local time and
excitation.  Requests are admitted, in arrival order, as soon as a scene slot
and room in the pool (sized from an HBM budget) are free; all admitted scenes
advance together, one launch per kernel per step, so their work overlaps on
the device.  When a request's steps are done its state is read back, its
ranges are freed and a waiting request can take them.  While a chunk of
steps runs (pg_session_run_async), the host copies requests that have
arrived into free ranges of the pool's host arrays; they are uploaded and
switched on after the chunk.

A scene's arithmetic does not depend on the other scenes in the pool, so a
request's result is bitwise the same alone and in the mix
(tests/test_gpu_serving.py).  Each request runs `steps` steps from its initial
state (no initial half step: the half step of the reference's first DEM call
is a property of a standalone run).
"""
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi, batch
from .engine import GpuEngine
from .model import Model


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the stream starts
    model: Model              # a sphere scene (particles == spheres)
    steps: int
    excitation: np.ndarray    # batch.excitation record
    dt: float


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    spheres: int
    position: np.ndarray = field(repr=False)
    linear: np.ndarray = field(repr=False)
    error: str = None
    energy: float = None      # kinetic + rotational + potential of the base gravity g0, at the end

    @property
    def wait(self):
        return self.admitted - self.arrival

    @property
    def latency(self):
        return self.finished - self.arrival


class _Ranges:
    """First-fit allocator over [0, n)."""

    def __init__(self, n):
        self.free = [(0, n)]

    def take(self, size):
        if size == 0:
            return 0
        for k, (b, e) in enumerate(self.free):
            if e - b >= size:
                if e - b == size:
                    del self.free[k]
                else:
                    self.free[k] = (b + size, e)
                return b
        return None

    def give(self, b, size):
        if size == 0:
            return
        self.free.append((b, b + size))
        self.free.sort()
        merged = []
        for r in self.free:
            if merged and merged[-1][1] == r[0]:
                merged[-1] = (merged[-1][0], r[1])
            else:
                merged.append(r)
        self.free = merged


def bytes_per_sphere(form, kn=32, kr=32):
    """Device bytes one pooled sphere particle needs: state, candidate lists
    (kn slots) and the slave-list entry buffers (two key and two value words
    per slot); kr is accepted for older callers and unused."""
    state = 8 * (6 + 3 + 9 + 6 + 9 + 9 + 2 + 3 + 3) + 8 * (6 + 3) + 4 * 12 + 8 * 6 + 8 * 3 + 4 * 4
    if form == abi.PG_FORM_MIXED:
        state += 4 * (6 + 6 + 18 + 6 + 2 + 2 + 18 + 6 + 6 + 6 + 2 + 3)
        slots = kn * (4 + 1 + 12 + 12 + 12)
    else:
        slots = kn * (4 + 1 + 24 + 24 + 24 + 24 + 8 + 8 + 4)
    return state + slots + kn * 16 + 16


class Server:
    """One pooled session; serves requests with continuous batching."""

    def __init__(self, template, dt, form=abi.PG_FORM_MIXED, budget_bytes=150e9, max_scenes=256,
                 max_spheres=None, max_triangles=None, max_scene_extent=4.0, kn=32, kr=32, chunk=250,
                 fused=False):
        """fused: the mixed form steps the pool with the fused step kernel, its
        launch shape picked by the autotuner on the first steps; by default
        the per-phase kernels (one CUDA graph per step), which measured
        faster on the batch workload."""
        self.form = form
        self.dt = dt
        self.chunk = chunk
        self.bps = bytes_per_sphere(form, kn, kr)
        self.budget = float(budget_bytes)
        cap = int(budget_bytes // self.bps)
        if max_spheres is not None:
            cap = min(cap, int(max_spheres))
        self.cap = cap
        self.last_energy = None
        self.tcap = int(max_triangles if max_triangles is not None else 12 * max_scenes)
        self.max_scenes = max_scenes
        self.P = self._empty_pool(template, cap, self.tcap, max_scenes)
        use_fused = fused and form == abi.PG_FORM_MIXED
        self.eng = GpuEngine(form=form, capacity=(kn, kr), fused=use_fused, autotune=use_fused)
        self.eng.attach(self.P)
        self.P.engine = self.eng
        rmax = float(template.E.radii[0, :template.ellnum].max())
        rmin = float(template.E.radii[0, :template.ellnum].min())
        skin = 0.6 * rmin          # pool default: scenes share one rebuild flag
        self.cell = 2.0 * rmax + skin
        n = min(512, int(np.ceil(max_scene_extent / self.cell)) + 9)
        abi.check(self.eng.lib.pg_session_set_skin(self.eng.sess, skin), "pg_session_set_skin")
        self.eng.set_grid(self.cell, (n, n, n))
        self.spheres = _Ranges(cap)
        self.tris = _Ranges(self.tcap)
        self.slots = list(range(max_scenes))
        self.active = {}         # scene slot -> (request, ranges, remaining, admitted)
        self._zero_tab = None
        self._live = None
        self._update_live()

    @staticmethod
    def _empty_pool(template, cap, tcap, nscene):
        P = Model()
        P.mparam = [list(x) for x in template.mparam]
        P.pairs, P.ikind, P.iparam = list(template.pairs), list(template.ikind), [list(x) for x in template.iparam]
        P.compat = template.compat
        P.P.ensure(cap)
        P.E.ensure(cap)
        P.Tr.ensure(tcap)
        P.parnum = P.ellnum = cap
        P.trinum = tcap
        P.P.mass[:cap] = 1.0
        P.P.invm[:cap] = 1.0
        P.P.rotation[0, :cap] = P.P.rotation[4, :cap] = P.P.rotation[8, :cap] = 1.0
        P.E.part[:cap] = np.arange(cap, dtype=np.int32)
        P.E.radii[0, :cap] = 1e-6
        P.E.radii[1:3, :cap] = -1.0
        P.E.ellcol[:cap] = 1
        P.Tr.triobs[:tcap] = -1
        P.Tr.tricol[:tcap] = 2
        P.nscene = nscene
        P.pscene = np.full(P.P.cap, -1, dtype=np.int32)
        P.tscene = np.full(P.Tr.cap, -1, dtype=np.int32)
        P.oscene = np.full(max(1, P.O.cap), -1, dtype=np.int32)
        P.sactive = np.zeros(nscene, dtype=np.int32)
        return P

    # ---------------------------------------------------------------- load
    def _stage(self, req):
        """Take pool ranges for a request and copy its scene into the pool's
        host arrays: no device work, so this runs while a chunk of steps is
        in flight.  Returns the ranges, or None when the pool has no room."""
        m = req.model
        n, nt = m.parnum, m.trinum
        if m.ellnum != n or m.obsnum or m.sprnum or m.prescribe:
            raise ValueError("a request must be a sphere scene with static obstacles")
        e0 = self.spheres.take(n)
        if e0 is None:
            return None
        t0 = self.tris.take(nt)
        if t0 is None:
            self.spheres.give(e0, n)
            return None
        P = self.P
        for name in P.P.spec:
            getattr(P.P, name)[..., e0:e0 + n] = getattr(m.P, name)[..., :n]
        for name in P.E.spec:
            getattr(P.E, name)[..., e0:e0 + n] = getattr(m.E, name)[..., :n]
        P.E.part[e0:e0 + n] = np.arange(e0, e0 + n, dtype=np.int32)
        for name in P.Tr.spec:
            getattr(P.Tr, name)[..., t0:t0 + nt] = getattr(m.Tr, name)[..., :nt]
        return (e0, e0 + n, e0, e0 + n, t0, t0 + nt, 0, 0)

    def _commit(self, req, slot, r):
        """Upload a staged request's ranges and switch its scene on (no step
        is in flight)."""
        m = req.model
        e0, e1, _, _, t0, t1, _, _ = r
        self.P.pscene[e0:e1] = slot
        self.P.tscene[t0:t1] = slot
        self.eng.upload_range(r, refresh=False)      # the pool's arrays never move
        lo = m.E.center[0:3, :m.parnum].min(axis=1)
        self.eng.set_scene(slot, True, origin=lo - 4.0 * self.cell, excitation=req.excitation, start=-1)

    def _load(self, req, slot):
        r = self._stage(req)
        if r is not None:
            self._commit(req, slot, r)
        return r

    def _unload(self, slot):
        req, r, _, _ = self.active.pop(slot)
        e0, e1, _, _, t0, t1, _, _ = r
        self.eng.download_range_motion(r)          # mass and inertia are the request's own
        P = self.P
        pos = P.P.position[0:3, e0:e1].copy()
        lin = P.P.linear[:, e0:e1].copy()
        self.last_energy = range_energy(P, e0, e1, req.excitation[0:3])
        self.eng.set_scene(slot, False)
        P.pscene[e0:e1] = -1
        P.tscene[t0:t1] = -1
        self.eng.release_range(r)
        self.spheres.give(e0, e1 - e0)
        self.tris.give(t0, t1 - t0)
        self.slots.append(slot)
        return pos, lin

    LIVE_QUANTUM = 4096

    def _update_live(self):
        """Steps cover the pool up to the end of its last allocated range
        (rounded up), not its whole capacity (pg_session_set_live)."""
        def top(r, cap):
            end = r.free[-1][0] if r.free and r.free[-1][1] == cap else cap
            q = self.LIVE_QUANTUM
            return min(cap, ((end + q - 1) // q) * q)
        e, t = top(self.spheres, self.cap), top(self.tris, self.tcap)
        if (e, t) != self._live:
            self.eng.set_live(e, e, t)
            self._live = (e, t)

    # ---------------------------------------------------------------- loop
    def _tab(self, n):
        from .driver import StepTables
        if self._zero_tab is None or self._zero_tab[0] < n:
            t = StepTables.__new__(StepTables)
            t.curtime = np.zeros(n)
            t.gravity = np.zeros((n, 3))
            t.damping = np.zeros((n, 6))
            t.prs_lin = np.zeros((n, 1, 3))
            t.prs_ang = np.zeros((n, 1, 3))
            t.obs_ang = np.zeros((n, 1, 3))
            t.obs_lin = np.zeros((n, 1, 3))
            t.stepnum = 0
            self._zero_tab = (n, t)
        return self._zero_tab[1].ctab(0, n)

    def check(self, req):
        """Why a request cannot be served by this pool (None when it can)."""
        m = req.model
        if m.ellnum != m.parnum or m.obsnum or m.sprnum or m.prescribe:
            return "not a sphere scene with static obstacles"
        if m.parnum > self.cap or m.trinum > self.tcap:
            return "larger than the pool"
        if abs(req.dt - self.dt) > 1e-12 * self.dt:
            return "time step differs from the pool's"
        if req.steps <= 0:
            return "no steps"
        return None

    def serve(self, requests, realtime=True):
        """Serve `requests` (sorted by arrival).  Returns (results, stats);
        rejected requests come back with `error` set."""
        pending = []
        results = []
        for q in sorted(requests, key=lambda q: q.arrival):
            why = self.check(q)
            if why is None:
                pending.append(q)
            else:
                results.append(Result(q.rid, q.arrival, q.arrival, q.arrival, q.steps, q.model.parnum,
                                      np.zeros((3, 0)), np.zeros((3, 0)), error=why))
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        steps_done = 0
        psteps = 0
        peak_spheres = peak_scenes = 0
        staged = []                # (request, ranges): in the pool's host arrays, not yet on the device
        while pending or self.active or staged:
            # no step is in flight here: commit what was staged during the last chunk
            for req, r in staged:
                slot = self.slots.pop(0)
                self._commit(req, slot, r)
                self.active[slot] = (req, r, req.steps, now())
            staged = []
            # admit in arrival order while there is room
            while pending and (not realtime or pending[0].arrival <= now()) and self.slots:
                req = pending[0]
                slot = self.slots.pop(0)
                r = self._load(req, slot)
                if r is None:
                    self.slots.insert(0, slot)
                    break
                pending.pop(0)
                self.active[slot] = (req, r, req.steps, now())
            self._update_live()
            if not self.active:
                if pending and realtime:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now())))
                continue
            c = min(self.chunk, min(v[2] for v in self.active.values()))
            self.eng.run_async(self._tab(c), self.dt)
            # while the chunk runs, copy arrived requests into free ranges of
            # the host arrays, as many as there will be free slots after it
            # (the free ones and those of the scenes it finishes); they go to
            # the device after the wait
            room = len(self.slots) + sum(1 for v in self.active.values() if v[2] == c)
            while pending and (not realtime or pending[0].arrival <= now()) and len(staged) < room:
                r = self._stage(pending[0])
                if r is None:
                    break
                staged.append((pending.pop(0), r))
            self.eng.sync()
            steps_done += c
            for slot in list(self.active):
                req, r, rem, adm = self.active[slot]
                psteps += (r[1] - r[0]) * c
                rem -= c
                self.active[slot] = (req, r, rem, adm)
                if rem == 0:
                    pos, lin = self._unload(slot)
                    results.append(Result(req.rid, req.arrival, adm, now(), req.steps, r[1] - r[0], pos, lin,
                                          energy=self.last_energy))
            in_use = self.cap - sum(e - b for b, e in self.spheres.free)
            peak_spheres = max(peak_spheres, in_use)
            peak_scenes = max(peak_scenes, len(self.active) + len(staged))
        wall = now()
        ok = [x for x in results if x.error is None]
        lat = np.array([x.latency for x in ok])
        wait = np.array([x.wait for x in ok])
        edges = [0.0, 0.01, 0.1, 1.0, 10.0, float("inf")]
        hist = np.histogram(wait, bins=edges)[0].tolist() if len(wait) else [0] * (len(edges) - 1)
        stats = {"requests": len(lat), "rejected": sum(1 for x in results if x.error), "wall_s": wall,
                 "particle_steps": psteps,
                 "throughput": psteps / wall if wall > 0 else 0.0,
                 "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
                 "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
                 "admission_wait_s": {"p50": float(np.percentile(wait, 50)) if len(wait) else None,
                                      "p99": float(np.percentile(wait, 99)) if len(wait) else None,
                                      "histogram_edges_s": edges[:-1] + ["inf"], "histogram": hist},
                 "pool": {"sphere_capacity": self.cap, "peak_spheres": peak_spheres,
                          "scene_slots": self.max_scenes, "peak_scenes": peak_scenes,
                          "budget_bytes": self.budget, "bytes_per_sphere": self.bps},
                 "steps_launched": steps_done}
        return results, stats

    def close(self):
        self.eng.close()


def range_energy(P, e0, e1, g0):
    """Kinetic, rotational and gravity-potential energy (base gravity g0) of
    pool particles [e0, e1)."""
    mass = P.P.mass[e0:e1]
    v = P.P.linear[:, e0:e1]
    O = P.P.angular[0:3, e0:e1]
    J = P.P.inertia[:, e0:e1]
    JO = np.stack([J[0] * O[0] + J[3] * O[1] + J[6] * O[2],
                   J[1] * O[0] + J[4] * O[1] + J[7] * O[2],
                   J[2] * O[0] + J[5] * O[1] + J[8] * O[2]])
    g = np.asarray(g0, dtype=np.float64).reshape(3, 1)
    return (0.5 * float(np.sum(mass * np.sum(v * v, axis=0))) + 0.5 * float(np.sum(O * JO))
            - float(np.sum(mass * np.sum(g * P.P.position[0:3, e0:e1], axis=0))))


def excitation_gravity(exc):
    """The base excitation record as a host GRAVITY callable g(t) =
    g0 + dir * sum_k amp_k sin(2 pi freq_k t + phase_k): the same excitation
    for a request run through DEM() one at a time."""
    import math
    g0 = [float(x) for x in exc[0:3]]
    d = [float(x) for x in exc[3:6]]
    comps = [(float(exc[8 + 3 * k]), float(exc[9 + 3 * k]), float(exc[10 + 3 * k])) for k in range(int(exc[6]))]

    def g(t):
        a = 0.0
        for amp, f, ph in comps:
            a += amp * math.sin(2.0 * math.pi * f * t + ph)
        return (g0[0] + d[0] * a, g0[1] + d[1] * a, g0[2] + d[2] * a)
    return g


def request_stream(count, rate=200.0, seed=4, nmin=1024, nmax=262144, smin=200, smax=5000):
    """Config 4: Poisson arrivals at `rate` req/s; sphere counts log-uniform in
    [nmin, nmax]; steps uniform in [smin, smax]; half the requests a random
    sinusoid, half seeded band-limited noise."""
    import math
    from .scenes import hopper_fill
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    out = []
    for k in range(count):
        n = int(np.exp(rng.uniform(math.log(nmin), math.log(nmax))))
        side = max(2, int(round(n ** (1.0 / 3.0))))
        m, dt = hopper_fill(n_side=side, seed=seed * 1000003 + k, box=max(1.0, side / 16.0))
        steps = int(rng.integers(smin, smax + 1))
        if rng.random() < 0.5:
            exc = batch.sinusoid((0.0, 0.0, -9.81), (rng.uniform(0.1, 1.0) * 9.81, 0.0, 0.0),
                                 rng.uniform(1.0, 20.0))
        else:
            exc = batch.band_noise((0.0, 0.0, -9.81), (1.0, 0.0, 0.0), rng.uniform(0.1, 1.0) * 9.81,
                                   1.0, 20.0, seed=int(rng.integers(1 << 30)))
        out.append(Request(k, float(t[k]), m, steps, exc, dt))
    return out
