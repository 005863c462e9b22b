"""Compute engine over the device-resident session API of libparmec_gb300.so."""
import ctypes

import numpy as np

from . import abi


def _counts(m):
    return (m.parnum, m.ellnum, m.trinum, m.obsnum, m.nodnum, m.facnum, m.sprnum,
            len(m.prescribe), len(m.pairs), len(m.lcurves), len(m.restraints), len(m.unsprings), m.trqsprnum,
            len(m.body_forces), getattr(m, "tt_radius", 0.0), m.ellcon, m.tricon, m.faccon)


class GpuEngine:
    """Runs DEM steps of one Model in a pg_session on the current CUDA device."""

    def __init__(self, model=None, form=abi.PG_FORM_FP64, skin=None, record_geometry=False, graph=True,
                 capacity=None, fused=False, autotune=False):
        """fused: the mixed form's fused step kernel (pg_session_use_fused);
        autotune: pick its launch shape by timing the first steps."""
        self.lib = abi.load_library()
        self._pinned = {}
        self.fused = fused
        self.autotune = autotune
        self.graph = graph
        self.capacity = capacity
        self.form = form
        self.skin = skin
        self.record_geometry = record_geometry
        self.model = None
        self.sess = None
        self.scene = None
        self.counts = None

    # host arrays of at least this many bytes are page-locked while attached
    PIN_BYTES = 1 << 20

    def _pin(self, m):
        """Page-lock the model's large SoA arrays, so that upload/download copy
        at link speed instead of staging through pageable memory."""
        import numpy as np
        want = {}
        for soa in (m.P, m.E, m.Tr, m.N, m.F, m.S):
            for name in soa.spec:
                a = getattr(soa, name)
                if isinstance(a, np.ndarray) and a.nbytes >= self.PIN_BYTES:
                    want[a.ctypes.data] = (a, a.nbytes)
        for ptr in list(self._pinned):
            if ptr not in want:
                self.lib.pg_host_unregister(ctypes.c_void_p(ptr))
                del self._pinned[ptr]
        for ptr, (a, nb) in want.items():
            if ptr not in self._pinned and self.lib.pg_host_register(ctypes.c_void_p(ptr), nb) == 0:
                self._pinned[ptr] = a                 # keep the array alive while pinned

    def attach(self, m):
        self.close()
        self.model = m
        self._pin(m)
        self.scene = m.scene()
        self.counts = _counts(m)
        h = ctypes.c_void_p()
        abi.check(self.lib.pg_session_create(ctypes.byref(self.scene), self.form, ctypes.byref(h)),
                  "pg_session_create")
        self.sess = h
        if self.skin is not None:
            abi.check(self.lib.pg_session_set_skin(self.sess, float(self.skin)), "pg_session_set_skin")
        if self.record_geometry:
            abi.check(self.lib.pg_session_record_geometry(self.sess, 1), "pg_session_record_geometry")
        if not self.graph:
            abi.check(self.lib.pg_session_use_graph(self.sess, 0), "pg_session_use_graph")
        if self.capacity is not None:
            abi.check(self.lib.pg_session_set_capacity(self.sess, int(self.capacity[0]), int(self.capacity[1])),
                      "pg_session_set_capacity")
        if getattr(m, "tt_radius", 0.0) > 0.0:
            from .mesh import mesh_contact_grid
            cell, big = mesh_contact_grid(m)
            abi.check(self.lib.pg_session_mesh_contact(self.sess, m.tt_radius, cell, big.ctypes.data),
                      "pg_session_mesh_contact")
        if self.fused:
            abi.check(self.lib.pg_session_use_fused(self.sess, 1), "pg_session_use_fused")
            if self.autotune:
                abi.check(self.lib.pg_session_autotune(self.sess, 1), "pg_session_autotune")

    def stale(self):
        return self.model is None or _counts(self.model) != self.counts

    def upload(self):
        self._pin(self.model)
        self.scene = self.model.scene()
        abi.check(self.lib.pg_session_upload(self.sess, ctypes.byref(self.scene)), "pg_session_upload")

    def first_half_step(self, step, ang, lin):
        ang = np.ascontiguousarray(ang, dtype=np.float64)
        lin = np.ascontiguousarray(lin, dtype=np.float64)
        abi.check(self.lib.pg_session_first_half_step(self.sess, step, abi.dptr(ang), abi.dptr(lin)),
                  "pg_session_first_half_step")

    def invert_inertia(self):
        abi.check(self.lib.pg_session_invert_inertia(self.sess), "pg_session_invert_inertia")

    def restrain_velocities(self):
        abi.check(self.lib.pg_session_restrain_velocities(self.sess), "pg_session_restrain_velocities")

    def run(self, tab, step):
        abi.check(self.lib.pg_session_run(self.sess, ctypes.byref(tab), step), "pg_session_run")

    def run_async(self, tab, step):
        """Enqueue the steps and return (pg_session_run_async); sync() waits for them."""
        abi.check(self.lib.pg_session_run_async(self.sess, ctypes.byref(tab), step), "pg_session_run_async")

    def run_adaptive(self, tab, step0, adaptive):
        """tab.nsteps adaptive steps from step0 (pg_session_run_adaptive); returns each step's step1."""
        steps = np.zeros(max(1, tab.nsteps))
        abi.check(self.lib.pg_session_run_adaptive(self.sess, ctypes.byref(tab), step0, adaptive, abi.dptr(steps)),
                  "pg_session_run_adaptive")
        return steps[:tab.nsteps]

    def set_live(self, particles, spheres, triangles):
        """A pool's live extents (pg_session_set_live)."""
        abi.check(self.lib.pg_session_set_live(self.sess, int(particles), int(spheres), int(triangles)),
                  "pg_session_set_live")

    def mesh_contact_stats(self):
        """(pairs, active pairs) of the last step's mesh-mesh contact stage."""
        a, b = ctypes.c_int(), ctypes.c_int()
        abi.check(self.lib.pg_session_mesh_contact_stats(self.sess, ctypes.byref(a), ctypes.byref(b)),
                  "pg_session_mesh_contact_stats")
        return a.value, b.value

    def critical(self, which):
        """CRITICAL on the device (pg_session_critical): which = 0 per particle
        (parnum entries), 1 per spring (sprnum entries, sorted spring order);
        returns (step, omega, ratio) arrays."""
        n = self.model.parnum if which == 0 else self.model.sprnum
        out = [np.zeros(max(1, n)) for _ in range(3)]
        abi.check(self.lib.pg_session_critical(self.sess, int(which), *(abi.dptr(a) for a in out)),
                  "pg_session_critical")
        return tuple(a[:n] for a in out)

    def sync(self):
        abi.check(self.lib.pg_session_sync(self.sess), "pg_session_sync")

    def download(self):
        abi.check(self.lib.pg_session_download(self.sess, ctypes.byref(self.scene)), "pg_session_download")
        self.model.pull_obstacles()
        self.model.pull_body_forces()

    def download_rows(self, particles, springs):
        """Only the given particles' and springs' state (pg_session_download_particles/_springs)."""
        if len(particles):
            idx = np.ascontiguousarray(particles, dtype=np.int32)
            abi.check(self.lib.pg_session_download_particles(self.sess, ctypes.byref(self.scene), abi.iptr(idx),
                                                             len(idx)), "pg_session_download_particles")
        if len(springs):
            idx = np.ascontiguousarray(springs, dtype=np.int32)
            abi.check(self.lib.pg_session_download_springs(self.sess, ctypes.byref(self.scene), abi.iptr(idx),
                                                           len(idx)), "pg_session_download_springs")

    def fused_config(self):
        """(threads per block, blocks, tuned, graph) of the fused step kernel."""
        out = (ctypes.c_int * 4)()
        abi.check(self.lib.pg_session_fused_config(self.sess, out), "pg_session_fused_config")
        return tuple(out)

    def kernel_launches(self):
        n = ctypes.c_longlong()
        abi.check(self.lib.pg_session_kernel_launches(self.sess, ctypes.byref(n)), "kernel_launches")
        return n.value

    # ---- scenes sharing the session
    def set_scene(self, k, active=True, origin=None, excitation=None, start=-1):
        o = None if origin is None else np.ascontiguousarray(origin, dtype=np.float64)
        e = None if excitation is None else np.ascontiguousarray(excitation, dtype=np.float64)
        abi.check(self.lib.pg_session_scene(self.sess, int(k), 1 if active else 0, abi.dptr(o), abi.dptr(e),
                                            int(start)), "pg_session_scene")

    def set_grid(self, cell, dims):
        d = np.ascontiguousarray(dims, dtype=np.int32)
        abi.check(self.lib.pg_session_set_grid(self.sess, float(cell), abi.iptr(d)), "pg_session_set_grid")

    def upload_range(self, r, refresh=True):
        """Upload pool ranges r (pg_session_upload_range); refresh=False keeps
        the scene structure of the last call, for a model whose arrays are
        the same objects (a serving pool's)."""
        if refresh or self.scene is None:
            self.scene_refresh()
        rr = np.ascontiguousarray(r, dtype=np.int32)
        abi.check(self.lib.pg_session_upload_range(self.sess, ctypes.byref(self.scene), abi.iptr(rr)),
                  "pg_session_upload_range")

    def download_range(self, r):
        rr = np.ascontiguousarray(r, dtype=np.int32)
        abi.check(self.lib.pg_session_download_range(self.sess, ctypes.byref(self.scene), abi.iptr(rr)),
                  "pg_session_download_range")
        self.model.pull_obstacles()

    def download_range_motion(self, r):
        """Positions, linear and angular velocities of pool range r alone
        (pg_session_download_range_motion)."""
        rr = np.ascontiguousarray(r, dtype=np.int32)
        abi.check(self.lib.pg_session_download_range_motion(self.sess, ctypes.byref(self.scene), abi.iptr(rr)),
                  "pg_session_download_range_motion")

    def release_range(self, r):
        """Free pool ranges on the device: scene id -1 for their entries."""
        rr = np.ascontiguousarray(r, dtype=np.int32)
        abi.check(self.lib.pg_session_release_range(self.sess, abi.iptr(rr)), "pg_session_release_range")

    def scene_refresh(self):
        """Re-point the ctypes scene at the model's arrays (after host edits)."""
        self.scene = self.model.scene()

    def global_step(self):
        n = ctypes.c_longlong()
        abi.check(self.lib.pg_session_global_step(self.sess, ctypes.byref(n)), "pg_session_global_step")
        return n.value

    def profile(self, on=True):
        abi.check(self.lib.pg_session_profile(self.sess, 1 if on else 0), "pg_session_profile")

    def profile_read(self):
        ms = (ctypes.c_double * 8)()
        n = (ctypes.c_longlong * 8)()
        abi.check(self.lib.pg_session_profile_read(self.sess, ms, n), "pg_session_profile_read")
        names = ["rebuild", "contacts", "springs", "integrate", "mesh", "obstacles"]
        return {names[g]: (ms[g], n[g]) for g in range(6)}

    def diagnostics(self):
        out = (ctypes.c_int * 16)()
        abi.check(self.lib.pg_session_diagnostics(self.sess, out), "pg_session_diagnostics")
        v = list(out)
        return {"error": v[0:4], "rebuilds": v[4], "max_candidates": v[5], "max_slave": v[6],
                "max_triangles": v[7], "grid": v[12:15], "bits": v[15]}

    def stream(self):
        p = ctypes.c_void_p()
        abi.check(self.lib.pg_session_stream(self.sess, ctypes.byref(p)), "pg_session_stream")
        return p.value

    def contacts(self):
        """Active contacts in canonical order as a dict of numpy arrays."""
        n = ctypes.c_int()
        abi.check(self.lib.pg_session_contact_count(self.sess, ctypes.byref(n)), "contact_count")
        cap = max(1, n.value)
        out = {"mpart": np.zeros(cap, np.int32), "code": np.zeros(cap, np.int32),
               "point": np.zeros((cap, 3)), "normal": np.zeros((cap, 3)), "depth": np.zeros(cap),
               "force": np.zeros((cap, 3)), "state": np.zeros((cap, 3))}
        cnt = ctypes.c_int()
        abi.check(self.lib.pg_session_contacts(
            self.sess, cap, ctypes.byref(cnt), abi.iptr(out["mpart"]), abi.iptr(out["code"]),
            abi.dptr(out["point"]), abi.dptr(out["normal"]), abi.dptr(out["depth"]),
            abi.dptr(out["force"]), abi.dptr(out["state"])), "contacts")
        return {k: v[:cnt.value] for k, v in out.items()}

    def close(self):
        if self.sess is not None:
            self.lib.pg_session_destroy(self.sess)
            self.sess = None
        for ptr in list(getattr(self, "_pinned", {})):
            self.lib.pg_host_unregister(ctypes.c_void_p(ptr))
        self._pinned = {}
        self.model = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
