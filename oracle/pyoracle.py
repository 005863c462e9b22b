"""ctypes wrapper of the oracle (TEST INFRASTRUCTURE ONLY).

Exposes the oracle's restated dem() loop body as an engine with the same
interface as parmec_gb300.engine.GpuEngine, so that a Model can be stepped by
either.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

from parmec_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build():
    """Compile the oracle (g++, -ffp-contract=off so no multiply-add is fused, OpenMP);
    the same command as oracle/Makefile."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    subprocess.run(["g++", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-std=c++17",
                    "-Wall", "-shared", "-o", LIB, os.path.join(HERE, "oracle.cpp")], check=True)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "oracle.cpp")):
        build()
    lib = ctypes.CDLL(LIB)
    P = ctypes.c_void_p
    S = ctypes.POINTER(abi.PgScene)
    D = abi.D
    sig = {
        "or_create": (P, [S]),
        "or_destroy": (None, [P]),
        "or_set_threads": (None, [P, ctypes.c_int]),
        "or_invert_inertia": (None, [P, S]),
        "or_first_half_step": (None, [P, S, ctypes.c_double, D, D]),
        "or_condet_forces": (None, [P, S, ctypes.c_double, ctypes.c_double, D, D, D]),
        "or_run": (ctypes.c_int, [P, S, ctypes.POINTER(abi.PgStepTab), ctypes.c_double]),
        "or_run_adaptive": (ctypes.c_int, [P, S, ctypes.POINTER(abi.PgStepTab), ctypes.c_double, ctypes.c_double, D]),
        "or_critical_terms": (ctypes.c_int, [P, S, D, D, D]),
        "or_mesh_contact": (None, [P, S, ctypes.c_double, ctypes.c_void_p]),
        "or_mesh_contact_stats": (None, [P, abi.I, abi.I]),
        "or_tt_contact": (ctypes.c_double, [D, D, ctypes.c_double, ctypes.c_double, D, D]),
        "or_restrain_velocities": (None, [P, S]),
        "or_restrain_forces": (None, [P, S]),
        "or_dynamics": (None, [P, S, D, ctypes.c_double, ctypes.c_double]),
        "or_shapes": (None, [P, S]),
        "or_obstacles": (None, [P, S, ctypes.c_double]),
        "or_expmap": (None, [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, D]),
        "or_triangle_sphere": (ctypes.c_double, [D, D, D, D, ctypes.c_double, D, D, ctypes.c_int]),
        "or_eqm": (ctypes.c_double, [S, ctypes.c_int, D, ctypes.c_int, D, D]),
        "or_contact_count": (ctypes.c_int, [P]),
        "or_contacts": (ctypes.c_int, [P, ctypes.c_int, abi.I, abi.I, D, D, D, D, D]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class OracleEngine:
    """Steps a Model with the oracle, in place on the model's host arrays."""

    def __init__(self, threads=1):
        self.lib = load()
        self.threads = threads
        self.model = None
        self.ctx = None
        self.counts = None

    def attach(self, m):
        from parmec_gb300.engine import _counts
        self.close()
        self.model = m
        self.scene = m.scene()
        self.counts = _counts(m)
        self.ctx = self.lib.or_create(ctypes.byref(self.scene))
        self.lib.or_set_threads(self.ctx, self.threads)
        if getattr(m, "tt_radius", 0.0) > 0.0:
            from parmec_gb300.mesh import mesh_contact_grid
            _, big = mesh_contact_grid(m)
            self._tt_big = big
            self.lib.or_mesh_contact(self.ctx, ctypes.byref(self.scene), m.tt_radius, big.ctypes.data)

    def stale(self):
        from parmec_gb300.engine import _counts
        return self.model is None or _counts(self.model) != self.counts

    def upload(self):
        self.scene = self.model.scene()

    def first_half_step(self, step, ang, lin):
        ang = np.ascontiguousarray(ang, dtype=np.float64)
        lin = np.ascontiguousarray(lin, dtype=np.float64)
        self.lib.or_first_half_step(self.ctx, ctypes.byref(self.scene), step, abi.dptr(ang), abi.dptr(lin))

    def invert_inertia(self):
        self.lib.or_invert_inertia(self.ctx, ctypes.byref(self.scene))

    def run(self, tab, step):
        self.lib.or_run(self.ctx, ctypes.byref(self.scene), ctypes.byref(tab), step)

    def restrain_velocities(self):
        self.lib.or_restrain_velocities(self.ctx, ctypes.byref(self.scene))

    def run_adaptive(self, tab, step0, adaptive):
        """tab.nsteps adaptive steps from step0; returns each step's step1."""
        steps = np.zeros(max(1, tab.nsteps))
        self.lib.or_run_adaptive(self.ctx, ctypes.byref(self.scene), ctypes.byref(tab), step0, adaptive,
                                 abi.dptr(steps))
        return steps[:tab.nsteps]

    def critical_terms(self):
        """Per-particle (step, omega, ratio) from the latest adaptive step's terms."""
        n = self.model.parnum
        h, o, r = np.zeros(max(1, n)), np.zeros(max(1, n)), np.zeros(max(1, n))
        if self.lib.or_critical_terms(self.ctx, ctypes.byref(self.scene), abi.dptr(h), abi.dptr(o), abi.dptr(r)):
            raise RuntimeError("no adaptive step has run")
        return h[:n], o[:n], r[:n]

    def mesh_contact_stats(self):
        """(pairs, active pairs) of the last step's mesh-mesh contact stage."""
        a, b = ctypes.c_int(), ctypes.c_int()
        self.lib.or_mesh_contact_stats(self.ctx, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def critical(self, which):
        """CRITICAL restated on the host (oracle/critical_host.py) over this
        engine's contacts: which = 0 per particle, 1 per spring."""
        from oracle import critical_host
        if which == 1:
            return tuple(np.array(a) for a in critical_host.critical_perspring(self.model))
        return critical_host.critical_perparticle(self.model, self.contacts())

    def sync(self):
        pass

    def download(self):
        self.model.pull_obstacles()
        self.model.pull_body_forces()

    def contacts(self):
        n = self.lib.or_contact_count(self.ctx)
        cap = max(1, n)
        out = {"mpart": np.zeros(cap, np.int32), "code": np.zeros(cap, np.int32),
               "point": np.zeros((cap, 3)), "normal": np.zeros((cap, 3)), "depth": np.zeros(cap),
               "force": np.zeros((cap, 3)), "state": np.zeros((cap, 3))}
        cnt = self.lib.or_contacts(self.ctx, cap, abi.iptr(out["mpart"]), abi.iptr(out["code"]),
                                   abi.dptr(out["point"]), abi.dptr(out["normal"]), abi.dptr(out["depth"]),
                                   abi.dptr(out["force"]), abi.dptr(out["state"]))
        return {k: v[:cnt] for k, v in out.items()}

    def close(self):
        if self.ctx is not None:
            self.lib.or_destroy(self.ctx)
            self.ctx = None
        self.model = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
