"""parmec.cpp's dem() loop over a library of the reference's ISPC entry points
(TEST INFRASTRUCTURE ONLY).

This restates, in Python on a Model's host arrays, what an unmodified
parmec.cpp does when it links against such a library: the call sequence of
dem() (parmec.cpp:2386-2517) with the host code between the calls
(read_gravity_and_damping, prescribe_acceleration, prescribe_velocity and
obstaclev, input.cpp:4199-4503).  It drives two libraries with the same
exports: libparmec_gb300.so's drop-in (include/parmec_ispc.h; the GPU parity
tests) and the reference's own hot path translated from its ISPC sources
(oracle/ispc_ref.py; the CPU pins and bench.py's reference arm).
"""
import ctypes

import numpy as np

from parmec_gb300 import abi
from parmec_gb300.driver import StepTables, obstaclev, step_times

NULL = None


def library(path=None):
    """The drop-in exports of libparmec_gb300.so, or (path given) of another
    library with the reference's ISPC entry points, such as the reference's
    own hot path built by oracle/ispc_ref.py."""
    lib = ctypes.CDLL(path) if path else abi.load_library()
    lib.adaptive_timestep.restype = ctypes.c_double
    lib.partitioning_create.restype = ctypes.c_void_p
    lib.master_alloc.restype = ctypes.c_void_p
    lib.slave_alloc.restype = ctypes.c_void_p
    if hasattr(lib, "pg_compat_kernel_launches"):
        lib.pg_compat_kernel_launches.restype = ctypes.c_longlong
    for name in ("master_alloc", "slave_alloc"):
        getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.master_free.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.slave_free.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.partitioning_destroy.argtypes = [ctypes.c_void_p]
    return lib


D = ctypes.c_double


class Host:
    """The reference's global buffers for one Model (parmec.cpp:61-285) and
    its contact-list arrays, as the loop passes them."""

    def __init__(self, lib, m, buffer_size=None, orient=False, ntasks=1):
        self.lib = lib
        self.m = m
        n = buffer_size or max(m.parnum, 1)
        self.size = n
        self.ntasks = ntasks
        self.master = lib.master_alloc(None, 0, n)
        self.slave = lib.slave_alloc(None, 0, n)
        # parmec.cpp passes its orient buffers (18 rows); the drop-in ignores
        # them for spheres, the reference's partitioning_store reads them
        # only for ellipsoids
        self.orient_rows = None
        self.orient = NULL
        if orient:
            self.orient_rows = np.zeros((18, max(m.ellnum, m.parnum, 1)))
            self.orient = abi.rows(self.orient_rows, 18)
            # shapes() tests radii[1][j] with the particle index j
            m.E.ensure(max(m.parnum, m.ellnum))

    def close(self):
        self.lib.master_free(self.master, self.size)
        self.lib.slave_free(self.slave, self.size)


def _prescribe_acceleration(m, tab, k, s):
    """prescribe_acceleration (input.cpp:4247-4341) on the host arrays."""
    P = m.P
    for i, pr in enumerate(m.prescribe):
        j = pr["part"]
        if pr["lin"] is not None and pr["linkind"] == 1:
            a = tab.prs_lin[k, i]
            ma = P.mass[j]
            P.force[0, j] = ma * a[0]
            P.force[1, j] = ma * a[1]
            P.force[2, j] = ma * a[2]
        elif pr["lin"] is not None and pr["linkind"] == 0:
            P.force[:, j] = 0.0
        if pr["ang"] is not None and pr["angkind"] == 1:
            a = [float(x) for x in tab.prs_ang[k, i]]
            J = [float(x) for x in P.inertia[:, j]]
            P.torque[0, j] = J[0] * a[0] + J[3] * a[1] + J[6] * a[2]
            P.torque[1, j] = J[1] * a[0] + J[4] * a[1] + J[7] * a[2]
            P.torque[2, j] = J[2] * a[0] + J[5] * a[1] + J[8] * a[2]
        elif pr["ang"] is not None and pr["angkind"] == 0:
            P.torque[:, j] = 0.0


def _prescribe_velocity(m, tab, k):
    """prescribe_velocity (input.cpp:4344-4421) on the host arrays."""
    P = m.P
    for i, pr in enumerate(m.prescribe):
        j = pr["part"]
        if pr["lin"] is not None and pr["linkind"] == 0:
            P.linear[:, j] = tab.prs_lin[k, i]
        if pr["ang"] is not None and pr["angkind"] == 0:
            o = [float(x) for x in tab.prs_ang[k, i]]
            L = [float(x) for x in P.rotation[:, j]]
            P.angular[0, j] = L[0] * o[0] + L[1] * o[1] + L[2] * o[2]
            P.angular[1, j] = L[3] * o[0] + L[4] * o[1] + L[5] * o[2]
            P.angular[2, j] = L[6] * o[0] + L[7] * o[1] + L[8] * o[2]
            P.angular[3:6, j] = o


def dem(lib, host, duration, step, adaptive=0.0):
    """One DEM() call (no output) through the drop-in exports; adaptive in
    (0, 1] runs forces with the stiffness terms and adaptive_timestep
    (parmec.cpp:2435-2450), sampling each step's host inputs at its start."""
    from parmec_gb300.springs import sort_springs
    m = host.m
    # dem() prologue: sort_materials and sort_springs (parmec.cpp:1636-1965)
    m.sort_materials()
    if m.springs_changed:
        sort_springs(m)
        m.springs_changed = False
    if m.torsion_changed:
        from parmec_gb300.torsion import sort_torsion
        sort_torsion(m)
        m.torsion_changed = False
    s = m.scene()
    obspnt, obsang, obslin = m._obs_views
    ntasks = host.ntasks
    orient = host.orient
    adapt = 0.0 < adaptive <= 1.0
    if adapt:
        times = None
    else:
        times, _ = step_times(m.curtime, duration, step)
        tab = StepTables(m, times, step, [1e9, 1e9], [None, None], [-1, -1])
    ellcon = tricon = faccon = 0
    step0 = step
    if m.curtime == 0.0:
        lib.euler(ntasks, s.parnum, s.angular, s.linear, s.rotation, s.position, D(0.5 * step0))
        lib.shapes(ntasks, s.ellnum, s.part, s.center, s.radii, orient, s.nodnum, s.nodes, s.nodpart, NULL,
                   s.facnum, s.facnod, s.factri, s.tri, s.rotation, s.position)
        a, l = obstaclev(m, 0.5 * step0)
        obsang[:a.size] = a[:obsang.size]
        obslin[:l.size] = l[:obslin.size]
        lib.obstacles(s.obsnum, s.trirng, s.obspnt, s.obsang, s.obslin, s.tri, D(step0))
    else:
        step0 = m.curstep
    lib.invert_inertia(ntasks, s.parnum, s.inertia, s.inverse, s.mass, s.invm)
    lib.restrain_velocities(ntasks, s.rstnum, s.rstpart, s.rstlin, s.rstang, s.linear, s.angular, s.rotation)
    tree = lib.partitioning_create(ntasks, s.ellnum - ellcon, s.center)
    kmax = np.zeros(max(1, s.parnum))
    emax = np.zeros(max(1, s.parnum))
    kact = [np.zeros(max(1, s.parnum)) for _ in range(3)]
    krot = [np.zeros(max(1, s.parnum)) for _ in range(6)]
    kact_p = (abi.D * 3)(*[abi.dptr(a) for a in kact])
    krot_p = (abi.D * 6)(*[abi.dptr(a) for a in krot])
    gravity = np.zeros(3)
    damping = np.zeros(6)
    step1 = step0

    def steps():
        nonlocal tab
        if not adapt:
            yield from enumerate(times)
            return
        time = 0.0
        while time < duration:
            s0 = step0
            tab = StepTables(m, [m.curtime], s0, [1e9, 1e9], [None, None], [-1, -1])
            yield 0, m.curtime
            time += 0.5 * (s0 + step1)                 # the body has set step1 (and step0 = step1)

    for k, t in steps():
        if lib.partitioning_store(ntasks, ctypes.c_void_p(tree), s.ellnum - ellcon, s.ellcol, s.part, s.center,
                                  s.radii, orient) > 0:
            # a leaf overflowed: parmec.cpp:2421-2428 rebuilds the tree
            lib.partitioning_destroy(ctypes.c_void_p(tree))
            tree = lib.partitioning_create(ntasks, s.ellnum - ellcon, s.center)
            if lib.partitioning_store(ntasks, ctypes.c_void_p(tree), s.ellnum - ellcon, s.ellcol, s.part,
                                      s.center, s.radii, orient) != 0:
                raise AssertionError("Repartitioning failed")
        lib.condet(ntasks, ctypes.c_void_p(tree), ctypes.c_void_p(host.master), s.parnum, s.ellnum - ellcon,
                   s.ellcol, s.part, s.center, s.radii, orient, s.trinum - tricon, s.tricol, s.triobs, s.tri)
        gravity[:] = tab.gravity[k]
        damping[:] = tab.damping[k]
        lib.forces(ntasks, ctypes.c_void_p(host.master), ctypes.c_void_p(host.slave), s.parnum,
                   s.angular, s.linear, s.rotation, s.position, s.inertia, s.inverse, s.mass, s.invm,
                   s.obspnt, s.obslin, s.obsang, s.parmat, NULL, s.pairnum, s.pairs, s.ikind, s.iparam,
                   D(step0), s.sprnum, s.sprtype, s.unspring, s.sprmap, s.sprpart, s.sprpnt, s.spring, s.spridx,
                   s.dashpot, s.dashidx, s.unload, s.unidx, s.yield_, s.sprdir, s.sprflg, s.sproffset,
                   s.sprfric, s.sprkskn, s.sprsdsp, s.stroke0, s.stroke, s.sprfrc, s.lcurve, s.lcidx,
                   abi.dptr(gravity), s.trqsprnum, s.trqsprpart, s.trqzdir0, s.trqxdir0, s.krpy, s.krpyidx,
                   s.drpy, s.drpyidx, s.trqcone, s.trqzdir1, s.trqxdir1, s.trqrpy, s.trqrpytot, s.trqrpyspr,
                   s.force, s.torque, kact_p, abi.dptr(kmax), abi.dptr(emax),
                   krot_p, 1 if adapt else 0, s.unsprnum,
                   s.tsprings, s.tspridx, s.msprings, s.mspridx, s.unlim, s.unent, s.unop, s.unabs, s.nsteps,
                   s.nfreq, s.unaction, s.activate, s.actidx, m.stepnum, D(t))
        if adapt:
            step1 = lib.adaptive_timestep(ntasks, s.parnum, s.mass, s.inertia, kact_p, abi.dptr(kmax),
                                          abi.dptr(emax), krot_p, D(step0), D(adaptive))
        else:
            step1 = step0
        lib.restrain_forces(ntasks, s.rstnum, s.rstpart, s.rstlin, s.rstang, s.force, s.torque)
        _prescribe_acceleration(m, tab, k, s)
        lib.dynamics(ntasks, ctypes.c_void_p(host.master), ctypes.c_void_p(host.slave), s.parnum, s.angular,
                     s.linear, s.rotation, s.position, s.inertia, s.inverse, s.mass, s.invm, abi.dptr(damping),
                     s.force, s.torque, s.flags, D(step0), D(step1))
        _prescribe_velocity(m, tab, k)
        lib.shapes(ntasks, s.ellnum - ellcon, s.part, s.center, s.radii, orient, s.nodnum, s.nodes, s.nodpart,
                   s.flags, s.facnum - faccon, s.facnod, s.factri, s.tri, s.rotation, s.position)
        a, l = obstaclev(m, t + step0)
        obsang[:a.size] = a[:obsang.size]
        obslin[:l.size] = l[:obslin.size]
        lib.obstacles(s.obsnum, s.trirng, s.obspnt, s.obsang, s.obslin, s.tri, D(0.5 * (step0 + step1)))
        m.curtime += 0.5 * (step0 + step1)
        step0 = step1
    lib.partitioning_destroy(ctypes.c_void_p(tree))
    m.curstep = step1
    m.stepnum += 1
    m.pull_obstacles()
    if hasattr(lib, "pg_compat_status"):
        st = lib.pg_compat_status()
        if st != 0:
            raise RuntimeError(f"drop-in entry points reported status {st}")


class Master(ctypes.Structure):
    """master_conpnt (condet.h:33-49) at REAL=8."""


Master._fields_ = [("master", ctypes.c_int * 8), ("slave", (ctypes.c_int * 8) * 2),
                   ("color", (ctypes.c_int * 8) * 2), ("point", (ctypes.c_double * 8) * 3),
                   ("normal", (ctypes.c_double * 8) * 3), ("depth", ctypes.c_double * 8),
                   ("force", (ctypes.c_double * 8) * 3), ("kcur", ctypes.c_double * 8),
                   ("ecur", ctypes.c_double * 8), ("state", (ctypes.c_double * 8) * 8),
                   ("size", ctypes.c_int), ("next", ctypes.POINTER(Master)), ("lock", ctypes.c_int)]


def master_lists(host):
    """Every contact in the master lists, in list order: a dict of arrays with
    the master particle, the slave code (sphere index, or -(triangle+1)), the
    slave particle, point, normal, depth, force and tangential state."""
    P = host.m.parnum
    arr = (Master * P).from_address(host.master)
    out = {k: [] for k in ("mpart", "code", "spart", "point", "normal", "depth", "force", "state")}
    for p in range(P):
        b = arr[p]
        while True:
            for k in range(b.size):
                out["mpart"].append(p)
                out["code"].append(b.slave[1][k])
                out["spart"].append(b.slave[0][k])
                out["point"].append([b.point[c][k] for c in range(3)])
                out["normal"].append([b.normal[c][k] for c in range(3)])
                out["depth"].append(b.depth[k])
                out["force"].append([b.force[c][k] for c in range(3)])
                out["state"].append([b.state[c][k] for c in range(3)])
            if not b.next:
                break
            b = b.next.contents
    return {k: np.array(v) for k, v in out.items()}


def critical(lib, host):
    """CRITICAL's two exports (critical_perspring, critical_perparticle) on
    the host arrays, as input.cpp:3064-3140 calls them: per-spring and
    per-particle (step, omega, ratio) arrays."""
    m = host.m
    s = m.scene()
    P, S = m.parnum, m.sprnum
    out_s = [np.zeros(max(1, S)) for _ in range(3)]
    out_p = [np.zeros(max(1, P)) for _ in range(3)]
    kact = [np.zeros(max(1, P)) for _ in range(3)]
    krot = [np.zeros(max(1, P)) for _ in range(6)]
    kmax, emax = np.zeros(max(1, P)), np.zeros(max(1, P))
    if S:
        lib.critical_perspring(S, s.sprpart, s.sprpnt, s.sprdir, s.spring, s.spridx, s.dashpot, s.dashidx,
                               s.inverse, s.invm, s.position, *(abi.dptr(a) for a in out_s))
    lib.critical_perparticle.restype = ctypes.c_double
    lib.critical_perparticle(host.ntasks, ctypes.c_void_p(host.master), ctypes.c_void_p(host.slave), P, s.mass,
                             s.inertia, s.invm, s.inverse, s.rotation, s.position, S, s.sprflg, s.sprpart,
                             s.sprpnt, s.sprdir, s.spring, s.spridx, s.dashpot, s.dashidx,
                             (abi.D * 3)(*[abi.dptr(a) for a in kact]), abi.dptr(kmax), abi.dptr(emax),
                             (abi.D * 6)(*[abi.dptr(a) for a in krot]), *(abi.dptr(a) for a in out_p))
    return tuple(a[:S] for a in out_s), tuple(a[:P] for a in out_p)
