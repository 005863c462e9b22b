"""parmec.cpp's dem() loop over the drop-in ISPC entry points.

This restates, in Python on a Model's host arrays, what an unmodified
parmec.cpp does when it links against libparmec_gb300.so in place of the
ISPC objects (include/parmec_ispc.h): the call sequence of dem()
(parmec.cpp:2386-2517) with the host code between the calls
(read_gravity_and_damping, prescribe_acceleration, prescribe_velocity and
obstaclev, input.cpp:4199-4503).  Test infrastructure: the GPU parity tests
run it beside the oracle.
"""
import ctypes

import numpy as np

from parmec_gb300 import abi
from parmec_gb300.driver import StepTables, obstaclev, step_times

NULL = None


def library():
    lib = abi.load_library()
    lib.adaptive_timestep.restype = ctypes.c_double
    lib.partitioning_create.restype = ctypes.c_void_p
    lib.master_alloc.restype = ctypes.c_void_p
    lib.slave_alloc.restype = ctypes.c_void_p
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

    def __init__(self, lib, m, buffer_size=None):
        self.lib = lib
        self.m = m
        n = buffer_size or max(m.parnum, 1)
        self.size = n
        self.master = lib.master_alloc(None, 0, n)
        self.slave = lib.slave_alloc(None, 0, n)

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
    ntasks = 1
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
        lib.shapes(ntasks, s.ellnum, s.part, s.center, s.radii, NULL, s.nodnum, s.nodes, s.nodpart, NULL,
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
                                  s.radii, NULL) > 0:
            raise AssertionError("partitioning_store overflowed")
        lib.condet(ntasks, ctypes.c_void_p(tree), ctypes.c_void_p(host.master), s.parnum, s.ellnum - ellcon,
                   s.ellcol, s.part, s.center, s.radii, NULL, s.trinum - tricon, s.tricol, s.triobs, s.tri)
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
                   s.force, s.torque, kact_p if adapt else NULL, abi.dptr(kmax), abi.dptr(emax),
                   krot_p if adapt else NULL, 1 if adapt else 0, s.unsprnum,
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
        lib.shapes(ntasks, s.ellnum - ellcon, s.part, s.center, s.radii, NULL, s.nodnum, s.nodes, s.nodpart,
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
    st = lib.pg_compat_status()
    if st != 0:
        raise RuntimeError(f"drop-in entry points reported status {st}")
