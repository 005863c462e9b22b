"""The drop-in ISPC entry points (include/parmec_ispc.h) on the GPU.

parmec.cpp's dem() loop over condet/forces/dynamics/shapes/obstacles/euler/
invert_inertia (tests/ispc_loop.py) must give the oracle's state bit for bit,
as the session does: the entry points run the same kernels, with host arrays
copied in and out at every call.
"""
import ctypes

import numpy as np
import pytest

from oracle import dem_loop as ispc_loop
from helpers import assert_bitwise, assert_spheres_bitwise, bits, make_collision_scene

pytestmark = pytest.mark.gpu


def run_both(make, steps, calls=1, skin=0.0):
    from oracle.pyoracle import OracleEngine
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    lib.pg_compat_set_skin(ctypes.c_double(skin))
    mc, dt = make()
    mo, _ = make()
    host = ispc_loop.Host(lib, mc)
    eo = OracleEngine()
    for c in range(calls):
        mo.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eo)
        ispc_loop.dem(lib, host, steps * dt - 0.5 * dt, dt)
        assert_bitwise(mc, mo, where=f"after DEM call {c + 1}: ")
    return lib, host, mc, mo, eo


def materialized(lib, host):
    """Contacts written into the reference's list layout, as (particle, code, force) rows."""
    P = host.m.parnum

    class Master(ctypes.Structure):
        pass
    Master._fields_ = [("master", ctypes.c_int * 8), ("slave", (ctypes.c_int * 8) * 2),
                       ("color", (ctypes.c_int * 8) * 2), ("point", (ctypes.c_double * 8) * 3),
                       ("normal", (ctypes.c_double * 8) * 3), ("depth", ctypes.c_double * 8),
                       ("force", (ctypes.c_double * 8) * 3), ("kcur", ctypes.c_double * 8),
                       ("ecur", ctypes.c_double * 8), ("state", (ctypes.c_double * 8) * 8),
                       ("size", ctypes.c_int), ("next", ctypes.POINTER(Master)), ("lock", ctypes.c_int)]
    n = lib.pg_compat_materialize(ctypes.c_void_p(host.master), ctypes.c_void_p(host.slave), P)
    assert n >= 0
    arr = (Master * P).from_address(host.master)
    rows = []
    for p in range(P):
        b = arr[p]
        while True:
            for k in range(b.size):
                rows.append((p, b.slave[1][k], b.force[0][k], b.force[1][k], b.force[2][k], b.depth[k]))
            if not b.next:
                break
            b = b.next.contents
    assert len(rows) == n
    return rows


def test_dropin_collisions_bitwise(gpu_lib, oracle_lib):
    """Sphere-sphere and sphere-triangle contacts through condet/forces/dynamics."""
    lib, host, mc, mo, eo = run_both(lambda: make_collision_scene(n_side=5), 120)
    assert_bitwise(mc, mo)
    assert_spheres_bitwise(mc, mo)
    rows = materialized(lib, host)
    co = eo.contacts()
    assert len(rows) == len(co["mpart"]) > 10
    got = sorted((r[0], r[1]) for r in rows)
    want = sorted(zip(co["mpart"].tolist(), co["code"].tolist()))
    assert got == want
    fg = np.array(sorted((r[0], r[1], r[2], r[3], r[4]) for r in rows))[:, 2:]
    f = co["force"]
    fo = np.array(sorted(zip(co["mpart"].tolist(), co["code"].tolist(), f[:, 0], f[:, 1], f[:, 2])))[:, 2:]
    assert np.array_equal(bits(fg), bits(fo))
    assert lib.pg_compat_kernel_launches() > 0
    host.close()


def test_dropin_moving_obstacle_two_calls(gpu_lib, oracle_lib):
    """A rotating wall, two DEM() calls: contact state survives between calls."""
    lib, host, mc, mo, eo = run_both(lambda: make_collision_scene(n_side=4, moving=True, seed=11), 70, calls=2)
    assert_bitwise(mc, mo)
    a = mc.Tr.tri[:, :mc.trinum]
    b = mo.Tr.tri[:, :mo.trinum]
    assert np.array_equal(bits(a), bits(b))
    host.close()


def test_dropin_small_skin(gpu_lib, oracle_lib):
    """A tiny skin: condet() rebuilds the candidate lists nearly every step."""
    lib, host, mc, mo, eo = run_both(lambda: make_collision_scene(n_side=4, seed=5), 60, skin=1e-5)
    assert_bitwise(mc, mo)
    host.close()
    lib.pg_compat_set_skin(ctypes.c_double(0.0))


def test_dropin_springs_and_prescribe(gpu_lib, oracle_lib):
    """The spring lattice with a prescribed base: springs in forces(), the
    prescribed motion on the host between forces() and dynamics()."""
    from test_gpu_springs import lattice, spring_state_equal
    step = 2e-5
    lib, host, mc, mo, eo = run_both(lambda: (lattice(), step), 200)
    assert_bitwise(mc, mo)
    spring_state_equal(mc, mo)
    host.close()


def test_dropin_unsupported_cases_report(gpu_lib):
    """Ellipsoids report PG_ERR_UNSUPPORTED instead of running."""
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    m, dt = make_collision_scene(n_side=2)
    m.E.radii[1, 0] = 0.01                     # an ellipsoid
    host = ispc_loop.Host(lib, m)
    with pytest.raises(RuntimeError):
        ispc_loop.dem(lib, host, 2.5 * dt, dt)
    host.close()
    assert lib.pg_compat_status() == 0               # read (and cleared) by ispc_loop.dem's raise
    lib.pg_compat_exit_on_error(1)


def test_dropin_adaptive_bitwise(gpu_lib, oracle_lib):
    """Adaptive stepping through forces(adaptive=1) + adaptive_timestep: the
    stiffness terms come back to the host arrays, the step is chosen on the
    device, and the state and chosen steps equal the oracle's bit for bit."""
    from oracle.pyoracle import OracleEngine
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    lib.pg_compat_set_skin(ctypes.c_double(0.0))
    mc, dt = make_collision_scene(n_side=4)
    mo, _ = make_collision_scene(n_side=4)
    host = ispc_loop.Host(lib, mc)
    eo = OracleEngine()
    mo.dem(40 * dt, dt, interval=1e9, adaptive=0.6, engine=eo)
    ispc_loop.dem(lib, host, 40 * dt, dt, adaptive=0.6)
    assert mc.curstep == mo.curstep and mc.curtime == mo.curtime
    assert mc.curstep != dt
    assert_bitwise(mc, mo)
    host.close()


def test_dropin_adaptive_springs_bitwise(gpu_lib, oracle_lib):
    """Analytical bodies with full inertia tensors on springs of every
    direction mode and a prescribed base, with adaptive steps (the rotational
    eigenproblem takes its general branch)."""
    from oracle.pyoracle import OracleEngine
    from test_gpu_springs import lattice
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    step = 2e-5
    mc, mo = lattice(), lattice()
    host = ispc_loop.Host(lib, mc)
    eo = OracleEngine()
    mo.dem(40 * step, step, interval=1e9, adaptive=0.5, engine=eo)
    ispc_loop.dem(lib, host, 40 * step, step, adaptive=0.5)
    assert mc.curstep == mo.curstep and mc.curtime == mo.curtime
    assert_bitwise(mc, mo)
    host.close()


def test_dropin_restraints_bitwise(gpu_lib, oracle_lib):
    """restrain_velocities at the DEM call and restrain_forces every step
    through the exports, beside the oracle's restraints."""
    from oracle.pyoracle import OracleEngine

    def make():
        m, dt = make_collision_scene(n_side=3)
        m.restrain(0, linear=[0.0, 0.0, 1.0])
        m.restrain(1, linear=[1.0, 1.0, 0.0, 0.0, 1.0, 1.0], angular=[0.0, 0.0, 1.0])
        m.restrain(1, angular=[1.0, 0.0, 0.0])
        m.restrain(5, angular=[1.0, 0.2, 0.0, 0.0, 1.0, 0.3, 0.1, 0.0, 1.0])
        return m, dt
    run_both(make, 30)


def test_dropin_critical(gpu_lib, oracle_lib):
    """critical_perparticle and critical_perspring through the drop-in
    exports (input.cpp:3064-3140) after a DEM call: the device contact
    lists of the master array and the host spring arrays, against the host
    restatement over the oracle's equal state; and eqm (the EQM command)
    against the model's."""
    from oracle.critical_host import critical_perparticle, critical_perspring
    from test_gpu_springs import lattice
    lib, host, mc, mo, eo = run_both(lambda: make_collision_scene(n_side=5), 40)
    _, (h, o, r) = ispc_loop.critical(lib, host)
    hh, oh, rh = critical_perparticle(mo, eo.contacts())
    touched = hh < 1e300
    assert touched.sum() > 10 and np.array_equal(touched, h < 1e300)
    # rotational frequencies: eigenvalues of nearly double-rooted 3x3s, 1e-7
    for a, b in ((h, hh), (o, oh), (r, rh)):
        assert np.allclose(a[touched], b[touched], rtol=1e-7, atol=0.0)
    host.close()
    step = 2e-5
    lib, host, mc, mo, eo = run_both(lambda: (lattice(), step), 50)
    (hs, os_, rs), (h, o, r) = ispc_loop.critical(lib, host)
    for a, b in zip((hs, os_, rs), critical_perspring(mo)):
        assert np.allclose(a, np.array(b), rtol=1e-7, atol=0.0)
    hh, oh, rh = critical_perparticle(mo, eo.contacts())
    for a, b in ((h, hh), (o, oh), (r, rh)):
        assert np.allclose(a, b, rtol=1e-7, atol=0.0)
    s = mc.scene()
    p1 = (ctypes.c_double * 3)(0.001, 0.002, 0.0)
    p2 = (ctypes.c_double * 3)(0.0, 0.0, -0.01)
    for part2, d in ((-1, (0.0, 0.0, 0.0)), (1, (0.0, 0.0, 1.0)), (3, (0.6, 0.8, 0.0))):
        dd = (ctypes.c_double * 3)(*d)
        lib.eqm.restype = ctypes.c_double
        got = lib.eqm(0, p1, part2, p2, dd, s.inverse, s.invm, s.position)
        want = mc.eqm(0, tuple(p1), part2, tuple(p2) if part2 >= 0 else None, d)
        assert abs(got - want) <= 1e-12 * abs(want)
    host.close()


def test_dropin_critical_against_reference(gpu_lib, oracle_lib):
    """The drop-in CRITICAL against the reference's own critical_perparticle
    (oracle/ispc_ref.py, when its translation is on this host): spheres
    resting on a plane, each master of its contacts."""
    from oracle import ispc_ref
    from test_reference_pin import spheres_on_a_plane
    if ispc_ref.build() is None:
        pytest.skip("the reference's translation is not on this host")
    ref = ispc_loop.library(ispc_ref.LIB)
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    lib.pg_compat_set_skin(ctypes.c_double(0.0))
    mc, dt = spheres_on_a_plane()
    mr, _ = spheres_on_a_plane()
    hc = ispc_loop.Host(lib, mc)
    hr = ispc_loop.Host(ref, mr, orient=True)
    ispc_loop.dem(lib, hc, 30 * dt - 0.5 * dt, dt)
    ispc_loop.dem(ref, hr, 30 * dt - 0.5 * dt, dt)
    _, (h, o, r) = ispc_loop.critical(lib, hc)
    _, (h2, o2, r2) = ispc_loop.critical(ref, hr)
    touched = h2 < 1e300
    assert touched.sum() >= 20 and np.array_equal(touched, h < 1e300)
    for a, b in ((h, h2), (o, o2), (r, r2)):
        assert np.allclose(a[touched], b[touched], rtol=1e-7, atol=0.0)
    hc.close()
