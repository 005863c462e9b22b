"""CRITICAL (input.cpp:3034-3154): per-spring and per-particle critical step
estimates against closed forms, through the oracle's restatement on the CPU
and the device (pg_session_critical) on the GPU."""
import math

import pytest

from parmec_gb300.model import REAL_MAX, Model


def spring_particle(k=1e4, ratio=None, mass_density=1000.0):
    m = Model()
    mat = m.material(mass_density, 1e9, 0.25)
    p = m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    m.spring(p, (0.0, 0.0, 0.0), -1, (0.0, 0.0, -0.1), [-1.0, -k, 1.0, k],
             dashpot=ratio if ratio is not None else None)
    return m, p


def damped_step(omega, ksi):
    return (2.0 / omega) * (math.sqrt(1.0 + ksi * ksi) - ksi)


def engines():
    from oracle.pyoracle import OracleEngine
    return [pytest.param(lambda: OracleEngine(), id="oracle"),
            pytest.param(lambda: __import__("parmec_gb300.engine", fromlist=["GpuEngine"]).GpuEngine(),
                         id="gpu", marks=pytest.mark.gpu)]


def attached(make_engine, m, request):
    """An engine of the parametrised kind attached to m (springs sorted first,
    as DEM and CRITICAL sort them)."""
    from parmec_gb300.springs import sort_springs
    if "gpu" in request.node.callspec.id:
        request.getfixturevalue("gpu_lib")
    m.sort_materials()
    if m.springs_changed:
        sort_springs(m)
        m.springs_changed = False
    eng = make_engine()
    eng.attach(m)
    return eng


@pytest.mark.parametrize("make_engine", engines())
def test_particle_on_a_spring(make_engine, request):
    """kact = 1 per axis (no direction yet), k = the curve slope, no arm:
    h = 2/sqrt(k/m) without damping."""
    m, p = spring_particle()
    eng = attached(make_engine, m, request)
    w = math.sqrt(1e4 / m.P.mass[p])
    h = m.critical(engine=eng)
    assert abs(h - 2.0 / w) <= 1e-12 * h
    (hp, i, om, ra), = m.critical(perparticle=1, engine=eng)
    assert i == p and abs(om - w) <= 1e-12 * w and ra == 0.0


@pytest.mark.parametrize("make_engine", engines())
def test_particle_on_a_damped_spring(make_engine, request):
    m, p = spring_particle(ratio=0.3)
    eng = attached(make_engine, m, request)
    w = math.sqrt(1e4 / m.P.mass[p])
    h = m.critical(engine=eng)
    assert abs(h - damped_step(w, 0.3)) <= 1e-12 * h
    s, q = m.critical(perspring=1, perparticle=1, engine=eng)
    assert len(s) == 1 and len(q) == 1
    assert abs(s[0][0] - damped_step(w, 0.3)) <= 1e-12 * h      # the spring's own estimate agrees


@pytest.mark.parametrize("make_engine", engines())
def test_nothing_restrains_nothing(make_engine, request):
    """No contact and no spring: REAL_MAX, as the reference returns before any contact."""
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    assert m.critical(engine=attached(make_engine, m, request)) == REAL_MAX


def test_argument_ranges():
    m, p = spring_particle()
    with pytest.raises(ValueError):
        m.critical(perspring=5)
    with pytest.raises(ValueError):
        m.critical(perparticle=-2)


def sphere_on_plane():
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    r = 0.05
    p = m.sphere((0.3, -0.2, r - 1e-4), r, mat, 1)              # inside one triangle, off the shared edge
    L = 1.0
    m.obstacle([(-L, -L, 0.0, L, -L, 0.0, L, L, 0.0), (-L, -L, 0.0, L, L, 0.0, -L, L, 0.0)], 2)
    m.granular(0, 0, 1e6, 0.2, 0.5)
    m.set_gravity(0.0, 0.0, -9.81)
    return m, p


def sphere_pair():
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    a = m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    b = m.sphere((0.0999, 0.0, 0.0), 0.05, mat, 1)
    m.granular(0, 0, 1e6, 0.2, 0.5)
    return m, a, b


@pytest.mark.parametrize("make_engine", engines())
def test_sphere_on_a_plane(make_engine, oracle_lib, request):
    """One contact along +z with arm a = point - centre: translational
    omega = sqrt(kn/m), rotational omega = sqrt(kn a_perp^2 / J), damping
    ratio en (obstacle: ma = m), and the smaller damped step wins."""
    if "gpu" in request.node.callspec.id:
        request.getfixturevalue("gpu_lib")
    m, p = sphere_on_plane()
    dt = 1e-6
    eng = make_engine()
    m.dem(5 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    c = eng.contacts()
    assert len(c["mpart"]) == 1
    mass = m.P.mass[p]
    ine = m.P.inertia[0, p]
    arm = c["point"][0] - m.P.position[0:3, p]
    perp2 = arm[2] * arm[2] + arm[1] * arm[1]         # about x; y likewise, z none (arm along z)
    w = math.sqrt(1e6 / mass)
    wr = math.sqrt(1e6 * perp2 / ine)
    e = 0.2 * 2.0 * math.sqrt(1e6 * mass)
    hx = damped_step(w, e / (2.0 * mass * w))
    hr = damped_step(wr, e / (2.0 * ine * wr))
    (h, i, om, ra), = m.critical(perparticle=1)
    assert i == p
    assert abs(h - min(hx, hr)) <= 1e-9 * h
    assert abs(om - max(w, wr)) <= 1e-9 * om
    assert m.critical() == h


@pytest.mark.parametrize("make_engine", engines())
def test_sphere_pair(make_engine, oracle_lib, request):
    """Master and slave both see the contact (the slave through the force
    direction): equal estimates, damping ratio en/sqrt(2) (ma = m/2)."""
    if "gpu" in request.node.callspec.id:
        request.getfixturevalue("gpu_lib")
    m, a, b = sphere_pair()
    dt = 1e-6
    eng = make_engine()
    m.dem(3 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    c = eng.contacts()
    assert len(c["mpart"]) == 1
    mass = m.P.mass[a]
    ine = m.P.inertia[0, a]
    w = math.sqrt(1e6 / mass)
    e = 0.2 * 2.0 * math.sqrt(1e6 * 0.5 * mass)
    out = m.critical(perparticle=2)
    assert sorted(x[1] for x in out) == [a, b]
    for h, i, om, ra in out:
        arm = c["point"][0] - m.P.position[0:3, i]
        wr = math.sqrt(1e6 * (arm[0] * arm[0] + arm[1] * arm[1]) / ine)   # about z (y likewise)
        hx = damped_step(w, e / (2.0 * mass * w))
        hr = damped_step(wr, e / (2.0 * ine * wr))
        assert abs(h - min(hx, hr)) <= 1e-9 * h
        assert abs(om - max(w, wr)) <= 1e-9 * om
        assert abs(e / (2.0 * mass * w) - 0.2 / math.sqrt(2.0)) <= 1e-12


@pytest.mark.gpu
def test_gpu_critical_matches_restatement(gpu_lib, oracle_lib):
    """The device CRITICAL (pg_session_critical) against the host
    restatement over the same contacts and springs: colliding spheres in a
    box (master and slave contact terms), and bodies with full inertia
    tensors on springs of every direction mode with a prescribed base."""
    import numpy as np
    from helpers import make_collision_scene
    from oracle.critical_host import critical_perparticle, critical_perspring
    from parmec_gb300.engine import GpuEngine
    from test_gpu_springs import lattice
    cases = ((lambda: make_collision_scene(n_side=5), 40), (lambda: (lattice(), 2e-5), 60))
    for make, steps in cases:
        m, dt = make()
        eng = GpuEngine(record_geometry=True)
        m.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        h, o, r = eng.critical(0)
        hh, oh, rh = critical_perparticle(m, eng.contacts())
        touched = hh < 1e300
        assert touched.sum() > 10
        assert np.array_equal(touched, h < 1e300)
        # the rotational frequency is an eigenvalue of a nearly double-rooted
        # 3x3 (a contact arm gives a rank-two stiffness): last-bit differences
        # of two evaluations grow by its conditioning, so 1e-7 relative
        for a, b in ((h, hh), (o, oh), (r, rh)):
            assert np.allclose(a[touched], b[touched], rtol=1e-7, atol=0.0)
        if m.sprnum:
            hs, os_, rs = eng.critical(1)
            for a, b in zip((hs, os_, rs), critical_perspring(m)):
                assert np.allclose(a, np.array(b), rtol=1e-7, atol=0.0)
        # Model.critical takes the session the DEM call stepped with
        (hp, i, om, ra), = m.critical(perparticle=1)
        assert hp == float(np.min(h)) and i == int(np.argmin(h))
        eng.close()
