"""CRITICAL (input.cpp:3034-3154): per-spring and per-particle critical step
estimates against closed forms (CPU: springs need no device session)."""
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


def test_particle_on_a_spring():
    """kact = 1 per axis (no direction yet), k = the curve slope, no arm:
    h = 2/sqrt(k/m) without damping."""
    m, p = spring_particle()
    w = math.sqrt(1e4 / m.P.mass[p])
    h = m.critical()
    assert abs(h - 2.0 / w) <= 1e-12 * h
    (hp, i, om, ra), = m.critical(perparticle=1)
    assert i == p and abs(om - w) <= 1e-12 * w and ra == 0.0


def test_particle_on_a_damped_spring():
    m, p = spring_particle(ratio=0.3)
    w = math.sqrt(1e4 / m.P.mass[p])
    h = m.critical()
    assert abs(h - damped_step(w, 0.3)) <= 1e-12 * h
    s, q = m.critical(perspring=1, perparticle=1)
    assert len(s) == 1 and len(q) == 1
    assert abs(s[0][0] - damped_step(w, 0.3)) <= 1e-12 * h      # the spring's own estimate agrees


def test_nothing_restrains_nothing():
    """No contact and no spring: REAL_MAX, as the reference returns before any contact."""
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    assert m.critical() == REAL_MAX


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


def engines():
    from oracle.pyoracle import OracleEngine
    return [pytest.param(lambda: OracleEngine(), id="oracle"),
            pytest.param(lambda: __import__("parmec_gb300.engine", fromlist=["GpuEngine"]).GpuEngine(),
                         id="gpu", marks=pytest.mark.gpu)]


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
