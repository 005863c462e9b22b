"""Adaptive time stepping (DEM adaptive=..., parmec.cpp:2443-2450,
adaptive_timestep parmec.ispc:397-420): the next step is 'adaptive' times the
smallest per-particle critical step estimated from the current contacts and
springs.  CPU tests check the oracle against closed forms; the GPU tests
check the device path against the oracle bit for bit."""
import math

import numpy as np
import pytest

from helpers import assert_bitwise, assert_spheres_bitwise, make_collision_scene
from parmec_gb300.model import Model


def damped_step(omega, ksi):
    return (2.0 / omega) * (math.sqrt(1.0 + ksi * ksi) - ksi)


def sphere_on_plane(kn=1e6, damper=0.2):
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    r = 0.05
    p = m.sphere((0.3, -0.2, r - 1e-4), r, mat, 1)
    L = 1.0
    m.obstacle([(-L, -L, 0.0, L, -L, 0.0, L, L, 0.0), (-L, -L, 0.0, L, L, 0.0, -L, L, 0.0)], 2)
    m.granular(0, 0, kn, damper, 0.5)
    m.set_gravity(0.0, 0.0, -9.81)
    return m, p


def test_single_contact_step(oracle_lib):
    """One sphere resting on a plane: step1 = adaptive * min(h_xyz, h_rot) of
    the single-contact closed form (arm along the normal)."""
    from oracle.pyoracle import OracleEngine
    m, p = sphere_on_plane()
    eng = OracleEngine()
    dt = 1e-6
    m.dem(3 * dt - 0.5 * dt, dt, interval=1e9, adaptive=0.5, engine=eng)
    c = eng.contacts()
    assert len(c["mpart"]) == 1
    mass, ine = m.P.mass[p], m.P.inertia[0, p]
    arm = c["point"][0] - m.P.position[0:3, p]
    w = math.sqrt(1e6 / mass)
    wr = math.sqrt(1e6 * (arm[0] ** 2 + arm[1] ** 2 + arm[2] ** 2) / ine)
    e = 0.2 * 2.0 * math.sqrt(1e6 * mass)
    h = min(damped_step(w, e / (2 * mass * w)), damped_step(wr, e / (2 * ine * wr)))
    assert abs(m.curstep - 0.5 * h) <= 1e-6 * h
    hp, om, ra = eng.critical_terms()
    assert abs(hp[p] - h) <= 1e-6 * h


def test_free_particle_keeps_its_step(oracle_lib):
    """Nothing restrains the particle: step1 = step0 (parmec.ispc:419)."""
    from oracle.pyoracle import OracleEngine
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    m.velocity(0, linear=(1.0, 0.0, 0.0))
    m.dem(1e-4 - 0.5e-5, 1e-5, interval=1e9, adaptive=0.5, engine=OracleEngine())
    assert m.curstep == 1e-5
    assert abs(m.P.position[0, 0] - 1.05e-4) < 1e-12        # half step, then 10 steps


def test_time_accumulates_chosen_steps(oracle_lib):
    """curtime advances by (step0 + step1)/2 per step and ends past the duration."""
    from oracle.pyoracle import OracleEngine
    m, _ = make_collision_scene(n_side=3)
    dt = 1e-5
    m.dem(40 * dt, dt, interval=1e9, adaptive=0.2, engine=OracleEngine())
    assert m.curtime >= 40 * dt
    assert m.curstep != dt


def test_contact_terms_match_critical(oracle_lib):
    """The in-step stiffness terms of contacts equal CRITICAL's per-particle
    estimate over the same contacts (no springs), up to the positions moved by
    the last step's dynamics."""
    from oracle.pyoracle import OracleEngine
    from oracle.critical_host import critical_perparticle
    m, dt = make_collision_scene(n_side=4, speed=0.2)
    eng = OracleEngine()
    m.dem(20 * dt - 0.5 * dt, dt, interval=1e9, adaptive=1.0, engine=eng)
    h_dev, _, _ = eng.critical_terms()
    h_host, _, _ = critical_perparticle(m, eng.contacts())
    touched = h_host < 1e300
    assert touched.sum() > 10
    assert np.array_equal(touched, h_dev < 1e300)
    assert np.allclose(h_dev[touched], h_host[touched], rtol=1e-6)


def test_rejects_out_of_range():
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    with pytest.raises(ValueError):
        m.dem(1e-3, 1e-5, adaptive=1.5)


# ------------------------------------------------------------------ GPU parity
def run_pair(make, duration, step, adaptive):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    mg, _ = make()
    mo, _ = make()
    eg = GpuEngine(record_geometry=True)
    eo = OracleEngine()
    mg.dem(duration, step, interval=1e9, adaptive=adaptive, engine=eg)
    mo.dem(duration, step, interval=1e9, adaptive=adaptive, engine=eo)
    return mg, mo, eg, eo


@pytest.mark.gpu
def test_gpu_adaptive_collisions_bitwise(gpu_lib, oracle_lib):
    """Contacts form and break while the step adapts: the chosen steps, the
    time and every state array equal the oracle's bit for bit."""
    make = lambda: make_collision_scene(n_side=5)
    _, dt = make()
    mg, mo, eg, eo = run_pair(make, 60 * dt, dt, 0.7)
    assert mg.curstep == mo.curstep and mg.curtime == mo.curtime
    assert mg.curstep != dt
    assert_bitwise(mg, mo)
    assert_spheres_bitwise(mg, mo)


@pytest.mark.gpu
def test_gpu_adaptive_springs_bitwise(gpu_lib, oracle_lib):
    """Spring stiffness terms, including the chunked long runs of the base
    particle (289 springs), give the oracle's steps bit for bit."""
    from parmec_gb300.scenes import spring_lattice

    def make():
        m, dt = spring_lattice(17)
        return m, dt
    _, dt = make()
    mg, mo, eg, eo = run_pair(make, 30 * dt, dt, 0.5)
    assert mg.curstep == mo.curstep and mg.curtime == mo.curtime
    assert_bitwise(mg, mo)


@pytest.mark.gpu
def test_gpu_adaptive_then_fixed(gpu_lib, oracle_lib):
    """An adaptive DEM followed by a fixed-step DEM on the same session: the
    fixed graph is re-captured and both engines stay equal."""
    make = lambda: make_collision_scene(n_side=4)
    _, dt = make()
    mg, mo, eg, eo = run_pair(make, 20 * dt, dt, 0.5)
    for m, e in ((mg, eg), (mo, eo)):
        m.dem(10 * dt, dt, interval=1e9, engine=e)
    assert mg.curtime == mo.curtime
    assert_bitwise(mg, mo)
