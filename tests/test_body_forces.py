"""Prescribed body forces, the coupling interface of the reference's library
(struct prescribed_body_force, parmec.h:281-289; prescribe_body_forces,
parmec.cpp:2202-2224): each step the particle's force and torque after
forces() are exported (inner) and the prescribed ones (outer) added."""
import numpy as np
import pytest

from helpers import assert_bitwise, make_collision_scene
from parmec_gb300.model import Model


def sphere():
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    p = m.sphere((0.0, 0.0, 0.0), 0.1, mat, 1)
    m.set_gravity(0.0, 0.0, -9.81)
    return m, p


def test_outer_force_accelerates_inner_is_gravity(oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, p = sphere()
    mass = m.P.mass[p]
    m.set_body_force(p, force=(2.0 * mass, 0.0, 0.0), torque=(0.0, 0.0, 0.0))
    dt = 1e-4
    m.dem(100 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
    assert abs(m.P.linear[0, p] - 2.0 * 100 * dt) < 1e-12          # a = 2 m/s^2 along x
    f, t = m.body_force_inner(p)
    assert f == (0.0, 0.0, -9.81 * mass) and t == (0.0, 0.0, 0.0)   # exported before the addition


def test_outer_torque_spins(oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, p = sphere()
    J = m.P.inertia[0, p]
    m.set_body_force(p, torque=(0.0, 0.0, 3.0 * J))
    dt = 1e-4
    m.dem(50 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
    assert abs(m.P.angular[5, p] - 3.0 * 50 * dt) < 1e-10


def test_record_removed():
    m, p = sphere()
    m.set_body_force(p, force=(1.0, 0.0, 0.0))
    m.set_body_force(p, force=None)
    assert m.body_forces == {}
    with pytest.raises(ValueError):
        m.set_body_force(3, force=(1.0, 0.0, 0.0))


@pytest.mark.gpu
def test_gpu_body_forces_bitwise(gpu_lib, oracle_lib):
    """Colliding spheres with body forces on a few of them, over two DEM
    calls with changed outer forces between them: state and exported inner
    forces equal the oracle's bit for bit."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine

    def make():
        m, dt = make_collision_scene(n_side=4)
        m.set_body_force(3, force=(0.5, -0.2, 1.0), torque=(0.0, 1e-3, 0.0))
        m.set_body_force(17, force=(-1.0, 0.0, 0.0))
        return m, dt
    mg, dt = make()
    mo, _ = make()
    eg, eo = GpuEngine(), OracleEngine()
    for k in range(2):
        if k:
            for m in (mg, mo):
                m.set_body_force(17, force=(0.0, 2.0, 0.0), torque=(1e-3, 0.0, 0.0))
        mg.dem(30 * dt, dt, interval=1e9, engine=eg)
        mo.dem(30 * dt, dt, interval=1e9, engine=eo)
        assert_bitwise(mg, mo)
        for p in (3, 17):
            a, b = mg.body_force_inner(p), mo.body_force_inner(p)
            assert np.array_equal(np.array(a).view(np.int64), np.array(b).view(np.int64))
