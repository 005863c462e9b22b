"""RESTRAIN (input.cpp:2458-2644, restrain.ispc): velocities lose their
components along the restrained directions at each DEM call, forces and
torques at every step.  CPU tests run the oracle; the GPU test compares the
session with it bit for bit."""
import math

import numpy as np
import pytest

from helpers import assert_bitwise, make_collision_scene
from parmec_gb300.model import Model


def falling_sphere():
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    p = m.sphere((0.0, 0.0, 1.0), 0.1, mat, 1)
    m.velocity(p, linear=(1.0, 2.0, 3.0), angular=(4.0, 5.0, 6.0))
    m.set_gravity(0.0, 0.0, -9.81)
    return m, p


def test_directions_orthonormalised():
    m, p = falling_sphere()
    m.restrain(p, linear=[1.0, 1.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 2.0], angular=[0.0, 0.0, 3.0])
    _, lin, ang = m.restraints[0]
    D = np.array(lin).reshape(3, 3)
    assert np.allclose(D @ D.T, np.eye(3), atol=1e-15)
    assert np.allclose(D[0], [math.sqrt(0.5), math.sqrt(0.5), 0.0])
    assert ang[:3] == [0.0, 0.0, 1.0] and ang[3:] == [0.0] * 6


def test_argument_errors():
    m, p = falling_sphere()
    with pytest.raises(ValueError):
        m.restrain(p, linear=[1.0, 0.0])
    with pytest.raises(ValueError):
        m.restrain(5, linear=[1.0, 0.0, 0.0])
    with pytest.raises(TypeError):
        m.restrain(p, linear=(1.0, 0.0, 0.0))
    m.restrain(p)                                   # nothing given: no record
    assert m.restraints == []


def test_linear_restraint_holds_height(oracle_lib):
    """Gravity along the restrained z axis: after the initial half step (taken
    before restrain_velocities, parmec.cpp:2397-2413) z and its velocity stay
    put; x and y move freely."""
    from oracle.pyoracle import OracleEngine
    m, p = falling_sphere()
    m.restrain(p, linear=[0.0, 0.0, 1.0])
    dt = 1e-4
    m.dem(100 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
    assert m.P.position[2, p] == 1.0 + (0.5 * dt) * 3.0 and m.P.linear[2, p] == 0.0
    assert abs(m.P.linear[0, p] - 1.0) < 1e-15 and abs(m.P.position[0, p] - 100.5 * dt) < 1e-12


def test_angular_restraint_removes_spin(oracle_lib):
    """The spatial angular velocity loses its restrained axes at the DEM call
    (4 and 5 rad/s before; what remains is the drift of the reproduced expmap
    typo over ten steps) and keeps the free one."""
    from oracle.pyoracle import OracleEngine
    m, p = falling_sphere()
    m.restrain(p, angular=[1.0, 0.0, 0.0, 0.0, 1.0, 0.0])
    dt = 1e-4
    m.dem(10 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
    assert abs(m.P.angular[3, p]) < 1e-7 and abs(m.P.angular[4, p]) < 1e-7
    assert abs(m.P.angular[5, p] - 6.0) < 1e-7


@pytest.mark.gpu
def test_gpu_restraints_bitwise(gpu_lib, oracle_lib):
    """Restrained particles in a colliding pack: the session equals the oracle."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine

    def make():
        m, dt = make_collision_scene(n_side=4)
        m.restrain(0, linear=[0.0, 0.0, 1.0])
        m.restrain(3, linear=[1.0, 1.0, 0.0, 0.0, 1.0, 1.0], angular=[0.0, 0.0, 1.0])
        m.restrain(3, angular=[1.0, 0.0, 0.0])
        m.restrain(7, angular=[1.0, 0.2, 0.0, 0.0, 1.0, 0.3, 0.1, 0.0, 1.0])
        return m, dt
    mg, dt = make()
    mo, _ = make()
    for k in range(2):                              # restrain_velocities runs at each DEM call
        mg.dem(25 * dt, dt, interval=1e9, engine=GpuEngine() if k == 0 else mg.last_engine)
        mo.dem(25 * dt, dt, interval=1e9, engine=OracleEngine() if k == 0 else mo.last_engine)
        assert_bitwise(mg, mo)


def test_eqm_command():
    """EQM (input.cpp:2336-2381): a sphere at its centre along a direction has
    its own mass; two equal spheres in series half of it; off-centre points
    lower the mass through the rotational term."""
    from parmec_gb300 import parmec as P
    P.RESET()
    mat = P.MATERIAL(1000.0, 1e9, 0.25)
    a = P.SPHERE((0.0, 0.0, 0.0), 0.1, mat, 1)
    b = P.SPHERE((1.0, 0.0, 0.0), 0.1, mat, 1)
    m = P.model().P.mass[a]
    assert abs(P.EQM(a, (0.0, 0.0, 0.0), direction=(1.0, 0.0, 0.0)) - m) <= 1e-12 * m
    assert abs(P.EQM(a, (0.0, 0.0, 0.0), b, (1.0, 0.0, 0.0), (1.0, 0.0, 0.0)) - 0.5 * m) <= 1e-12 * m
    assert P.EQM(a, (0.0, 0.1, 0.0), direction=(1.0, 0.0, 0.0)) < m
    with pytest.raises(ValueError):
        P.EQM(5, (0.0, 0.0, 0.0))
    P.RESET()

