"""TORSION_SPRING (input.cpp:1791-2080, trqspr_task forces.ispc:1415-2057).

The reference's own decks (tests/torsion_spring_one.py, torsion_spring_two.py)
spin a unit cube (1000 kg, J = m/6 about its centre) on a torsion spring of
slope -1e4 N m/rad about roll, pitch or yaw, and plot the angular velocity.
Restated here with the closed forms they illustrate: one cube on a spring to
the ground spins as cos(w t), w = sqrt(k/J); two cubes share the momentum,
w1 = (1 + cos(w2 t))/2 with w2 = sqrt(2k/J).  CPU tests run the oracle; the
GPU tests compare the session and the drop-in exports with it bit for bit.
"""
import math

import numpy as np
import pytest

from helpers import assert_bitwise
from parmec_gb300.model import Model

K = [-1.0, 1e4, 1.0, -1e4]


def cube(m, mat, z0=0.0):
    nodes = [0, 0, z0, 1, 0, z0, 1, 1, z0, 0, 1, z0, 0, 0, z0 + 1, 1, 0, z0 + 1, 1, 1, z0 + 1, 0, 1, z0 + 1]
    return m.mesh([float(x) for x in nodes], [8, 0, 1, 2, 3, 4, 5, 6, 7, mat], mat,
                  [1, 4, 0, 1, 2, 3, 2, 4, 4, 5, 6, 7, 3])


# (zdir, xdir, axis name, spin axis) of the reference's one-particle cases 0-8
CASES = [((1, 0, 0), (0, 0, 1), "kroll", 2), ((0, 1, 0), (1, 0, 0), "kroll", 0), ((1, 0, 0), (0, 1, 0), "kroll", 1),
         ((0, 0, 1), (0, 1, 0), "kyaw", 2), ((1, 0, 0), (0, 0, 1), "kyaw", 0), ((0, 1, 0), (0, 0, 1), "kyaw", 1),
         ((1, 0, 0), (0, 1, 0), "kpitch", 2), ((0, 0, 1), (0, 1, 0), "kpitch", 0), ((0, 0, 1), (1, 0, 0), "kpitch", 1)]


def one(case, two=False, **extra):
    m = Model()
    mat = m.material(1e3, 1e9, 0.25)
    p = cube(m, mat)
    q = cube(m, mat, 1.0) if two else -1
    if case < 9:
        z, x, key, ax = CASES[case]
        m.torsion_spring(p, q, tuple(float(v) for v in z), tuple(float(v) for v in x), **{key: K}, **extra)
        w = [0.0, 0.0, 0.0]
        w[ax] = 1.0
    else:
        damp = ({"droll": [-1.0, 7e2, 1.0, -7e2], "dyaw": [-1.0, 5e2, 1.0, -5e2], "dpitch": [-1.0, 3e2, 1.0, -3e2]}
                if case == 9 else {"droll": 0.25, "dyaw": 0.5, "dpitch": 1.0})
        m.torsion_spring(p, q, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), kroll=K, kyaw=K, kpitch=K, **damp, **extra)
        w, ax = [1.0, 1.0, 1.0], None
    m.velocity(p, angular=tuple(w))
    return m, p, q, ax


@pytest.mark.parametrize("case", range(9))
def test_one_particle_oscillates(case, oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, p, _, ax = one(case)
    J = m.P.inertia[0, p]
    w = math.sqrt(1e4 / J)
    h = 1e-3
    hist = m.history("O" + "XYZ"[ax], p)
    t = m.history("TIME")
    m.dem(1.0, h, interval=(1e9, 0.05), engine=OracleEngine())
    err = max(abs(o - math.cos(w * tt)) for o, tt in zip(hist, t))
    assert len(hist) > 15 and err < 2e-2


def test_two_particles_share_momentum(oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, p, q, ax = one(3, two=True)
    J = m.P.inertia[0, p]
    w2 = math.sqrt(2e4 / J)
    a = m.history("OZ", p)
    b = m.history("OZ", q)
    t = m.history("TIME")
    m.dem(1.0, 1e-3, interval=(1e9, 0.05), engine=OracleEngine())
    for oa, ob, tt in zip(a, b, t):
        assert abs(oa - 0.5 * (1 + math.cos(w2 * tt))) < 2e-2
        assert abs(oa + ob - 1.0) < 1e-9                  # the pair's momentum is conserved


def test_damped_decays(oracle_lib):
    """Dampers by lookup table and by critical ratio remove energy."""
    from oracle.pyoracle import OracleEngine
    for case in (9, 10):
        m, p, _, _ = one(case)
        m.dem(2.0, 1e-3, interval=1e9, engine=OracleEngine())
        assert np.linalg.norm(m.P.angular[3:6, p]) < 0.5


def test_command_errors():
    m = Model()
    mat = m.material(1e3, 1e9, 0.25)
    p = cube(m, mat)
    with pytest.raises(ValueError):
        m.torsion_spring(p, -1, (0.0, 0.0, 1.0), (0.0, 1.0, 1.0))         # not orthogonal
    with pytest.raises(ValueError):
        m.torsion_spring(p, -1, (0.0, 0.0, 0.0), (1.0, 0.0, 0.0))
    with pytest.raises(ValueError):
        m.torsion_spring(p, -1, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), kroll=[1.0, 0.0, 0.0, 1.0])
    with pytest.raises(ValueError):
        m.torsion_spring(p, -1, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), cone=("roll", "pitch"))
    with pytest.raises(ValueError):
        m.torsion_spring(p, -1, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), kroll=K, cone=("roll", "roll"))
    with pytest.raises(ValueError):
        m.torsion_spring(p, -1, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), droll=-0.5)
    assert m.torsion_spring(p, -1, (0.0, 0.0, 2.0), (3.0, 0.0, 0.0), kroll=K) == 0
    assert np.allclose(m.Q.zdir0[:, 0], [0.0, 0.0, 1.0]) and np.allclose(m.Q.xdir0[:, 0], [1.0, 0.0, 0.0])


GPU_CASES = [(c, False, {}) for c in range(11)] + [(c, True, {}) for c in (0, 4, 8, 10)] + \
    [(9, False, {"cone": ("roll", "pitch")}), (9, False, {"cone": ("roll", "yaw")}),
     (10, False, {"cone": ("pitch", "yaw")}), (10, True, {"cone": ("roll", "pitch", "yaw")})]


@pytest.mark.gpu
@pytest.mark.parametrize("case,two,extra", GPU_CASES)
def test_gpu_torsion_bitwise(case, two, extra, gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    mg, *_ = one(case, two, **extra)
    mo, *_ = one(case, two, **extra)
    mg.dem(0.3, 1e-3, interval=1e9, engine=GpuEngine())
    mo.dem(0.3, 1e-3, interval=1e9, engine=OracleEngine())
    assert_bitwise(mg, mo)
    for name in ("rpy", "rpytot", "rpyspr", "zdir1", "xdir1"):
        a, b = getattr(mg.Q, name)[:, :mg.trqsprnum], getattr(mo.Q, name)[:, :mo.trqsprnum]
        assert np.array_equal(a.view(np.int64), b.view(np.int64)), name


@pytest.mark.gpu
def test_gpu_torsion_adaptive_bitwise(gpu_lib, oracle_lib):
    """Adaptive steps with the torsion springs' rotational stiffness terms
    (a translational spring between the cubes gives the translational one)."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    def make():
        m, p, q, _ = one(10, True)
        m.spring(p, (0.5, 0.5, 0.5), q, (0.5, 0.5, 1.5), [-1.0, -1e5, 1.0, 1e5])
        m.velocity(p, linear=(0.0, 0.0, -0.1))
        return m
    mg, mo = make(), make()
    mg.dem(0.2, 1e-3, interval=1e9, adaptive=0.5, engine=GpuEngine())
    mo.dem(0.2, 1e-3, interval=1e9, adaptive=0.5, engine=OracleEngine())
    assert mg.curstep == mo.curstep and mg.curstep != 1e-3
    assert_bitwise(mg, mo)


@pytest.mark.gpu
def test_dropin_torsion_bitwise(gpu_lib, oracle_lib):
    """forces() with torsion springs through the drop-in exports."""
    from oracle import dem_loop as ispc_loop
    from oracle.pyoracle import OracleEngine
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    for case, two, extra in ((10, True, {}), (9, False, {"cone": ("roll", "pitch", "yaw")})):
        mc, *_ = one(case, two, **extra)
        mo, *_ = one(case, two, **extra)
        host = ispc_loop.Host(lib, mc)
        eo = OracleEngine()
        for _ in range(2):
            mo.dem(0.05, 1e-3, interval=1e9, engine=eo)
            ispc_loop.dem(lib, host, 0.05, 1e-3)
            assert_bitwise(mc, mo)
            assert np.array_equal(mc.Q.rpy[:, :mc.trqsprnum].view(np.int64), mo.Q.rpy[:, :mo.trqsprnum].view(np.int64))
        host.close()
