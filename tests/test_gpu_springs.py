"""GPU parity of the SPRING path (springs_task, forces.ispc:641-1412) and of
prescribed motion, damping and the reference's golden decks on the GPU."""
import math
import random

import numpy as np
import pytest

from helpers import assert_bitwise, bits

pytestmark = pytest.mark.gpu


def spring_state_equal(ma, mb):
    n = ma.sprnum
    for name in ("stroke", "sprfrc", "sprsdsp", "sprdir", "sprpnt", "yield_"):
        a = getattr(ma.S, name)[..., :n]
        b = getattr(mb.S, name)[..., :n]
        assert np.array_equal(bits(a), bits(b)), name
    assert np.array_equal(ma.S.sprflg[:n], mb.S.sprflg[:n])


def lattice(n=5, seed=3):
    """n x n analytical bodies on springs of every direction mode, tied to a
    base body driven by a prescribed acceleration."""
    from parmec_gb300.model import Model
    rng = random.Random(seed)
    m = Model()
    m.material(1000.0, 1e9, 0.25)
    ids = {}
    h = 0.01
    for i in range(n):
        for j in range(n):
            ids[i, j] = m.analytical([1e-6, 2e-6, 1.5e-6, 1e-7, 0.0, 0.0], 0.01,
                                     position=(i * h, j * h, 0.0))
    base = m.analytical([1.0, 1.0, 1.0, 0.0, 0.0, 0.0], 10.0, position=(0.5 * n * h, 0.5 * n * h, -h))
    off = m.tseries([0.0, 0.0, 0.01, 1e-4, 1.0, 1e-4])

    def curve(k):
        xs = sorted(rng.uniform(-0.01, 0.01) for _ in range(8))
        ys, f = [], -0.5 * k * 0.01
        for a in range(8):
            ys.append(f)
            f += rng.uniform(0.2, 1.0) * k * 0.0025
        return [v for p in zip(xs, ys) for v in p]

    for (i, j), p in ids.items():
        for (di, dj) in ((1, 0), (0, 1)):
            q = ids.get((i + di, j + dj))
            if q is None:
                continue
            kind = (i + j) % 4
            pa = (i * h + 0.3 * h * di, j * h + 0.3 * h * dj, 0.0)
            pb = ((i + di) * h - 0.3 * h * di, (j + dj) * h - 0.3 * h * dj, 0.0)
            if kind == 0:
                m.spring(p, pa, q, pb, curve(1e4), dashpot=0.05)
            elif kind == 1:
                m.spring(p, pa, q, pb, curve(3e4), dashpot=[-1.0, -10.0, 1.0, 10.0],
                         direction=(float(di), float(dj), 0.0), planar="OFF", offset=off)
            elif kind == 2:
                m.spring(p, pa, q, pb, curve(2e4), dashpot=0.1, direction=(0.0, 0.0, 1.0), planar="ON",
                         friction=0.3, kskn=0.5)
            else:
                m.spring(p, pa, q, pb, curve(5e4), unload=[-0.02, -50.0, 0.02, 50.0], ylim=(-5.0, 5.0),
                         friction=0.2)
        m.spring(base, (i * h, j * h, -h), p, (i * h, j * h, 0.0), curve(1e4), dashpot=0.2)
    m.prescribe_motion(base, linear=lambda t: (0.5 * 9.81 * math.sin(2 * math.pi * 5.0 * t), 0.0, 0.0),
                       kind="av")
    m.set_gravity(0.0, 0.0, -9.81)
    return m


def test_spring_lattice_bitwise(gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    mg, mo = lattice(), lattice()
    step = 2e-5
    mg.dem(300 * step - 0.5 * step, step, interval=1e9, engine=GpuEngine())
    mo.dem(300 * step - 0.5 * step, step, interval=1e9, engine=OracleEngine())
    assert_bitwise(mg, mo)
    spring_state_equal(mg, mo)
    assert np.any(mo.S.sprflg[:mo.sprnum] & 1)     # some general springs yielded


def test_spring_curves_on_gpu(gpu_lib, oracle_lib):
    """The reference's spring-curve deck through the GPU engine: same
    histories as the oracle, bit for bit, and within 0.1*h of the input."""
    from scipy.interpolate import interp1d
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.model import Model
    h = 0.02
    for seed in range(4):
        out = []
        for make in (GpuEngine, OracleEngine):
            rnd = random.Random(seed)
            m = Model()
            m.material(1, 1, 0.25)
            parnum = m.analytical()
            n = rnd.randint(2, 20)
            t = [0.]
            for i in range(1, n):
                t.append(t[i - 1] + rnd.uniform(1., 10.))
            s = []
            for i in range(n):
                t[i] = -1.0 + 2.0 * t[i] / t[-1]
                s.append(rnd.uniform(-1., 1.))
            sprnum = m.spring(parnum, (0, 0, 0), -1, (0, 0, 0), list(sum(zip(t, s), ())), direction=(-1, 0, 0))
            m.prescribe_motion(parnum, linear=lambda t: (-1, 0, 0))
            eng = make()
            m.dem(1.0, h, engine=eng)
            x = m.history('STROKE', sprnum)
            f = m.history('SF', sprnum)
            m.prescribe_motion(parnum, linear=lambda t: (1, 0, 0))
            m.dem(2.0 + h, h, engine=eng)
            out.append((t, s, x, f))
        (t, s, xg, fg), (_, _, xo, fo) = out
        assert np.array_equal(np.array(xg), np.array(xo)) and np.array_equal(np.array(fg), np.array(fo))
        g0, g1 = interp1d(t, s), interp1d(xg, fg)
        for w in np.arange(-1., xg[-1] - h, h):
            assert abs(g0(w) - g1(w)) <= 0.1 * h


def test_damping_projectile_on_gpu(gpu_lib):
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.model import Model
    m = Model()
    step = 1.976 / 1024.0
    num = m.analytical([1, 1, 1, 0, 0, 0], 0.45359237, position=(0, 0, 0))
    m.velocity(num, (2.54, 0, 12.7), (0, 0, 0))
    m.set_damping(lambda t: (1, 1, 1), lambda t: (0, 0, 0))
    m.set_gravity(0., 0., -9.81456)
    X = m.history('PX', num)
    m.dem(1.976, step, (64 * step, step), engine=GpuEngine())
    assert abs(X[-1] / 0.0254 - 86.138) / 86.138 < 0.005


def test_prescribed_velocity_and_acceleration_bitwise(gpu_lib, oracle_lib):
    """PRESCRIBE of every kind (vv, va, av, aa) with callables and TSERIES."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from helpers import make_collision_scene
    out = []
    for eng in (GpuEngine(), OracleEngine()):
        m, dt = make_collision_scene(n_side=4, seed=4)
        ts = m.tseries([0.0, 0.0, 1e-3, 0.5, 1.0, 0.5])
        m.prescribe_motion(0, linear=lambda t: (0.1, 0.0, math.sin(100 * t)), kind="vv")
        m.prescribe_motion(5, angular=lambda t: (0.0, 3.0, 0.0), kind="va")
        m.prescribe_motion(9, linear=(ts, ts, ts), angular=(ts, ts, ts), kind="aa")
        m.prescribe_motion(13, linear=lambda t: (0.0, -2.0, 0.0), angular=(ts, ts, ts), kind="av")
        m.dem(100 * dt, dt, interval=1e9, engine=eng)
        out.append(m)
    assert_bitwise(out[0], out[1])


def test_mesh_spring_lattice_bitwise(gpu_lib, oracle_lib):
    """The spring-lattice shaking table (MESH cubes, 8-point spring curves,
    lookup dashpots, prescribed base): particles, mesh nodes, triangles and
    spring state equal the oracle's bit for bit."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import spring_lattice
    (mg, dt), (mo, _) = spring_lattice(17), spring_lattice(17)     # 289 base springs: a long run of two chunks
    mg.dem(250 * dt - 0.5 * dt, dt, interval=1e9, engine=GpuEngine())
    mo.dem(250 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
    assert_bitwise(mg, mo)
    spring_state_equal(mg, mo)
    assert np.array_equal(bits(mg.N.nodes[:, :mg.nodnum]), bits(mo.N.nodes[:, :mo.nodnum]))
    assert np.array_equal(bits(mg.Tr.tri[:, :mg.trinum]), bits(mo.Tr.tri[:, :mo.trinum]))
    assert np.max(np.abs(mg.P.linear[0, :mg.parnum])) > 0.0      # the table moved the lattice


def test_spheres_on_a_mesh_particle_bitwise(gpu_lib, oracle_lib):
    """Spheres fall on a MESH plate that rests on springs: sphere-triangle
    contacts whose partner is a particle (the reaction goes to the plate
    through the slave lists)."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.model import Model

    def make():
        rng = np.random.default_rng(5)
        m = Model()
        mat = m.material(2000.0, 1e9, 0.25)
        a = 0.1
        nodes = [0.0, 0.0, 0.0, a, 0.0, 0.0, a, a, 0.0, 0.0, a, 0.0,
                 0.0, 0.0, 0.01, a, 0.0, 0.01, a, a, 0.01, 0.0, a, 0.01]
        plate = m.mesh(nodes, [8, 0, 1, 2, 3, 4, 5, 6, 7, 0], mat, 2)
        for k in range(4):
            for x, y in ((0.02, 0.02), (0.08, 0.02), (0.02, 0.08), (0.08, 0.08)):
                m.spring(plate, (x, y, 0.0), -1, (x, y, -0.01), [-1.0, -2e4, 1.0, 2e4], dashpot=0.3)
        for s in range(36):
            c = (0.012 + 0.015 * (s % 6), 0.012 + 0.015 * (s // 6), 0.0158 + 0.0005 * rng.random())
            m.sphere(c, 0.006, mat, 1)
        m.granular(0, 0, 1e4, 0.3, 0.4)
        m.set_gravity(0.0, 0.0, -9.81)
        return m
    step = 2e-5
    mg, mo = make(), make()
    mg.dem(400 * step - 0.5 * step, step, interval=1e9, engine=GpuEngine())
    eo = OracleEngine()
    mo.dem(400 * step - 0.5 * step, step, interval=1e9, engine=eo)
    assert_bitwise(mg, mo)
    assert len(eo.contacts()["mpart"]) >= 10                   # spheres rest on the plate
    assert np.array_equal(bits(mg.Tr.tri[:, :mg.trinum]), bits(mo.Tr.tri[:, :mo.trinum]))
