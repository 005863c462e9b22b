"""The oracle against the reference's own self-checking decks and analytic
known answers (CPU only).

Pins:
  * tests/damping.py:4-37 of the reference -- projectile with global linear
    damping: final x within 0.5 % of 86.138 in;
  * tests/spring_curve_tests.py:14-63 -- twelve random piecewise-linear
    spring curves driven through their stroke range by a prescribed velocity:
    recorded (stroke, force) within 0.1*h of the input curve;
  * analytic cases written from the mechanics (restitution of a linear
    spring-dashpot contact, static overlap of a sphere on a plane, closest
    point regions of a triangle, rotation matrices of the exponential map).
The contact detection and granular force paths have no golden vector in the
reference; the analytic cases are their only pins.
"""
import math
import random

import numpy as np
import pytest

from parmec_gb300.model import Model


def test_damping_projectile(oracle_lib):
    from oracle.pyoracle import OracleEngine
    m = Model()
    v0, w0 = (2.54, 0, 12.7), (0, 0, 0)
    gravity, stop = 9.81456, 1.976
    step = stop / 1024.0
    num = m.analytical([1, 1, 1, 0, 0, 0], 0.45359237, position=(0, 0, 0))
    m.velocity(num, v0, w0)
    m.set_damping(lambda t: (1, 1, 1), lambda t: (0, 0, 0))
    m.set_gravity(0., 0., -gravity)
    X = m.history('PX', num)
    m.dem(stop, step, (64 * step, step), engine=OracleEngine())
    value = X[-1] / 0.0254
    assert abs(value - 86.138) / 86.138 < 0.005


def spring_curve_case(seed, h=0.02):
    """One reference spring-curve case: returns (input t, s) and recorded (x, f)."""
    from oracle.pyoracle import OracleEngine
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
    ts = list(sum(zip(t, s), ()))
    sprnum = m.spring(parnum, (0, 0, 0), -1, (0, 0, 0), ts, direction=(-1, 0, 0))
    m.prescribe_motion(parnum, linear=lambda t: (-1, 0, 0))
    eng = OracleEngine()
    m.dem(1.0, h, engine=eng)
    x = m.history('STROKE', sprnum)
    f = m.history('SF', sprnum)
    m.prescribe_motion(parnum, linear=lambda t: (1, 0, 0))
    m.dem(2.0 + h, h, engine=eng)
    return t, s, x, f


@pytest.mark.parametrize("seed", range(12))
def test_spring_curves(oracle_lib, seed):
    scipy = pytest.importorskip("scipy.interpolate")
    h = 0.02
    t, s, x, f = spring_curve_case(seed, h)
    g0 = scipy.interp1d(t, s)
    g1 = scipy.interp1d(x, f)
    for w in np.arange(-1., x[-1] - h, h):
        assert abs(g0(w) - g1(w)) <= 0.1 * h


def expmap(o, typo=False):
    import ctypes
    from oracle import pyoracle
    L = (ctypes.c_double * 9)()
    pyoracle.load().or_expmap(o[0], o[1], o[2], 1 if typo else 0, L)
    return np.array(L[:]).reshape(3, 3).T      # column-major


@pytest.mark.parametrize("o", [(0.01, 0.0, 0.0), (0.003, -0.002, 0.001), (0.5, 0.2, -0.1), (0.0, 0.0, 0.0)])
def test_expmap_is_rotation(oracle_lib, o):
    R = expmap(o)
    assert np.allclose(R.T @ R, np.eye(3), atol=1e-13)
    assert abs(np.linalg.det(R) - 1.0) < 1e-13
    v = np.array(o)
    th = np.linalg.norm(v)
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    exact = np.eye(3) + (np.sin(th) / th if th else 1.0) * K + ((1 - np.cos(th)) / th ** 2 if th else 0.5) * K @ K
    assert np.allclose(R, exact, atol=1e-13)


def test_expmap_typo_switch(oracle_lib):
    o = (0.01, 0.02, 0.03)
    good, bad = expmap(o), expmap(o, typo=True)
    assert not np.allclose(good, bad, atol=1e-9)
    assert np.array_equal(expmap((0.01, 0, 0)), expmap((0.01, 0, 0), typo=True))


def tri_sphere(a, b, c, p, r, edge_typo=False):
    import ctypes
    from oracle import pyoracle
    D3 = ctypes.c_double * 3
    pt, nr = D3(), D3()
    d = pyoracle.load().or_triangle_sphere(D3(*a), D3(*b), D3(*c), D3(*p), r, pt, nr, 1 if edge_typo else 0)
    return d, np.array(pt[:]), np.array(nr[:])


@pytest.mark.parametrize("p,q", [
    ((0.2, 0.2, 1.0), (0.2, 0.2, 0.0)),      # face interior
    ((-1.0, -1.0, 1.0), (0.0, 0.0, 0.0)),    # vertex a
    ((2.0, -0.5, 1.0), (1.0, 0.0, 0.0)),     # vertex b
    ((-0.5, 2.0, 1.0), (0.0, 1.0, 0.0)),     # vertex c
    ((0.5, -1.0, 1.0), (0.5, 0.0, 0.0)),     # edge ab
    ((-1.0, 0.5, 1.0), (0.0, 0.5, 0.0)),     # edge ac
    ((1.0, 1.0, 1.0), (0.5, 0.5, 0.0)),      # edge bc
])
def test_closest_point_regions(oracle_lib, p, q):
    d, pt, nr = tri_sphere((0, 0, 0), (1, 0, 0), (0, 1, 0), p, 2.0, edge_typo=False)
    assert np.allclose(pt, q, atol=1e-15)
    dist = np.linalg.norm(np.array(p) - np.array(q))
    assert abs(d - (2.0 - dist)) < 1e-14
    assert np.allclose(nr, (np.array(p) - np.array(q)) / dist, atol=1e-15)


def test_closest_point_reference_edge_defect(oracle_lib):
    """With the reference's region formula (condet.ispc:373) a centre beyond
    vertex b, outside edge ab, is matched to vertex a; every other region is
    unaffected by the switch."""
    d, pt, nr = tri_sphere((0, 0, 0), (1, 0, 0), (0, 1, 0), (2.0, -0.5, 1.0), 2.0, edge_typo=True)
    assert np.allclose(pt, (0.0, 0.0, 0.0))
    for p in [(0.2, 0.2, 1.0), (-1.0, -1.0, 1.0), (-0.5, 2.0, 1.0), (0.5, -1.0, 1.0), (-1.0, 0.5, 1.0), (1.0, 1.0, 1.0)]:
        a = tri_sphere((0, 0, 0), (1, 0, 0), (0, 1, 0), p, 2.0, edge_typo=True)
        b = tri_sphere((0, 0, 0), (1, 0, 0), (0, 1, 0), p, 2.0, edge_typo=False)
        assert np.array_equal(a[1], b[1])


def head_on(xi, v=0.1, r=0.01, rho=2500.0, kn=1e6):
    """Two equal spheres, head-on, no gravity: returns post-collision relative speed ratio."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.scenes import critical_step
    m = Model()
    mat = m.material(rho, 1e9, 0.25)
    a = m.sphere((0.0, 0.0, 0.0), r, mat, 1)
    b = m.sphere((2 * r + 1e-4, 0.0, 0.0), r, mat, 1)
    m.velocity(a, (v, 0.0, 0.0))
    m.velocity(b, (-v, 0.0, 0.0))
    m.granular(0, 0, kn, xi, 0.0)
    mass = (4 / 3) * math.pi * r ** 3 * rho
    dt = 0.02 * critical_step(kn, mass, xi)
    t_contact = math.pi / math.sqrt(kn / (0.5 * mass) * (1 - xi * xi))
    m.dem(3 * t_contact + 1e-4 / v, dt, interval=1e9, engine=OracleEngine())
    return (m.P.linear[0, b] - m.P.linear[0, a]) / (2 * v)


@pytest.mark.parametrize("xi", [0.05, 0.2, 0.4])
def test_restitution_linear_spring_dashpot(oracle_lib, xi):
    """e = exp(-xi*pi/sqrt(1-xi^2)) for the linear spring-dashpot normal law
    (fn = kn*depth + 2*xi*sqrt(kn*m)*vn with m the reduced mass)."""
    e = head_on(xi)
    exact = math.exp(-xi * math.pi / math.sqrt(1 - xi * xi))
    assert abs(e - exact) < 0.01


def test_static_overlap_on_plane(oracle_lib):
    """A sphere settles on a triangle with overlap m*g/kn."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.scenes import critical_step
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    r, kn = 0.05, 1e5
    s = m.sphere((0.0, 0.0, r), r, mat, 1)
    m.obstacle([(-1.0, -1.0, 0.0, 1.0, -1.0, 0.0, 0.0, 1.0, 0.0)], 2)
    m.granular(0, 0, kn, 1.0, 0.0)
    m.set_gravity(0.0, 0.0, -10.0)
    mass = (4 / 3) * math.pi * r ** 3 * 1000.0
    dt = 0.1 * critical_step(kn, mass, 1.0)
    m.dem(0.5, dt, interval=1e9, engine=OracleEngine())
    overlap = r - m.P.position[2, s]
    assert abs(overlap - mass * 10.0 / kn) < 1e-3 * mass * 10.0 / kn


def test_oracle_threads_bitwise(oracle_lib):
    """The OpenMP oracle (CPU baseline) equals the single-thread oracle bit for bit."""
    from oracle.pyoracle import OracleEngine
    from helpers import assert_bitwise, make_collision_scene
    m1, dt = make_collision_scene(n_side=5)
    m8, _ = make_collision_scene(n_side=5)
    m1.dem(80 * dt, dt, interval=1e9, engine=OracleEngine(threads=1))
    m8.dem(80 * dt, dt, interval=1e9, engine=OracleEngine(threads=8))
    assert_bitwise(m1, m8)


def test_contact_set_exact(oracle_lib):
    """After one step the oracle's new contacts are exactly the overlapping pairs."""
    from oracle.pyoracle import OracleEngine
    from helpers import make_collision_scene
    m, dt = make_collision_scene(n_side=6, spacing=0.03)
    c = m.E.center[0:3, :m.ellnum].T.copy()
    r = m.E.radii[0, :m.ellnum].copy()
    eng = OracleEngine()
    m.dem(0.5 * dt, dt, interval=1e9, engine=eng)
    # the step moved the spheres: recompute the expected set from the positions condet saw
    # (the centres after the initial half step), which the oracle exports as contact points
    got = eng.contacts()
    pairs = set()
    for k in range(len(got["mpart"])):
        if got["code"][k] >= 0:
            pairs.add((int(got["mpart"][k]), int(got["code"][k])))
    d = np.linalg.norm(c[:, None, :] - c[None, :, :], axis=-1)
    close = {(i, j) for i in range(len(r)) for j in range(i + 1, len(r)) if d[i, j] < r[i] + r[j] - 1e-6}
    far = {(i, j) for i in range(len(r)) for j in range(i + 1, len(r)) if d[i, j] > r[i] + r[j] + 1e-6}
    assert close <= pairs
    assert not (pairs & far)


def test_history_of_a_list_is_the_mean(oracle_lib):
    """HISTORY over a particle list reports the mean over the list
    (output.cpp:5514-5516); a single index reports the value itself."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.model import Model
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    a = m.sphere((0.0, 0.0, 1.0), 0.1, mat, 1)
    b = m.sphere((5.0, 0.0, 3.0), 0.1, mat, 1)
    m.set_gravity(0.0, 0.0, 0.0)
    both = m.history("PZ", [a, b])
    one = m.history("PZ", b)
    m.dem(0.01, 0.001, interval=0.005, engine=OracleEngine())
    assert len(both) == len(one) > 0
    assert both[-1] == (1.0 + 3.0) / 2.0
    assert one[-1] == 3.0
