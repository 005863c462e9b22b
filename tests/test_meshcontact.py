"""Mesh-mesh contact (Model.mesh_contact, an extension: the reference detects no
contact between meshes).

CPU: the swept-triangle geometry (parmec_gb300/csrc/pg_tritri.cuh) against
closed forms -- parallel faces, crossing edges, a vertex over a face,
intersecting triangles, triangles apart; a cube comes to rest on a fixed
cube (the contacts carry its weight); without the extension it falls
through, as in the reference.
GPU: the device's search, contact law and per-particle sums against the
oracle's brute-force restatement, bit for bit, on a pile of cubes and on the
spring-lattice deck with contact on.
"""
import ctypes

import numpy as np
import pytest

from helpers import assert_bitwise, bits


def contact(a, b, ra=1e-3, rb=1e-3):
    from oracle import pyoracle
    lib = pyoracle.load()
    A = np.ascontiguousarray(a, dtype=np.float64).reshape(9)
    B = np.ascontiguousarray(b, dtype=np.float64).reshape(9)
    p, n = np.zeros(3), np.zeros(3)
    D = ctypes.POINTER(ctypes.c_double)
    d = lib.or_tt_contact(A.ctypes.data_as(D), B.ctypes.data_as(D), ra, rb, p.ctypes.data_as(D), n.ctypes.data_as(D))
    return d, p, n


def test_parallel_faces(oracle_lib):
    a = [(0, 0, 0.0015), (1, 0, 0.0015), (0, 1, 0.0015)]
    b = [(0.1, 0.1, 0), (0.9, 0.1, 0), (0.1, 0.9, 0)]
    d, p, n = contact(a, b)
    assert abs(d - (2e-3 - 1.5e-3)) <= 1e-15
    assert np.allclose(n, [0, 0, 1]) and abs(p[2] - 0.75e-3) <= 1e-15


def test_crossing_edges(oracle_lib):
    """A's edge along x at height g above B's edge along y: distance g."""
    g = 1.2e-3
    a = [(-1, 0, g), (1, 0, g), (0, 0, 1)]            # lowest edge along x at z = g
    b = [(0, -1, 0), (0, 1, 0), (0, 0, -1)]           # highest edge along y at z = 0
    d, p, n = contact(a, b)
    assert abs(d - (2e-3 - g)) <= 1e-15
    assert np.allclose(n, [0, 0, 1]) and np.allclose(p, [0, 0, 0.5 * g])


def test_vertex_over_face(oracle_lib):
    g = 0.5e-3
    a = [(0.2, 0.2, g), (0.3, 0.2, 1), (0.2, 0.3, 1)]
    b = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
    d, p, n = contact(a, b)
    assert abs(d - (2e-3 - g)) <= 1e-15 and np.allclose(n, [0, 0, 1])


def test_intersecting_triangles(oracle_lib):
    """An edge of A through B's interior: depth ra + rb, B's normal towards A."""
    a = [(0.2, 0.2, -0.5), (0.2, 0.2, 0.5), (0.3, 0.25, 1.0)]
    b = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
    d, p, n = contact(a, b, 1e-3, 2e-3)
    assert d == 3e-3
    assert np.allclose(n, [0, 0, 1])                 # A's centroid lies above B
    assert np.allclose(p, [0.2, 0.2, 0.0])


def test_triangles_apart(oracle_lib):
    a = [(0, 0, 1), (1, 0, 1), (0, 1, 1)]
    b = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
    d, _, _ = contact(a, b)
    assert d < 0.0


def two_cubes(radius=1e-3, gap=0.0021):
    from parmec_gb300 import mesh
    from parmec_gb300.model import Model
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    a = 0.01
    lower = int(mesh.hex_grid(m, np.array([[0.0, 0.0, 0.0]]), a, mat, 1)[0])
    upper = int(mesh.hex_grid(m, np.array([[0.002, 0.001, a + gap]]), a, mat, 1)[0])
    m.prescribe_motion(lower, linear=lambda t: (0.0, 0.0, 0.0), angular=lambda t: (0.0, 0.0, 0.0), kind="vv")
    m.granular(0, 0, 1e5, 0.5, 0.3)
    m.set_gravity(0.0, 0.0, -9.81)
    m.mesh_contact(radius)
    return m, lower, upper


def test_cube_rests_on_cube(oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, lower, upper = two_cubes()
    eng = OracleEngine()
    dt = 1e-5
    m.dem(1500 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    weight = m.P.mass[upper] * 9.81
    pairs, active = eng.mesh_contact_stats()
    assert active >= 4 and pairs >= active
    assert abs(m.P.force[2, upper]) <= 0.05 * weight          # the contacts carry the weight
    assert abs(m.P.linear[2, upper]) <= 1e-3
    assert abs(m.P.position[2, upper] - (0.01 + 0.002 + 0.005)) <= 1e-6   # resting on the 2r shell


def test_without_the_extension_meshes_pass_through(oracle_lib):
    """The reference's behaviour: no contact between meshes."""
    from oracle.pyoracle import OracleEngine
    m, lower, upper = two_cubes(radius=0.0)
    dt = 1e-5
    m.dem(4500 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
    assert m.P.position[2, upper] < 0.01            # its centre is inside the lower cube


def cube_pile(radius=1e-3, seed=3):
    """A 3 x 3 layer of cubes on a fixed plate and a second, rotated layer
    dropped on it."""
    from parmec_gb300 import mesh
    from parmec_gb300.model import Model
    rng = np.random.default_rng(seed)
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    L = 0.05
    plate = m.mesh([-0.01, -0.01, -0.005, L, -0.01, -0.005, L, L, -0.005, -0.01, L, -0.005,
                    -0.01, -0.01, 0.0, L, -0.01, 0.0, L, L, 0.0, -0.01, L, 0.0],
                   [8, 0, 1, 2, 3, 4, 5, 6, 7, mat], mat, 2)
    m.prescribe_motion(plate, linear=lambda t: (0.0, 0.0, 0.0), angular=lambda t: (0.0, 0.0, 0.0), kind="vv")
    org = []
    for i in range(3):
        for j in range(3):
            org.append((0.014 * i, 0.014 * j, 0.0021))
    for i in range(2):
        for j in range(2):
            org.append((0.007 + 0.014 * i + rng.uniform(-1e-3, 1e-3), 0.007 + 0.014 * j, 0.0162))
    parts = mesh.hex_grid(m, np.array(org), 0.01, mat, 1)
    for p in parts[9:]:
        m.velocity(int(p), angular=tuple(float(x) for x in rng.normal(0.0, 2.0, size=3)))
    m.granular(0, 0, 1e5, 0.3, 0.4)
    m.set_gravity(0.0, 0.0, -9.81)
    m.mesh_contact(radius)
    return m


@pytest.mark.gpu
def test_gpu_cube_pile_bitwise(gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    mg, mo = cube_pile(), cube_pile()
    eg, eo = GpuEngine(), OracleEngine()
    dt = 1e-5
    seen = 0
    for _ in range(4):
        mg.dem(200 * dt, dt, interval=1e9, engine=eg)
        mo.dem(200 * dt, dt, interval=1e9, engine=eo)
        assert_bitwise(mg, mo)
        assert eg.mesh_contact_stats() == eo.mesh_contact_stats()
        seen = max(seen, eo.mesh_contact_stats()[1])
    assert seen >= 20                                  # the layers touch each other and the plate
    assert np.array_equal(bits(mg.Tr.tri[:, :mg.trinum]), bits(mo.Tr.tri[:, :mo.trinum]))


@pytest.mark.gpu
def test_gpu_spring_lattice_with_contact_bitwise(gpu_lib, oracle_lib):
    """The spring-lattice deck (cubes on springs over a base plate driven by
    PRESCRIBE) with mesh contact at half the gap: cubes touch the plate and
    their neighbours; the big plate triangles go through the all-against-all
    range of the search."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import spring_lattice
    (mg, dt), (mo, _) = spring_lattice(8, contact_radius=1e-3), spring_lattice(8, contact_radius=1e-3)
    eg, eo = GpuEngine(), OracleEngine()
    mg.dem(150 * dt - 0.5 * dt, dt, interval=1e9, engine=eg)
    mo.dem(150 * dt - 0.5 * dt, dt, interval=1e9, engine=eo)
    assert_bitwise(mg, mo)
    assert eg.mesh_contact_stats() == eo.mesh_contact_stats()
    assert eo.mesh_contact_stats()[1] > 0


@pytest.mark.gpu
def test_gpu_lattice_plate_sums_in_chunks_bitwise(gpu_lib, oracle_lib):
    """A 24x24 lattice with contact on: tens of thousands of active pairs,
    the base plate's share of them summed in several chunks of 1,024 entries
    (one warp per chunk, the chunk sums in order), bit for bit against the
    oracle's chunked sums."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import spring_lattice
    (mg, dt), (mo, _) = spring_lattice(24, contact_radius=1e-3), spring_lattice(24, contact_radius=1e-3)
    eg, eo = GpuEngine(), OracleEngine()
    for k in range(2):
        d = 20 * dt - (0.5 * dt if k == 0 else 0.0)
        mg.dem(d, dt, interval=1e9, engine=eg)
        mo.dem(d, dt, interval=1e9, engine=eo)
        assert_bitwise(mg, mo)
        assert eg.mesh_contact_stats() == eo.mesh_contact_stats()
    assert eo.mesh_contact_stats()[1] > 8 * 1024
