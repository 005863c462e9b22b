"""MESH (input.cpp:840-1156, mesh.cpp:255-521): face extraction, mass
properties and argument errors (CPU only)."""
import numpy as np
import pytest

from parmec_gb300 import mesh
from parmec_gb300.model import Model


def cube_model(a=0.01, origin=(0.1, 0.2, 0.3), rho=2500.0):
    m = Model()
    mat = m.material(rho, 1e9, 0.25)
    nodes, ele = mesh.hexahedron(*origin, a)
    i = m.mesh(nodes, ele, mat, 3)
    return m, i


def test_hexahedron_mass_properties():
    """A cube: mass rho a^3, centre at its middle, inertia rho a^5 / 6 on the diagonal."""
    a, rho = 0.01, 2500.0
    m, i = cube_model(a, rho=rho)
    mass = rho * a ** 3
    assert abs(m.P.mass[i] - mass) <= 1e-12 * mass
    assert np.allclose(m.P.position[0:3, i], [0.105, 0.205, 0.305], rtol=0, atol=1e-15)
    J = m.P.inertia[:, i].reshape(3, 3)
    assert np.allclose(np.diag(J), mass * a * a / 6.0, rtol=1e-10, atol=0)
    assert np.max(np.abs(J - np.diag(np.diag(J)))) < 1e-12 * J[0, 0]
    assert np.allclose(m.P.inverse[:, i].reshape(3, 3) @ J, np.eye(3), atol=1e-9)
    assert m.P.invm[i] == 1.0 / m.P.mass[i]


def test_hexahedron_surface():
    """Six quads become twelve outward triangles owned by the particle."""
    m, i = cube_model()
    assert (m.nodnum, m.facnum, m.trinum) == (8, 12, 12)
    c = m.P.position[0:3, i]
    for t in range(m.trinum):
        A, B, C = m.Tr.tri[0:3, t], m.Tr.tri[3:6, t], m.Tr.tri[6:9, t]
        assert np.dot(np.cross(B - A, C - A), (A + B + C) / 3 - c) > 0
        assert m.Tr.triobs[t] == i and m.Tr.tricol[t] == 3
        for v in range(3):
            assert np.array_equal(m.N.nodes[0:3, m.F.facnod[v, t]], m.Tr.tri[3 * v:3 * v + 3, t])
    assert np.all(m.N.nodpart[:8] == i)


def test_two_hexahedra_share_an_inner_face():
    """Two elements of one mesh: the shared face is inner, 10 boundary quads remain,
    the mass doubles and the centre lies between them."""
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    a = 0.02
    n1, e1 = mesh.hexahedron(0.0, 0.0, 0.0, a)
    n2, _ = mesh.hexahedron(a, 0.0, 0.0, a)
    nodes = n1 + n2[3:6] + n2[6:9] + n2[15:18] + n2[18:21]     # the four new nodes (x = 2a)
    ele = e1[:-1] + [0] + [8, 1, 8, 9, 2, 5, 10, 11, 6, 0]
    i = m.mesh(nodes, ele, mat, [7, 4, 0, 1, 2, 3, 9])
    assert m.trinum == 20
    assert abs(m.P.mass[i] - 2 * 1000.0 * a ** 3) < 1e-15
    assert np.allclose(m.P.position[0:3, i], [a, 0.5 * a, 0.5 * a], atol=1e-15)
    cols = set(int(c) for c in m.Tr.tricol[:m.trinum])
    assert cols == {7, 9}                      # the coloured bottom quad, the rest global


def test_hex_grid_equals_separate_mesh_commands():
    origins = np.array([[0.1, 0.2, 0.3], [0.5, -0.2, 0.0], [1.0, 1.0, 1.0]])
    m2 = Model()
    mat = m2.material(2500.0, 1e9, 0.25)
    for o in origins:
        nodes, ele = mesh.hexahedron(*o, 0.01)
        m2.mesh(nodes, ele, mat, 3)
    m3 = Model()
    mat = m3.material(2500.0, 1e9, 0.25)
    mesh.hex_grid(m3, origins, 0.01, mat, 3)
    for name in ("position", "mass", "inertia", "inverse", "rotation", "flags"):
        assert np.array_equal(getattr(m2.P, name)[..., :3], getattr(m3.P, name)[..., :3]), name
    for name in ("tri", "tricol", "triobs"):
        assert np.array_equal(getattr(m2.Tr, name)[..., :m2.trinum], getattr(m3.Tr, name)[..., :m3.trinum])
    assert np.array_equal(m2.F.facnod[:, :m2.facnum], m3.F.facnod[:, :m3.facnum])
    assert np.array_equal(m2.N.nodes[:, :m2.nodnum], m3.N.nodes[:, :m3.nodnum])


@pytest.mark.parametrize("nodes, ele, err", [
    ([0.0] * 24, [7, 0, 1, 2, 3, 4, 5, 6, 0], "4, 5, 6, or 8 nodes"),
    ([0.0] * 24, [8, 0, 1, 2, 3, 4, 5, 6], "incomplete"),
    ([0.0] * 23, [4, 0, 1, 2, 3, 0], "multiple of 3"),
    ([0.0] * 12, [4, 0, 1, 2, 4, 0], "outside of range"),
])
def test_mesh_argument_errors(nodes, ele, err):
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    with pytest.raises(ValueError, match=err):
        m.mesh(nodes, ele, mat, 1)


def test_spring_lattice_scene():
    from parmec_gb300.scenes import spring_lattice
    m, dt = spring_lattice(8)
    assert m.parnum == 65 and m.trinum == 65 * 12 and m.nodnum == 65 * 8
    assert m.sprnum == 2 * 8 * 7 + 64
    assert 1e-7 < dt < 1e-4
