"""OUTPUT and the VTK/DUMP files (input.cpp:3560-3955, output.cpp:54-5140):
file names, frame counts, dataset layout and values, for unselected
particles and for a subset."""
import os

import numpy as np
import pytest

from parmec_gb300.model import Model


def scene(tmp):
    from parmec_gb300.scenes import box_triangles
    m = Model()
    m.out.path = os.path.join(tmp, "deck")
    mat = m.material(1000.0, 1e9, 0.25)
    a = m.sphere((0.3, 0.3, 0.3), 0.05, mat, 1)
    b = m.sphere((0.5, 0.3, 0.3), 0.05, mat, 1)
    m.obstacle(box_triangles((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), 2, point=(0.5, 0.5, 0.5),
               angular=lambda t: (0.0, 0.0, 0.5))
    m.granular(0, 0, 1e5, 0.2, 0.5)
    m.spring(a, (0.3, 0.3, 0.3), b, (0.5, 0.3, 0.3), [-1.0, -1e3, 1.0, 1e3])
    m.torsion_spring(a, b, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), kroll=[-1.0, 1e2, 1.0, -1e2])
    m.velocity(a, linear=(0.1, 0.0, 0.0), angular=(0.0, 0.0, 1.0))
    m.set_gravity(0.0, 0.0, -9.81)
    return m, a, b


def read_vtk(path):
    lines = open(path).read().split("\n")
    assert lines[0] == "# vtk DataFile Version 2.0" and lines[2] == "ASCII"
    return lines


def test_vtk_and_dump_files(tmp_path, oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, a, b = scene(str(tmp_path))
    from parmec_gb300 import output
    output.output_command(m, ["NUMBER", "DISPL", "LINVEL", "ANGVEL", "FORCE", "TORQUE", "COLOR", "F", "SF", "FF",
                              "LENGTH", "ORIENT", "ZDIR", "XDIR", "YDIR", "TRQROT", "TRQTOT", "TRQSPR",
                              "ORIENT1", "ORIENT2", "ORIENT3"], format=["VTK", "DUMP"])
    output.output_command(m, ["NUMBER", "LINVEL"], subset=[b], mode=["RB", "SL", "SPH"])
    dt = 1e-4
    m.dem(10 * dt, dt, interval=(3 * dt, 1e9), engine=OracleEngine())
    names = sorted(os.listdir(tmp_path))
    frames = sorted(int(n.split(".")[-1]) for n in names if n.startswith("deck0rb.vtk."))
    assert frames == list(range(len(frames))) and len(frames) == 4     # t = 0, 3, 6 and 9 steps
    for tag in ("deck0.vtk", "deck0rb.vtk", "deck0sl.vtk", "deck0st.vtk", "deck1rb.vtk", "deck1sl.vtk"):
        assert any(n.startswith(tag + ".") for n in names), tag
    assert "deck0.dump" in names and "deck1.dump" in names
    last = frames[-1]
    rb = read_vtk(os.path.join(tmp_path, f"deck0rb.vtk.{last}"))
    assert rb[3] == "DATASET UNSTRUCTURED_GRID" and rb[4] == "POINTS 1 float"
    x = [float(v) for v in rb[5].split()]
    assert np.allclose(x, m.P.position[0:3, a], rtol=1e-5)               # %g keeps six digits
    assert "VECTORS ORIENT1 float" in rb and "SCALARS NUMBER int" in rb
    sub = read_vtk(os.path.join(tmp_path, f"deck1rb.vtk.{last}"))
    assert sub[4] == "POINTS 1 float" and "VECTORS LINVEL float" in sub and "VECTORS FORCE float" not in sub
    tri = read_vtk(os.path.join(tmp_path, f"deck0.vtk.{last}"))
    assert "POINTS 36 float" in tri and "CELLS 12 48" in tri and "CELL_TYPES 12" in tri
    st = read_vtk(os.path.join(tmp_path, f"deck0st.vtk.{last}"))
    assert "VECTORS TRQTOT float" in st and "POINTS 1 float" in st
    sl = read_vtk(os.path.join(tmp_path, f"deck1sl.vtk.{last}"))
    assert "POINTS 1 float" in sl and "SCALARS number int" in sl
    dump = open(os.path.join(tmp_path, "deck0.dump")).read()
    assert dump.count("ITEM: TIMESTEP") == 4 and "ITEM: ATOMS id x y z radius vx vy vz" in dump


def test_output_command_errors(tmp_path):
    from parmec_gb300 import output
    m, a, b = scene(str(tmp_path))
    with pytest.raises(ValueError):
        output.output_command(m, ["NOPE"])
    with pytest.raises(ValueError):
        output.output_command(m, subset=[7])
    with pytest.raises(ValueError):
        output.output_command(m, mode="XX")
    with pytest.raises(ValueError):
        output.output_command(m, format="PNG")


def test_xdmf_default_writes_nothing(tmp_path, oracle_lib):
    from oracle.pyoracle import OracleEngine
    m, a, b = scene(str(tmp_path))
    m.dem(5e-4, 1e-4, interval=(2e-4, 1e9), engine=OracleEngine())
    assert os.listdir(tmp_path) == [] and m.out.frame > 0


@pytest.mark.gpu
def test_gpu_files_equal_oracle_files(tmp_path, gpu_lib, oracle_lib):
    """The files written from the GPU session's state equal, byte for byte,
    those written from the oracle's (the state is bit-identical)."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300 import output
    from parmec_gb300.engine import GpuEngine
    out = {}
    for tag, make_engine in (("gpu", GpuEngine), ("oracle", OracleEngine)):
        d = tmp_path / tag
        d.mkdir()
        m, a, b = scene(str(d))
        output.output_command(m, format=["VTK", "DUMP"])
        m.dem(10 * 1e-4, 1e-4, interval=(3e-4, 1e9), engine=make_engine())
        out[tag] = {n: (d / n).read_bytes() for n in sorted(os.listdir(d))}
    assert out["gpu"].keys() == out["oracle"].keys() and len(out["gpu"]) > 10
    for n in out["gpu"]:
        assert out["gpu"][n] == out["oracle"][n], n

