"""GPU parity: the CUDA session against the oracle, bit for bit (FP64 form).

Both engines step the same Model through the same host driver (the DEM
command), so every difference comes from the kernels.  Tolerance: zero -- the
FP64 form is compiled without multiply-add contraction and sums in the same
fixed order as the oracle.
"""
import numpy as np
import pytest

from helpers import assert_bitwise, assert_contacts_equal, assert_spheres_bitwise, make_collision_scene

pytestmark = pytest.mark.gpu


def run_pair(make, steps, dt_scale=1.0, record=True, skin=None):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    mg, dt = make()
    mo, _ = make()
    eg = GpuEngine(skin=skin, record_geometry=record)
    eo = OracleEngine()
    step = dt * dt_scale
    mg.dem(steps * step - 0.5 * step, step, interval=1e9, engine=eg)
    mo.dem(steps * step - 0.5 * step, step, interval=1e9, engine=eo)
    return mg, mo, eg, eo


def test_free_particles_bitwise(gpu_lib, oracle_lib):
    """dynamics + euler + shapes for spinning spheres without contacts."""
    def make():
        m, dt = make_collision_scene(n_side=3, spacing=0.2, speed=0.3)
        return m, dt
    mg, mo, eg, eo = run_pair(make, 40)
    assert_bitwise(mg, mo)
    assert_spheres_bitwise(mg, mo)


def test_collisions_bitwise(gpu_lib, oracle_lib):
    """Sphere-sphere and sphere-triangle contacts form and break; all state bitwise equal."""
    mg, mo, eg, eo = run_pair(lambda: make_collision_scene(n_side=5), 120)
    assert_bitwise(mg, mo)
    assert_spheres_bitwise(mg, mo)
    cg, co = eg.contacts(), eo.contacts()
    assert len(co["mpart"]) > 10
    assert_contacts_equal(cg, co)


def test_moving_obstacle_bitwise(gpu_lib, oracle_lib):
    mg, mo, eg, eo = run_pair(lambda: make_collision_scene(n_side=4, moving=True, seed=11), 150)
    assert_bitwise(mg, mo)
    a = mg.Tr.tri[:, :mg.trinum]
    b = mo.Tr.tri[:, :mo.trinum]
    assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_small_skin_many_rebuilds(gpu_lib, oracle_lib):
    """A tiny skin forces candidate-list rebuilds nearly every step."""
    mg, mo, eg, eo = run_pair(lambda: make_collision_scene(n_side=4, seed=5), 80, skin=1e-5)
    assert_bitwise(mg, mo)
    assert_contacts_equal(eg.contacts(), eo.contacts())


def test_hopper_fill_bitwise(gpu_lib, oracle_lib):
    from parmec_gb300.scenes import hopper_fill
    mg, mo, eg, eo = run_pair(lambda: hopper_fill(n_side=8, seed=2, spacing=0.038), 60)
    assert_bitwise(mg, mo)


def test_repeatable(gpu_lib):
    """Two GPU runs of the same deck are bitwise identical (no atomics in the sums)."""
    from parmec_gb300.engine import GpuEngine
    out = []
    for _ in range(2):
        m, dt = make_collision_scene(n_side=5, seed=9)
        m.dem(60 * dt, dt, interval=1e9, engine=GpuEngine())
        out.append(m)
    assert_bitwise(out[0], out[1])


def test_state_edit_between_dem_calls(gpu_lib, oracle_lib):
    """VELOCITY between two DEM calls: the host edit is uploaded, contacts persist."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    out = []
    for eng in (GpuEngine(record_geometry=True), OracleEngine()):
        m, dt = make_collision_scene(n_side=5, seed=21)
        m.dem(40 * dt, dt, interval=1e9, engine=eng)
        for i in range(0, m.parnum, 7):
            m.velocity(i, linear=(0.2, -0.1, 0.3), angular=(1.0, 0.0, -2.0))
        m.dem(40 * dt, dt, interval=1e9, engine=eng)
        out.append((m, eng))
    assert_bitwise(out[0][0], out[1][0])
    assert_contacts_equal(out[0][1].contacts(), out[1][1].contacts())


def test_graph_and_stream_launches_identical(gpu_lib):
    """A captured CUDA graph per step gives the same bits as stream launches."""
    from parmec_gb300.engine import GpuEngine
    out = []
    for graph in (True, False):
        m, dt = make_collision_scene(n_side=5, seed=31, moving=True)
        m.dem(80 * dt, dt, interval=1e9, engine=GpuEngine(graph=graph))
        out.append(m)
    assert_bitwise(out[0], out[1])


def test_run_async_equals_run(gpu_lib):
    """pg_session_run_async enqueues the same steps as pg_session_run: after
    pg_session_sync the state is the same bits; the step tables may be
    rebuilt on the host while the steps run."""
    from parmec_gb300 import driver
    from parmec_gb300.engine import GpuEngine
    out = []
    for asynchronous in (False, True):
        m, dt = make_collision_scene(n_side=5, seed=37, moving=True)
        eng = GpuEngine()
        m.dem(10 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        times, end = driver.step_times(m.curtime, 50 * dt - 0.5 * dt, dt)
        tabs = driver.StepTables(m, times, dt, [1e9, 1e9], [None, None], [-1, -1])
        tab = tabs.ctab(0, len(times))
        if asynchronous:
            eng.run_async(tab, dt)
            tabs = driver.StepTables(m, times, dt, [1e9, 1e9], [None, None], [-1, -1])   # host work meanwhile
            eng.sync()
        else:
            eng.run(tab, dt)
        m.curtime = end
        eng.download()
        out.append(m)
    assert_bitwise(out[0], out[1])
