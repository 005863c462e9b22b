"""The configurations at their stated sizes, and the long spring runs, on the GPU.

* The CPU-runnable hopper fill (4,096 spheres, friction 0.5, 1,000 steps):
  the session against the oracle bit for bit.
* The spring-lattice shaking table at 256 x 256 (65,536 MESH cubes, 196,096
  springs, a 65,536-spring base run, 786,444 triangles), 20 steps: every
  particle, node, triangle and spring word bit for bit.
* Spring runs summed in several groups of chunks (a 48 x 48 lattice: a
  2,304-spring base run, two groups) and a synthetic run of 67,320 springs
  (66,000 towards one particle with ground springs between them, so the
  chunks double past 65,536 and the run skips entries whose second particle
  is the ground): the session, adaptive steps and the drop-in exports bit for
  bit.
* The 512-scene batch (9.04M spheres) in the mixed form against the FP64
  form after 100 steps: per-scene energy within 1e-6 relative and positions
  within 1e-6 m.
* The exponential map above its Taylor threshold (|Omega h|^2 >= 0.0305,
  macros.h:1466): there the device's sin/cos and the host's differ in the
  last bits, so the rotations agree within 1e-12 relative instead of bit for
  bit.
"""
import copy
import math
import os

import numpy as np
import pytest

from helpers import assert_bitwise, bits

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def spring_state_equal(ma, mb):
    for name in ("stroke", "sprfrc", "sprpnt", "sprdir"):
        a, b = getattr(ma.S, name)[:, :ma.sprnum], getattr(mb.S, name)[:, :mb.sprnum]
        assert np.array_equal(bits(a), bits(b)), name


def test_hopper_fill_full_deck_bitwise(gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import hopper_fill
    (mg, dt), (mo, _) = hopper_fill(), hopper_fill()
    assert mg.parnum == 4096
    mg.dem(1000 * dt - 0.5 * dt, dt, interval=1e9, engine=GpuEngine())
    mo.dem(1000 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine(threads=THREADS))
    assert_bitwise(mg, mo, where="hopper 4096 x 1000: ")


def test_spring_lattice_full_size_bitwise(gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import spring_lattice
    (mg, dt), (mo, _) = spring_lattice(256), spring_lattice(256)
    assert mg.parnum == 65537 and mg.sprnum == 196096
    mg.dem(20 * dt - 0.5 * dt, dt, interval=1e9, engine=GpuEngine())
    mo.dem(20 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine(threads=THREADS))
    assert_bitwise(mg, mo, where="lattice 256: ")
    spring_state_equal(mg, mo)
    assert np.array_equal(bits(mg.N.nodes[:, :mg.nodnum]), bits(mo.N.nodes[:, :mo.nodnum]))
    assert np.array_equal(bits(mg.Tr.tri[:, :mg.trinum]), bits(mo.Tr.tri[:, :mo.trinum]))


def long_run(n=66000):
    """n bodies each on a spring to one base particle (a k-run of n springs
    on the base), every 50th also on a spring to the ground, sorted between
    them; the base moves with a prescribed velocity."""
    from parmec_gb300.model import Model
    m = Model()
    m.material(1000.0, 1e9, 0.25)
    base = m.analytical([1.0, 1.0, 1.0, 0.0, 0.0, 0.0], 10.0, position=(0.0, 0.0, 0.0))
    for i in range(n):
        x, y = 0.001 * (i % 300), 0.001 * (i // 300)
        p = m.analytical([1e-6, 1e-6, 1e-6, 0.0, 0.0, 0.0], 0.01, position=(x, y, 0.01))
        m.spring(p, (x, y, 0.01), base, (x, y, 0.0), [-1.0, -1e3, 1.0, 1e3], dashpot=0.1)
        if i % 50 == 7:
            m.spring(p, (x, y, 0.01), -1, (x, y, 0.02), [-1.0, -5e2, 1.0, 5e2])
    m.prescribe_motion(base, linear=lambda t: (0.5 * math.sin(2 * math.pi * 5.0 * t), 0.0, 0.0), kind="vv")
    return m


def lattice48():
    from parmec_gb300.scenes import spring_lattice
    return spring_lattice(48)


@pytest.mark.parametrize("make", [lattice48, lambda: (long_run(), 1e-4)], ids=["lattice48", "run67320"])
def test_long_spring_runs_session_and_adaptive(make, gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    (mg, dt), (mo, _) = make(), make()
    eg, eo = GpuEngine(), OracleEngine(threads=THREADS)
    mg.dem(20 * dt - 0.5 * dt, dt, interval=1e9, engine=eg)
    mo.dem(20 * dt - 0.5 * dt, dt, interval=1e9, engine=eo)
    assert_bitwise(mg, mo, where="fixed step: ")
    spring_state_equal(mg, mo)
    mg.dem(10 * dt, dt, interval=1e9, adaptive=0.5, engine=eg)
    mo.dem(10 * dt, dt, interval=1e9, adaptive=0.5, engine=eo)
    assert mg.curstep == mo.curstep
    assert_bitwise(mg, mo, where="adaptive: ")


@pytest.mark.parametrize("make", [lattice48, lambda: (long_run(), 1e-4)], ids=["lattice48", "run67320"])
def test_long_spring_runs_dropin(make, gpu_lib, oracle_lib):
    from oracle import dem_loop
    from oracle.pyoracle import OracleEngine
    lib = dem_loop.library()
    lib.pg_compat_exit_on_error(0)
    (mc, dt), (mo, _) = make(), make()
    host = dem_loop.Host(lib, mc)
    eo = OracleEngine(threads=THREADS)
    mo.dem(10 * dt - 0.5 * dt, dt, interval=1e9, engine=eo)
    dem_loop.dem(lib, host, 10 * dt - 0.5 * dt, dt)
    assert_bitwise(mc, mo)
    mo.dem(5 * dt, dt, interval=1e9, adaptive=0.5, engine=eo)
    dem_loop.dem(lib, host, 5 * dt, dt, adaptive=0.5)
    assert mc.curstep == mo.curstep
    assert_bitwise(mc, mo, where="adaptive drop-in: ")
    host.close()


def test_batch_full_size_mixed_against_fp64(gpu_lib):
    from parmec_gb300 import abi, batch
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import batch_scenes
    from parmec_gb300.serving import range_energy
    parts = batch_scenes(512)
    dt = parts[0][1]
    steps = 100
    out = {}
    for form in (abi.PG_FORM_FP64, abi.PG_FORM_MIXED):
        models = [copy.deepcopy(p[0]) for p in parts]
        P, ranges = batch.pool(models)
        eng = GpuEngine(form=form)
        eng.attach(P)
        for k, (_, _, exc) in enumerate(parts):
            eng.set_scene(k, True, excitation=exc, start=0)
        P.engine = eng
        P._dirty = False
        P.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        n = P.parnum
        out[form] = {"x": np.array(P.P.position[0:3, :n]),
                     "E": np.array([range_energy(P, r[0], r[1], p[2][0:3]) for r, p in zip(ranges, parts)])}
        eng.close()
        del P, models
    a, b = out[abi.PG_FORM_MIXED], out[abi.PG_FORM_FP64]
    assert float(np.max(np.abs(a["x"] - b["x"]))) <= 1e-6
    rel = np.abs(a["E"] - b["E"]) / np.abs(b["E"])
    assert float(rel.max()) <= 1e-6, float(rel.max())


def test_expmap_above_taylor_threshold(gpu_lib, oracle_lib):
    """Free spinning spheres with |Omega h|^2 of 0.04-0.09: both expmap calls
    of every step take the sin/cos branch; rotations and spins within 1e-12
    relative of the oracle's after 50 steps."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.model import Model
    step = 2e-5

    def make():
        rng = np.random.default_rng(9)
        m = Model()
        mat = m.material(2500.0, 1e9, 0.25)
        for k in range(64):
            p = m.sphere((0.1 * (k % 8), 0.1 * (k // 8), 0.0), 0.01, mat, 1)
            w = rng.normal(size=3)
            w *= rng.uniform(1.0e4, 1.5e4) / np.linalg.norm(w)
            m.velocity(p, angular=tuple(float(x) for x in w))
        return m
    mg, mo = make(), make()
    om = np.linalg.norm(mo.P.angular[3:6, :mo.parnum], axis=0)
    assert np.all((om * step) ** 2 >= 0.0305)
    mg.dem(50 * step - 0.5 * step, step, interval=1e9, engine=GpuEngine())
    mo.dem(50 * step - 0.5 * step, step, interval=1e9, engine=OracleEngine())
    for name in ("rotation", "angular", "position"):
        a, b = getattr(mg.P, name)[..., :mg.parnum], getattr(mo.P, name)[..., :mo.parnum]
        assert float(np.max(np.abs(a - b))) <= 1e-12 * float(np.max(np.abs(b))), name
