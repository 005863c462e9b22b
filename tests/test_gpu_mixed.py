"""The mixed-precision form (FP32 contact geometry and forces, compensated
FP32 pairs for positions, velocities, rotations and the near-touching gap)
against the plain FP64 form, which is bit-identical to the oracle.

Stated tolerances (checked here, reported by bench.py for the drum):
  positions     max |dx| <= 2e-7 * scene size after 200 steps of a fast
                collision scene (FP32 contact forces differ by ~1e-7
                relative; 200 steps of collisions amplify that to ~1e-8 m)
  forces        normwise max |dF| <= 1e-3 * max |F|
  energy        |E_mixed - E_fp64| <= 1e-6 * |E_fp64| (total) and
                <= 1e-4 * KE (kinetic alone)
and the two forms see the same contact pairs.
"""
import numpy as np
import pytest

from helpers import make_collision_scene

pytestmark = pytest.mark.gpu


def run(form, steps, make):
    from parmec_gb300 import abi
    from parmec_gb300.engine import GpuEngine
    m, dt = make()
    eng = GpuEngine(form=form)
    m.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    return m, eng


@pytest.mark.parametrize("seed,moving", [(7, False), (13, True)])
def test_mixed_against_fp64(gpu_lib, seed, moving):
    from parmec_gb300 import abi, energy
    make = lambda: make_collision_scene(n_side=5, seed=seed, moving=moving)
    m64, e64 = run(abi.PG_FORM_FP64, 200, make)
    mmx, emx = run(abi.PG_FORM_MIXED, 200, make)
    n = m64.parnum
    dx = np.max(np.abs(m64.P.position[0:3, :n] - mmx.P.position[0:3, :n]))
    assert dx <= 2e-7 * 0.4, dx
    F64, Fmx = m64.P.force[:, :n], mmx.P.force[:, :n]
    assert np.max(np.abs(F64 - Fmx)) <= 1e-3 * np.max(np.abs(F64)), np.max(np.abs(F64 - Fmx)) / np.max(np.abs(F64))
    E64, Emx = energy.total(m64), energy.total(mmx)
    assert abs(Emx - E64) <= 1e-6 * abs(E64), (E64, Emx)
    K64, Kmx = energy.kinetic(m64), energy.kinetic(mmx)
    assert abs(Kmx - K64) <= 1e-4 * K64, (K64, Kmx)
    c64, cmx = e64.contacts(), emx.contacts()
    p64 = set(zip(c64["mpart"].tolist(), c64["code"].tolist()))
    pmx = set(zip(cmx["mpart"].tolist(), cmx["code"].tolist()))
    assert p64 == pmx


def test_mixed_repeatable(gpu_lib):
    from parmec_gb300 import abi
    from helpers import bits
    a, _ = run(abi.PG_FORM_MIXED, 100, lambda: make_collision_scene(n_side=5, seed=3))
    b, _ = run(abi.PG_FORM_MIXED, 100, lambda: make_collision_scene(n_side=5, seed=3))
    assert np.array_equal(bits(a.P.position[:, :a.parnum]), bits(b.P.position[:, :b.parnum]))


def test_mixed_rejects_springs(gpu_lib):
    from parmec_gb300 import abi
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.model import Model
    m = Model()
    m.material(1.0, 1.0, 0.25)
    p = m.analytical()
    m.spring(p, (0, 0, 0), -1, (0, 0, 0), [-1.0, -1.0, 1.0, 1.0])
    with pytest.raises(RuntimeError):
        m.dem(0.1, 0.01, engine=GpuEngine(form=abi.PG_FORM_MIXED))
