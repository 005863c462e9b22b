"""The benchmark workloads at their full sizes, on the GPU.

* The 1,048,576-sphere rotating drum (4,096-triangle cylinder at 2 rad/s):
  the CUDA session against the oracle after the initial half step and 4
  steps, bit for bit -- every state word and the whole contact list.  The
  oracle runs on all host threads; its contact and force loops keep lists
  private to each master particle and sum in fixed orders, so its result does
  not depend on the thread count.
* The same drum in the mixed form against the FP64 form after 100 steps:
  total energy within 1e-6 relative (the stated bound of the mixed form),
  positions within 1e-6 m, the same contact pairs but for pairs whose gap is
  within twice the largest position difference of zero (at most one in 1e5).
* The 512-scene batch (9.04M spheres, sizes log-uniform in [2048, 65536],
  each scene with its own base excitation): the fused step kernel
  gives the per-phase kernels' state bit for bit after 20 steps.
"""
import copy

import numpy as np
import pytest

from helpers import assert_bitwise, assert_contacts_equal, assert_spheres_bitwise, bits

pytestmark = pytest.mark.gpu

DRUM = 1 << 20


@pytest.fixture(scope="module")
def drum_model():
    from parmec_gb300.scenes import drum
    m, dt, _ = drum(DRUM)
    return m, dt


def test_drum_full_size_bitwise_against_oracle(gpu_lib, oracle_lib, drum_model):
    import os
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    m0, dt = drum_model
    mg, mo = copy.deepcopy(m0), copy.deepcopy(m0)
    eg, eo = GpuEngine(), OracleEngine(threads=os.cpu_count() or 1)
    steps = 4
    mg.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eg)
    mo.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eo)
    assert mg.parnum == DRUM
    assert_bitwise(mg, mo, where="drum 1M: ")
    assert_spheres_bitwise(mg, mo)
    cg, co = eg.contacts(), eo.contacts()
    assert len(co["mpart"]) > DRUM // 2
    assert_contacts_equal(cg, co)
    eg.close()
    eo.close()


def test_drum_full_size_mixed_within_bounds(gpu_lib, drum_model):
    from parmec_gb300 import abi, energy
    from parmec_gb300.engine import GpuEngine
    m0, dt = drum_model
    out = {}
    for form in (abi.PG_FORM_FP64, abi.PG_FORM_MIXED):
        m = copy.deepcopy(m0)
        eng = GpuEngine(form=form)
        m.dem(100 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        c = eng.contacts()
        out[form] = (m, set(zip(c["mpart"].tolist(), c["code"].tolist())))
        eng.close()
    (m64, p64), (mmx, pmx) = out[abi.PG_FORM_FP64], out[abi.PG_FORM_MIXED]
    n = m64.parnum
    dx = np.max(np.abs(m64.P.position[0:3, :n] - mmx.P.position[0:3, :n]))
    assert dx <= 1e-6, dx
    E64, Emx = energy.total(m64), energy.total(mmx)
    assert abs(Emx - E64) <= 1e-6 * abs(E64), (E64, Emx)
    # contact sets: at a million spheres a few pairs sit at a gap closer to
    # zero than the two forms' position difference, and the forms may count
    # them differently; any pair in one set only must be such a pair
    diff = p64 ^ pmx
    assert len(diff) <= max(2, len(p64) // 100000), len(diff)
    c, r = m64.E.center, m64.E.radii[0]
    for i, j in diff:
        if j >= 0:
            gap = r[i] + r[j] - np.sqrt(np.sum((c[0:3, i] - c[0:3, j]) ** 2))
            assert abs(gap) <= 2.0 * dx + 1e-12, (i, j, gap, dx)


def test_batch_full_size_fused_equals_per_phase(gpu_lib):
    from parmec_gb300 import abi, batch
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import batch_scenes
    parts = batch_scenes(512)
    assert sum(p[0].parnum for p in parts) > 9_000_000
    dt = parts[0][1]
    steps = 20
    states = []
    for fused in (False, True):
        models = [copy.deepcopy(p[0]) for p in parts]
        P, _ = batch.pool(models)
        eng = GpuEngine(form=abi.PG_FORM_MIXED, fused=fused, autotune=fused)
        eng.attach(P)
        for k, (_, _, exc) in enumerate(parts):
            eng.set_scene(k, True, excitation=exc, start=0)
        P.engine = eng
        P._dirty = False
        P.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        n = P.parnum
        states.append({k: np.array(getattr(P.P, k)[..., :n]) for k in ("position", "linear", "angular",
                                                                        "rotation", "force", "torque")})
        eng.close()
        del P, models
    for k in states[0]:
        assert np.array_equal(bits(states[0][k]), bits(states[1][k])), k
