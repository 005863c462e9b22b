"""Scenes sharing one session: each scene's result is bitwise the same alone
and in the pool (both forms), and the pool matches the oracle for scenes
driven by the step table (FP64)."""
import numpy as np
import pytest

from helpers import bits

pytestmark = pytest.mark.gpu


def run_pool(makers, steps, form, fused=False, autotune=False, info=None):
    from parmec_gb300 import abi, batch
    from parmec_gb300.engine import GpuEngine
    parts = [mk() for mk in makers]
    models = [p[0] for p in parts]
    dt = parts[0][1]
    P, ranges = batch.pool(models)
    eng = GpuEngine(form=form, fused=fused, autotune=autotune)
    eng.attach(P)
    for k, (_, _, exc) in enumerate(parts):
        eng.set_scene(k, True, excitation=exc, start=0)
    P.engine = eng
    P._dirty = False
    P.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    out = []
    for k, m in enumerate(models):
        batch.extract(P, k, m)
        out.append(m)
    if info is not None:
        info["config"] = eng.fused_config() if fused else None
        info["launches"] = eng.kernel_launches()
    eng.close()
    return out


def makers():
    from parmec_gb300.scenes import shaken_box
    return [lambda: shaken_box(64, 1, 5.0, 0.5), lambda: shaken_box(216, 2, 12.0, 0.9),
            lambda: shaken_box(27, 3, 2.0, 0.2), lambda: shaken_box(125, 4, 17.0, 1.0)]


@pytest.mark.parametrize("form", [0, 1])
def test_alone_equals_in_the_pool(gpu_lib, form):
    mk = makers()
    together = run_pool(mk, 120, form)
    for k, f in enumerate(mk):
        alone = run_pool([f], 120, form)[0]
        m = together[k]
        n = m.parnum
        for name in ("position", "linear", "angular", "rotation"):
            a = getattr(alone.P, name)[..., :n]
            b = getattr(m.P, name)[..., :n]
            assert np.array_equal(bits(a), bits(b)), (k, name)


def test_pool_of_table_driven_scenes_matches_oracle(gpu_lib, oracle_lib):
    """Without excitation the pool steps every scene with the step table's
    gravity; each scene then equals the oracle run of that scene alone."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300 import batch
    from parmec_gb300.engine import GpuEngine
    from helpers import make_collision_scene, assert_bitwise
    mk = [lambda: make_collision_scene(n_side=3, seed=41), lambda: make_collision_scene(n_side=4, seed=42)]
    models = [f()[0] for f in mk]
    dt = mk[0]()[1]
    P, ranges = batch.pool(models)
    eng = GpuEngine()
    eng.attach(P)
    P.engine = eng
    P._dirty = False
    P.dem(60 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    for k, f in enumerate(mk):
        batch.extract(P, k, models[k])
        ref, _ = f()
        ref.dem(60 * dt - 0.5 * dt, dt, interval=1e9, engine=OracleEngine())
        assert_bitwise(models[k], ref, names=("position", "linear", "angular", "rotation"))


def same_state(a, b):
    n = a.parnum
    for name in ("position", "linear", "angular", "rotation"):
        x = getattr(a.P, name)[..., :n]
        y = getattr(b.P, name)[..., :n]
        assert np.array_equal(bits(x), bits(y)), name


@pytest.mark.parametrize("autotune", [False, True])
def test_fused_step_kernel_equals_per_phase_kernels(gpu_lib, autotune):
    """The fused step kernel (mixed form) gives the per-phase kernels'
    state bit for bit, whatever launch shapes the autotuner tries on the way."""
    mk = makers()
    ref = run_pool(mk, 150, 1)
    info = {}
    got = run_pool(mk, 150, 1, fused=True, autotune=autotune, info=info)
    for a, b in zip(ref, got):
        same_state(a, b)
    threads, blocks, tuned, graph = info["config"]
    assert threads in (256, 512) and blocks >= 1
    assert graph == 1                          # replayed as a captured CUDA graph
    if autotune:
        assert tuned == 1


def test_fused_single_scene_with_rebuilds(gpu_lib):
    """One collision scene with a tiny skin: the in-kernel rebuild (radix sort,
    candidate lists, slave lists) runs nearly every step."""
    from helpers import make_collision_scene
    from parmec_gb300 import abi
    from parmec_gb300.engine import GpuEngine
    out = []
    for fused in (False, True):
        m, dt = make_collision_scene(n_side=5, seed=3)
        eng = GpuEngine(form=abi.PG_FORM_MIXED, skin=1e-5, fused=fused)
        m.dem(100 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        out.append(m)
    same_state(out[0], out[1])
