"""Failure detection without a GPU fault: a bounded device wait that runs out.

The cooperative kernels' grid barrier waits at most 2 s.  The self-test makes
a small cooperative grid wait at a barrier that cannot complete; the kernel
must give up, record PG_ERR_TIMEOUT for the host, and leave the context
usable (a DEM call runs afterwards and still matches the oracle)."""
import ctypes

import pytest

from helpers import assert_bitwise, make_collision_scene

pytestmark = pytest.mark.gpu


def test_grid_barrier_gives_up_and_the_session_survives(gpu_lib, oracle_lib):
    from oracle.pyoracle import OracleEngine
    from parmec_gb300 import abi
    from parmec_gb300.engine import GpuEngine
    mg, dt = make_collision_scene(n_side=3, seed=2)
    eng = GpuEngine()
    mg.dem(10 * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    ms = ctypes.c_double()
    assert eng.lib.pg_session_barrier_selftest(eng.sess, ctypes.byref(ms)) == abi.PG_OK
    assert 1500.0 < ms.value < 10000.0           # waited for its limit, then returned
    mg.dem(20 * dt, dt, interval=1e9, engine=eng)
    mo, _ = make_collision_scene(n_side=3, seed=2)
    eo = OracleEngine()
    mo.dem(10 * dt - 0.5 * dt, dt, interval=1e9, engine=eo)
    mo.dem(20 * dt, dt, interval=1e9, engine=eo)
    assert_bitwise(mg, mo)
