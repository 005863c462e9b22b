"""HISTORY sampling on the GPU: a sample reads only the rows its sources name
(particles, spring positions), gathered on the device, and must equal the
oracle's samples of its full state bit for bit."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_gpu_history_rows_bitwise(gpu_lib, oracle_lib):
    """HISTORY samples taken from gathered rows (pg_session_download_particles
    and _springs) equal the oracle's samples of its full state bit for bit:
    particle, list, point and spring sources."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    from test_gpu_springs import lattice

    def make():
        m = lattice()
        h = [m.history("PX", 3), m.history("VZ", [1, 2, 5]), m.history("|F|", 4),
             m.history("OY", 2), m.history("DX", 6, point=(0.0, 0.0, 0.0)),
             m.history("STROKE", 1), m.history("SF", [0, 2]), m.history("TIME")]
        return m, h
    mg, hg = make()
    mo, ho = make()
    mg.dem(200 * 2e-5, 2e-5, interval=5 * 2e-5, engine=GpuEngine())
    mo.dem(200 * 2e-5, 2e-5, interval=5 * 2e-5, engine=OracleEngine())
    for a, b in zip(hg, ho):
        assert len(a) == len(b) > 30
        assert np.array_equal(np.array(a).view(np.int64), np.array(b).view(np.int64))
