"""UNSPRING (input.cpp:2083-2295, unspring_task forces.ispc:2058-2127):
springs fail when a monitored quantity of tested springs leaves its limits
nfreq times, and inactive springs switch on.  CPU tests run the oracle; the
GPU tests compare the session and the drop-in exports with it bit for bit."""
import pytest

from helpers import assert_bitwise
from parmec_gb300.model import Model


def hanging(k=1e4, nfreq=3, unload=None, entity=None, operator=None):
    """A sphere on a spring to a ground point above it; gravity stretches the
    spring until its elastic force passes 0.8 m g, which fails it and switches
    on a second, inactive spring to a point below."""
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    p = m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    s0 = m.spring(p, (0.0, 0.0, 0.0), -1, (0.0, 0.0, 0.5), [-1.0, -k, 1.0, k])
    s1 = m.spring(p, (0.0, 0.0, 0.0), -1, (0.0, 0.0, -0.5), [-1.0, -k, 1.0, k], inactive=True)
    m.set_gravity(0.0, 0.0, -9.81)
    mg = m.P.mass[p] * 9.81
    tl = None
    if unload is not None:
        tl = m.tseries(unload)
    m.unspring([s0], [s0], (None, 0.8 * mg), entity=entity, operator=operator, nfreq=nfreq,
               unload=-1 if tl is None else tl, activate=[s1])
    return m, p, s0, s1


def run_oracle(m, calls, dt=1e-4, steps=20):
    from oracle.pyoracle import OracleEngine
    eng = OracleEngine()
    out = []
    for _ in range(calls):
        m.dem(steps * dt, dt, interval=1e9, engine=eng)
        S = m.S
        out.append((list(S.unspring[:2]), int(m.unspring_nfreq[0]), float(S.sprfrc[1, S.sprmap[0]]),
                    float(S.sprfrc[1, S.sprmap[1]])))
    return out


def test_failure_and_activation(oracle_lib):
    m, p, s0, s1 = hanging()
    out = run_oracle(m, 6)
    assert out[0][:2] == ([-2, -1], 3)                  # monitored: in use; second: inactive
    fired = [o for o in out if o[1] == 0]
    assert fired, "the rule never fired"
    u, nf, f0, f1 = fired[0]
    assert u == [-1, -3] and f0 == 0.0 and f1 < 0.0      # failed to zero; the lower spring pushes
    counts = [o[1] for o in out]
    assert counts == sorted(counts, reverse=True)       # nfreq counts down once per violating step


def test_rule_within_limits_never_fires(oracle_lib):
    """MIN of |SF| stays far below a huge upper limit."""
    m = Model()
    mat = m.material(1000.0, 1e9, 0.25)
    p = m.sphere((0.0, 0.0, 0.0), 0.05, mat, 1)
    s0 = m.spring(p, (0.0, 0.0, 0.0), -1, (0.0, 0.0, 0.5), [-1.0, -1e4, 1.0, 1e4])
    m.set_gravity(0.0, 0.0, -9.81)
    m.unspring([s0], [s0], (-1e9, 1e9), entity="SF", operator="MIN", abs=True)
    out = run_oracle(m, 3)
    assert all(o[0][0] == -2 and o[1] == 1 for o in out)


def test_unload_curve_reaches_zero(oracle_lib):
    """With an unload TSERIES the failed spring's force returns towards zero
    along the curve and the spring is switched off once it crosses zero."""
    m, p, s0, s1 = hanging(nfreq=1, unload=[0.0, 0.0, 1.0, 1e5])
    from oracle.pyoracle import OracleEngine
    eng = OracleEngine()
    S = m.S
    seen = []
    for _ in range(40):
        m.dem(5e-4, 1e-4, interval=1e9, engine=eng)
        seen.append((int(S.unspring[S.sprmap[0]]), float(S.sprfrc[1, S.sprmap[0]])))
    states = [u for u, _ in seen]
    assert 0 in states                                  # unloading along lcurve 0
    assert states[-1] == -1 and seen[-1][1] == 0.0


def test_command_errors():
    m, p, s0, s1 = hanging()
    with pytest.raises(ValueError):
        m.unspring([s0], [s0], (None, 1.0))            # s0 already monitored
    with pytest.raises(ValueError):
        m.unspring([s0], [s1], (None, 1.0))            # s1 is inactive
    s2 = m.spring(p, (0.0, 0.0, 0.0), -1, (0.5, 0.0, 0.0), [-1.0, -1.0, 1.0, 1.0])
    with pytest.raises(ValueError):
        m.unspring([s0], [s2], (1.0, 0.0))             # lower >= upper
    with pytest.raises(ValueError):
        m.unspring([s0], [s2], (None, 1.0), entity="LENGTH")
    with pytest.raises(ValueError):
        m.unspring([s0], [s2], (None, 1.0), operator="AVG")
    with pytest.raises(ValueError):
        m.unspring([7], [s2], (None, 1.0))
    with pytest.raises(ValueError):
        m.unspring([s0], [s2], (None, 1.0), activate=[s0])   # s0 is active
    assert m.unspring([s0], [s2], (None, 1.0)) == 1


@pytest.mark.gpu
def test_gpu_unspring_bitwise(gpu_lib, oracle_lib):
    """Session steps: the rule's countdown, the failure, the activation and the
    unload curve equal the oracle's bit for bit."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.engine import GpuEngine
    for kw in ({}, {"nfreq": 1, "unload": [0.0, 0.0, 1.0, 1e5]}, {"entity": "F", "operator": "MAX"}):
        mg, *_ = hanging(**kw)
        mo, *_ = hanging(**kw)
        eg, eo = GpuEngine(), OracleEngine()
        for _ in range(8):
            mg.dem(2e-3, 1e-4, interval=1e9, engine=eg)
            mo.dem(2e-3, 1e-4, interval=1e9, engine=eo)
            assert list(mg.unspring_nfreq) == list(mo.unspring_nfreq)
            assert list(mg.S.unspring[:2]) == list(mo.S.unspring[:2])
            assert_bitwise(mg, mo)


@pytest.mark.gpu
def test_dropin_unspring_bitwise(gpu_lib, oracle_lib):
    """forces() with UNSPRING rules through the drop-in exports."""
    import ctypes

    from oracle import dem_loop as ispc_loop
    from oracle.pyoracle import OracleEngine
    lib = ispc_loop.library()
    lib.pg_compat_exit_on_error(0)
    mc, *_ = hanging(nfreq=1, unload=[0.0, 0.0, 1.0, 1e5])
    mo, *_ = hanging(nfreq=1, unload=[0.0, 0.0, 1.0, 1e5])
    host = ispc_loop.Host(lib, mc)
    eo = OracleEngine()
    for _ in range(6):
        mo.dem(2e-3, 1e-4, interval=1e9, engine=eo)
        ispc_loop.dem(lib, host, 2e-3, 1e-4)
        assert list(mc.unspring_nfreq) == list(mo.unspring_nfreq)
        assert_bitwise(mc, mo)
    host.close()
    lib.pg_compat_set_skin(ctypes.c_double(0.0))
