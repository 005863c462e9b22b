"""The committed golden fixtures (tests/golden/, made by make_golden.py).

CPU: the oracle, run again, reproduces every stored array bit for bit, and
the projectile deck stays within the reference's own tolerance of its
published answer.  GPU: the CUDA session reproduces the same stored bits, so
the device path is checked against a fixed target as well as against a live
oracle run.
"""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_golden  # noqa: E402


def _digests():
    with open(os.path.join(HERE, "digests.json")) as f:
        return json.load(f)


def _check(name, out):
    want = _digests()[name]
    assert sorted(want) == sorted(out), f"{name}: stored arrays {sorted(want)} vs produced {sorted(out)}"
    bad = []
    for k, (shape, dig) in want.items():
        a = out[k]
        if list(a.shape) != shape or make_golden.digest(a) != dig:
            bad.append(k)
    if bad and name not in make_golden.DIGEST_ONLY:
        ref = np.load(os.path.join(HERE, name + ".npz"))
        msg = []
        for k in bad:
            a, b = out[k], ref[k]
            if a.shape != b.shape:
                msg.append(f"{k}: shape {a.shape} vs stored {b.shape}")
            else:
                msg.append(f"{k}: {int(np.sum(a != b))} words differ, max abs diff {np.max(np.abs(a - b)):.3e}")
        raise AssertionError(f"{name}: " + "; ".join(msg))
    assert not bad, f"{name}: arrays differ from the stored digests: {bad}"


@pytest.mark.parametrize("name", list(make_golden.CASES))
def test_oracle_reproduces_golden(oracle_lib, name):
    from oracle.pyoracle import OracleEngine
    _, out = make_golden.run_case(name, OracleEngine())
    _check(name, out)


def test_oracle_damping_deck(oracle_lib):
    from oracle.pyoracle import OracleEngine
    with open(os.path.join(HERE, "reference_decks.json")) as f:
        deck = json.load(f)["damping"]
    x = make_golden.damping_history(OracleEngine())
    ref = np.load(os.path.join(HERE, "damping.npz"))["x"]
    assert np.array_equal(x.view(np.int64), ref.view(np.int64))
    assert abs(x[-1] / 0.0254 - deck["expected"]) / deck["expected"] < deck["rel_tol"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(make_golden.CASES))
def test_gpu_reproduces_golden(gpu_lib, name):
    from parmec_gb300.engine import GpuEngine
    eng = GpuEngine()
    try:
        _, out = make_golden.run_case(name, eng)
    finally:
        eng.close()
    _check(name, out)


@pytest.mark.gpu
def test_gpu_damping_deck(gpu_lib):
    from parmec_gb300.engine import GpuEngine
    eng = GpuEngine()
    try:
        x = make_golden.damping_history(eng)
    finally:
        eng.close()
    ref = np.load(os.path.join(HERE, "damping.npz"))["x"]
    assert np.array_equal(x.view(np.int64), ref.view(np.int64))
