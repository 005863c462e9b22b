"""The bit-pattern comparisons of the mesh-contact geometry (pg_tritri.cuh,
the same functions the device and the oracle compile) against IEEE
comparisons on the CPU: edge values and seeded random bit patterns."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bit_comparisons_equal_ieee(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ is absent")
    exe = str(tmp_path / "cmp_bits")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "cmp_bits.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe, "2000000"], check=True, capture_output=True, text=True).stdout.split()
    cases, bad = int(out[0]), int(out[1])
    assert cases > 2000000 and bad == 0
