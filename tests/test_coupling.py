"""The C library interface (include/parmec_coupling.h, parmec.h:291-310).

A C program links libparmec_gb300_coupling.so and drives a deck the way a
coupling code drives libparmec8: init, input, prescribed body forces, DEM,
the inner forces back, declare_analytical.  On the CPU it checks the
exports and everything up to DEM; on the GPU it runs two DEM calls and its
printed state equals the oracle's run of the same deck bit for bit.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "parmec_gb300", "_build")
LIB = os.path.join(BUILD, "libparmec_gb300_coupling.so")

DECK = """
import math
mat = MATERIAL(2500.0, 1e9, 0.25)
for k in range(4):
    SPHERE((0.03 * k, 0.0, 0.0105 + 0.001 * k), 0.01, mat, 1)
L = 1.0
OBSTACLE([(-L, -L, 0.0, L, -L, 0.0, L, L, 0.0), (-L, -L, 0.0, L, L, 0.0, -L, L, 0.0)], 2)
GRANULAR(0, 0, 1e5, 0.2, 0.5)
GRAVITY(0.0, 0.0, -9.81)
"""

PROGRAM = r"""
#include <stdio.h>
#include "parmec_coupling.h"
int main(int argc, char **argv)
{
  if (pg_parmec_init() != 0) return 1;
  if (pg_parmec_input(argv[1], argv + 2, argc - 2) != 0) return 2;
  int n = pg_parmec_parnum();
  printf("parnum %d\n", n);
  double f[3] = {0.0, 0.0, 0.5}, t[3] = {0.0, 0.0, 1e-4}, fi[3], ti[3];
  if (pg_parmec_set_body_force(1, f, t) != 0) return 3;
  printf("inner_before %d\n", pg_parmec_get_body_force(1, fi, ti));
  if (argc > 2 && argv[2][0] == 'r')
  {
    double dt = 1e-5, interval[2] = {1e9, 1e9};
    for (int call = 0; call < 2; call ++)
    {
      if (pg_parmec_dem(50 * dt, dt, interval, NULL, 0, 0.0) < 0.0) return 4;
      if (pg_parmec_get_body_force(1, fi, ti) != 0) return 5;
      printf("inner %.17g %.17g %.17g %.17g %.17g %.17g\n", fi[0], fi[1], fi[2], ti[0], ti[1], ti[2]);
    }
  }
  if (pg_parmec_declare_analytical(3) != 0) return 6;
  for (int k = 0; k < n; k ++)
  {
    double x[3], v[3], w[3];
    if (pg_parmec_particle(k, x, v, w) != 0) return 7;
    printf("particle %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", k, x[0], x[1], x[2], v[0], v[1],
           v[2], w[0], w[1], w[2]);
  }
  if (pg_parmec_reset() != 0 || pg_parmec_parnum() != 0) return 8;
  return 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if not os.path.exists(LIB):
        from parmec_gb300 import build
        if build.build_coupling() is None:
            pytest.skip("the Python headers or library are missing: no coupling library")
    if not shutil.which("gcc"):
        pytest.skip("gcc missing")
    d = tmp_path_factory.mktemp("coupling")
    src = d / "drive.c"
    src.write_text(PROGRAM)
    exe = str(d / "drive")
    subprocess.run(["gcc", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe, "-L", BUILD,
                    "-Wl,-rpath," + BUILD, "-lparmec_gb300_coupling"], check=True)
    deck = d / "deck.py"
    deck.write_text(DECK)
    return exe, str(deck)


def run(program, *args):
    exe, deck = program
    env = dict(os.environ)
    env["PYTHONPATH"] = ROOT + os.pathsep + env.get("PYTHONPATH", "")
    r = subprocess.run([exe, deck, *args], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, f"rc {r.returncode}\n{r.stdout}\n{r.stderr[-3000:]}"
    return r.stdout


def test_exports_match_the_header():
    if not os.path.exists(LIB):
        pytest.skip("no coupling library")
    with open(os.path.join(ROOT, "include", "parmec_coupling.h")) as f:
        declared = set(re.findall(r"\b(pg_parmec_\w+)\s*\(", f.read()))
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert declared and declared <= exported


def test_deck_through_the_c_interface(program):
    """init, input, body forces, declare_analytical, particle state, reset (no DEM: no GPU needed)."""
    out = run(program)
    assert "parnum 4" in out
    assert "inner_before -1" in out                     # no step has run
    rows = [ln.split() for ln in out.splitlines() if ln.startswith("particle ")]
    assert len(rows) == 4
    assert float(rows[2][4]) == pytest.approx(0.0125)   # z of the third sphere, as the deck placed it


@pytest.mark.gpu
def test_dem_through_the_c_interface_bitwise(program, gpu_lib, oracle_lib):
    """Two DEM calls through pg_parmec_dem on the GPU against the oracle
    running the same deck with the same body force."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300 import parmec
    out = run(program, "r")
    rows = {int(ln.split()[1]): [float(x) for x in ln.split()[2:]] for ln in out.splitlines()
            if ln.startswith("particle ")}
    inner = [[float(x) for x in ln.split()[1:]] for ln in out.splitlines() if ln.startswith("inner ")]
    parmec.RESET()
    parmec.run_deck(program[1], [])
    m = parmec.model()
    m.set_body_force(1, (0.0, 0.0, 0.5), (0.0, 0.0, 1e-4))
    eng = OracleEngine()
    dt = 1e-5
    got_inner = []
    for _ in range(2):
        m.dem(50 * dt, dt, interval=(1e9, 1e9), engine=eng)
        f, t = m.body_force_inner(1)
        got_inner.append(list(f) + list(t))
    assert np.array_equal(np.array(inner), np.array(got_inner))
    for k in range(m.parnum):
        want = list(m.P.position[0:3, k]) + list(m.P.linear[:, k]) + list(m.P.angular[3:6, k])
        assert rows[k] == want, k
    parmec.RESET()
