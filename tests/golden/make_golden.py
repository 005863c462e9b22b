"""Generates the golden fixtures of this directory.

The reference (parmes/parmec) cannot be built here: its kernels are ISPC
sources and its output needs HDF5, and neither `ispc` nor HDF5 is installed.
Its own self-checking decks give two numeric pins (tests/damping.py: the
projectile's final x of 86.138 in within 0.5 %; tests/spring_curve_tests.py:
recorded stroke-force pairs within 0.1*h of the input curve), which
`reference_decks.json` records with their tolerances.

Every other fixture is the CPU oracle's output (oracle/oracle.cpp, the
statement-by-statement restatement of the reference's FP64 path) on small
seeded scenes, stored bit for bit (the drum as SHA-256 digests of each
array's bytes, to keep the files small):

  hopper216   216 spheres in a 12-triangle box (the hopper-fill deck at a
              smaller side), 100 steps;
  drum4096    4,096 spheres in the rotating 4,096-triangle drum, 60 steps;
  lattice8    8 x 8 MESH cubes on nonlinear SPRINGs with a PRESCRIBEd base
              plate, 60 steps;
  damping     the projectile deck's sampled x history.

They pin the oracle against regressions (tests/test_golden.py runs it again
on the CPU and compares bits) and give the GPU path a second, stored target
that does not depend on the oracle's build on the GPU host.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

STATE = ("position", "linear", "angular", "rotation", "force", "torque")


def hopper216():
    from parmec_gb300.scenes import hopper_fill
    m, dt = hopper_fill(n_side=6, seed=3, spacing=0.036)
    return m, dt, 100


def drum4096():
    from parmec_gb300.scenes import drum
    m, dt, _ = drum(4096, seed=1)
    return m, dt, 60


def lattice8():
    from parmec_gb300.scenes import spring_lattice
    m, dt = spring_lattice(n_side=8, seed=2)
    return m, dt, 60


CASES = {"hopper216": hopper216, "drum4096": drum4096, "lattice8": lattice8}
DIGEST_ONLY = ("drum4096",)


def digest(a):
    import hashlib
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def run_case(name, engine):
    """Runs one case on `engine`; returns (model, arrays to compare)."""
    m, dt, steps = CASES[name]()
    m.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=engine)
    out = {}
    for k in STATE:
        out[k] = np.ascontiguousarray(getattr(m.P, k)[..., :m.parnum])
    if m.ellnum:
        out["center"] = np.ascontiguousarray(m.E.center[0:3, :m.ellnum])
    if m.trinum:
        out["tri"] = np.ascontiguousarray(m.Tr.tri[:, :m.trinum])
    c = engine.contacts()
    for k in ("mpart", "code", "point", "force", "state"):
        out["contact_" + k] = np.ascontiguousarray(c[k])
    out["curtime"] = np.array([m.curtime])
    return m, out


def damping_history(engine):
    """The reference's projectile deck (tests/damping.py:4-37): a point mass
    thrown at (2.54, 0, 12.7) m/s under linear global damping."""
    from parmec_gb300.model import Model
    m = Model()
    stop = 1.976
    step = stop / 1024.0
    num = m.analytical([1, 1, 1, 0, 0, 0], 0.45359237, position=(0, 0, 0))
    m.velocity(num, (2.54, 0, 12.7), (0, 0, 0))
    m.set_damping(lambda t: (1, 1, 1), lambda t: (0, 0, 0))
    m.set_gravity(0., 0., -9.81456)
    X = m.history('PX', num)
    m.dem(stop, step, (64 * step, step), engine=engine)
    return np.asarray(X, dtype=np.float64)


def main():
    from oracle import pyoracle
    from oracle.pyoracle import OracleEngine
    pyoracle.build()
    digests = {}
    for name in CASES:
        _, out = run_case(name, OracleEngine())
        digests[name] = {k: [list(v.shape), digest(v)] for k, v in out.items()}
        if name not in DIGEST_ONLY:
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(digests, f, indent=1)
    x = damping_history(OracleEngine())
    np.savez_compressed(os.path.join(HERE, "damping.npz"), x=x)
    decks = {
        "damping": {"source": "tests/damping.py:4-37", "quantity": "final x / 0.0254 (in)",
                    "expected": 86.138, "rel_tol": 0.005},
        "spring_curves": {"source": "tests/spring_curve_tests.py:14-63",
                          "quantity": "|input curve(w) - recorded curve(w)| on w in [-1, x_end - h) step h",
                          "h": 0.02, "abs_tol": "0.1*h", "cases": 12},
    }
    with open(os.path.join(HERE, "reference_decks.json"), "w") as f:
        json.dump(decks, f, indent=1)
    print("damping final x (in):", x[-1] / 0.0254)


if __name__ == "__main__":
    main()
