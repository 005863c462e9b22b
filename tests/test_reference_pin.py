"""The oracle against the reference's own ISPC hot path, on the CPU.

oracle/ispc_ref.py translates the reference's condet, forces, dynamics,
parmec, partition, restrain, shapes and obstacles .ispc mechanically into
C++ at gang size one and builds oracle/_ref/libparmec_ref.so, which exports
the reference's own entry points.  tests/ispc_loop.py drives it with
parmec.cpp's dem() call sequence (partitioning tree, linked contact lists,
spin locks and all), and the results are compared here with the oracle's on
the same seeded decks.  Since the CUDA path equals the oracle bit for bit
(the -m gpu tests), these comparisons pin the CUDA path to the reference's
source as well.

Tolerances (relative to the largest magnitude of each quantity):
  - state after the run (position, velocity, spin, rotation, force, torque):
    1e-10; most decks agree to the last bit, the rest differ by sums taken in
    another order (the reference's contact lists are in insertion order, the
    oracle's are sorted);
  - contact pairs: the same set, unless the reference's tree misses a pair
    (a pair whose centres each lie outside the other's query box);
  - per-contact forces: 1e-12 of the largest contact force.

The reference never initialises a contact's tangential friction state and
does not move it when it compacts a list, so with friction a contact created
in a reused slot starts from the state of the contact that was there.  Decks
with friction where contacts come and go therefore run against the
friction-state variant (libparmec_ref_state.so), whose two edits give that
state the oracle's definition (zero at creation, moved with the contact).
"""
import re
import os
import subprocess

import numpy as np
import pytest

from oracle import dem_loop as ispc_loop
from helpers import make_collision_scene

STATE = ("position", "linear", "angular", "rotation", "force", "torque")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ref():
    from oracle import ispc_ref
    lib = ispc_ref.build()
    if lib is None:
        pytest.skip("neither the reference's ISPC sources nor their translation are on this host")
    return {"plain": ispc_loop.library(ispc_ref.LIB), "state": ispc_loop.library(ispc_ref.LIB_STATE)}


def run_reference(lib, m, duration, step, ntasks=1, calls=1):
    host = ispc_loop.Host(lib, m, orient=True, ntasks=ntasks)
    for _ in range(calls):
        ispc_loop.dem(lib, host, duration, step)
    return host


def run_oracle(m, duration, step, threads=1, calls=1):
    from oracle.pyoracle import OracleEngine
    eng = OracleEngine(threads=threads)
    for _ in range(calls):
        m.dem(duration, step, interval=1e9, engine=eng)
    return eng


def rel_diff(mr, mo, names=STATE):
    out = {}
    n = mr.parnum
    for name in names:
        a = getattr(mr.P, name)[..., :n]
        b = getattr(mo.P, name)[..., :n]
        scale = float(np.max(np.abs(b))) or 1.0
        out[name] = float(np.max(np.abs(a - b))) / scale
    return out


def assert_close_state(mr, mo, tol=1e-10, where=""):
    d = rel_diff(mr, mo)
    bad = {k: v for k, v in d.items() if not v <= tol}
    assert not bad, f"{where}state differs from the reference beyond {tol}: {bad}"


def tree_miss(m, a, b):
    """True when neither sphere centre lies inside the other sphere's query
    box [c - r, c + r], the only case in which the reference's partitioning
    tree can miss a touching pair (condet.ispc:279-283, partition.ispc:604-609)."""
    ca, cb = m.E.center[0:3, a], m.E.center[0:3, b]
    ra, rb = m.E.radii[0, a], m.E.radii[0, b]
    inside_a = np.all(np.abs(cb - ca) <= ra)
    inside_b = np.all(np.abs(ca - cb) <= rb)
    return not (inside_a or inside_b)


def compare_contacts(host, eng, m):
    """Reference master lists against the oracle's contacts: the same pair
    set (modulo tree misses) and the same forces."""
    r = ispc_loop.master_lists(host)
    o = eng.contacts()
    rk = {(int(p), int(c)): k for k, (p, c) in enumerate(zip(r["mpart"], r["code"]))}
    ok = {(int(p), int(c)): k for k, (p, c) in enumerate(zip(o["mpart"], o["code"]))}
    assert len(rk) == len(r["mpart"]), "duplicate contact in the reference's lists"
    extra = set(rk) - set(ok)
    assert not extra, f"the reference holds contacts the oracle does not: {sorted(extra)[:5]}"
    missing = set(ok) - set(rk)
    for (p, c) in missing:
        sphere = [j for j in range(m.ellnum) if m.E.part[j] == p]
        assert c >= 0 and sphere and tree_miss(m, sphere[0], c), \
            f"oracle contact ({p}, {c}) is not in the reference's lists and is not a tree miss"
    common = sorted(set(rk) & set(ok))
    fr = np.array([r["force"][rk[k]] for k in common]).reshape(-1, 3)
    fo = np.array([o["force"][ok[k]] for k in common]).reshape(-1, 3)
    if len(common):
        scale = float(np.max(np.abs(fo))) or 1.0
        assert float(np.max(np.abs(fr - fo))) <= 1e-12 * scale
    return len(common), len(missing)


def test_reference_exports_are_declared_by_the_dropin_header(ref):
    """Every entry point the reference's ISPC objects export is declared by
    include/parmec_ispc.h, so an unmodified parmec.cpp and input.cpp link
    against libparmec_gb300.so."""
    from oracle import ispc_ref
    nm = subprocess.run(["nm", "-D", "--defined-only", ispc_ref.LIB], capture_output=True, text=True, check=True)
    exports = {ln.split()[-1] for ln in nm.stdout.splitlines() if " T " in ln}
    exports = {e for e in exports if not e.startswith("_")}
    with open(os.path.join(ROOT, "include", "parmec_ispc.h")) as f:
        header = f.read()
    declared = set(re.findall(r"\b(\w+)\s*\(", re.sub(r"/\*.*?\*/", "", header, flags=re.S)))
    assert exports, "no exports found"
    missing = sorted(exports - declared)
    assert not missing, f"reference exports missing from include/parmec_ispc.h: {missing}"


def test_hopper_fill_full_deck_matches_reference(ref):
    """The CPU-runnable configuration at its stated size: 4,096 spheres,
    friction 0.5, 1,000 steps (its initial overlaps open and close, so the
    friction-state variant)."""
    from parmec_gb300.scenes import hopper_fill
    mr, dt = hopper_fill()
    mo, _ = hopper_fill()
    run_reference(ref["state"], mr, 1000 * dt - 0.5 * dt, dt)
    run_oracle(mo, 1000 * dt - 0.5 * dt, dt, threads=4)
    assert_close_state(mr, mo)


def test_collisions_without_friction_match_reference(ref):
    """216 fast spinning spheres in a box, 400 steps: contacts form and break
    all the time; the reference as written."""
    mr, dt = make_collision_scene(n_side=6, friction=0.0)
    mo, _ = make_collision_scene(n_side=6, friction=0.0)
    host = run_reference(ref["plain"], mr, 400 * dt - 0.5 * dt, dt)
    eng = run_oracle(mo, 400 * dt - 0.5 * dt, dt)
    assert_close_state(mr, mo)
    compare_contacts(host, eng, mo)


def test_collisions_with_friction_match_reference_before_slots_are_reused(ref):
    """With friction, the reference as written agrees while no contact has
    been created in a slot that another contact left."""
    mr, dt = make_collision_scene(n_side=5, friction=0.5)
    mo, _ = make_collision_scene(n_side=5, friction=0.5)
    run_reference(ref["plain"], mr, 5 * dt - 0.5 * dt, dt)
    run_oracle(mo, 5 * dt - 0.5 * dt, dt)
    assert_close_state(mr, mo, tol=1e-12)


def test_collisions_with_friction_match_reference_state_variant(ref):
    """The same collisions with friction over 400 steps and two DEM calls,
    against the friction-state variant."""
    mr, dt = make_collision_scene(n_side=5, friction=0.5)
    mo, _ = make_collision_scene(n_side=5, friction=0.5)
    host = run_reference(ref["state"], mr, 200 * dt - 0.5 * dt, dt, calls=2)
    eng = run_oracle(mo, 200 * dt - 0.5 * dt, dt, calls=2)
    assert_close_state(mr, mo)
    compare_contacts(host, eng, mo)


def test_rotating_drum_matches_reference(ref):
    """16,384 spheres of the drum deck (radii log-uniform in [0.5, 2] mm, a
    4,096-triangle cylinder turning at 2 rad/s, friction 0.3), 50 steps,
    with the reference's moving-obstacle indexing (PG_COMPAT_OBSIDX) on both
    sides: the state, the moved triangles, every contact pair and force."""
    from parmec_gb300 import abi
    from parmec_gb300.scenes import drum

    def make():
        m, dt, _ = drum(16384)
        m.compat |= abi.PG_COMPAT_OBSIDX
        return m, dt
    mr, dt = make()
    mo, _ = make()
    host = run_reference(ref["state"], mr, 50 * dt - 0.5 * dt, dt)
    eng = run_oracle(mo, 50 * dt - 0.5 * dt, dt, threads=4)
    assert_close_state(mr, mo, tol=1e-12)
    t = mr.Tr.tri[:, :mr.trinum] - mo.Tr.tri[:, :mo.trinum]
    assert float(np.max(np.abs(t))) == 0.0
    n, _ = compare_contacts(host, eng, mo)
    assert n > 10000


def test_rotating_drum_matches_reference_with_parallel_tasks(ref):
    """The reference's tasks spread over threads (the schedule its CPU
    baseline runs): list order changes with the schedule, so sums differ in
    the last bits only."""
    from parmec_gb300 import abi
    from parmec_gb300.scenes import drum

    def make():
        m, dt, _ = drum(8192)
        m.compat |= abi.PG_COMPAT_OBSIDX
        return m, dt
    mr, dt = make()
    mo, _ = make()
    run_reference(ref["state"], mr, 30 * dt - 0.5 * dt, dt, ntasks=8)
    run_oracle(mo, 30 * dt - 0.5 * dt, dt, threads=4)
    assert_close_state(mr, mo, tol=1e-12)


def test_spring_lattice_matches_reference(ref):
    """Bodies with full inertia tensors on springs of every direction mode,
    nonlinear curves, dashpots, a TSERIES stroke offset and a prescribed
    base, 200 steps and a second DEM call."""
    from test_gpu_springs import lattice
    step = 2e-5
    mr, mo = lattice(), lattice()
    run_reference(ref["plain"], mr, 200 * step, step, calls=2)
    run_oracle(mo, 200 * step, step, calls=2)
    assert_close_state(mr, mo)


def test_mesh_spring_lattice_matches_reference(ref):
    """The spring-lattice deck's construction (hexahedral MESH particles,
    8-point curves, lookup dashpots, a base plate driven by PRESCRIBE) on a
    12 x 12 grid, 100 steps: mesh nodes and triangles follow the bodies."""
    from parmec_gb300.scenes import spring_lattice
    mr, dt = spring_lattice(12)
    mo, _ = spring_lattice(12)
    run_reference(ref["plain"], mr, 100 * dt - 0.5 * dt, dt)
    run_oracle(mo, 100 * dt - 0.5 * dt, dt)
    assert_close_state(mr, mo)
    t = mr.Tr.tri[:, :mr.trinum] - mo.Tr.tri[:, :mo.trinum]
    assert float(np.max(np.abs(t))) <= 1e-12 * float(np.max(np.abs(mo.Tr.tri[:, :mo.trinum])))


def test_torsion_springs_match_reference(ref):
    """TORSION_SPRING decks (one and two cubes, every stiffness/damper kind
    and cone) against the reference as written.  The pitch-yaw cone is left
    out: there the reference's pitch damper reads the roll ratio entry
    (forces.ispc:1823), which the oracle fixes."""
    from test_torsion import GPU_CASES, one
    for case, two, extra in GPU_CASES:
        if extra.get("cone") == ("pitch", "yaw"):
            continue
        mr, *_ = one(case, two, **extra)
        mo, *_ = one(case, two, **extra)
        run_reference(ref["plain"], mr, 0.3, 1e-3)
        run_oracle(mo, 0.3, 1e-3)
        assert_close_state(mr, mo, where=f"torsion case {case} {two} {extra}: ")
        for name in ("rpy", "rpytot", "rpyspr"):
            a, b = getattr(mr.Q, name)[:, :mr.trqsprnum], getattr(mo.Q, name)[:, :mo.trqsprnum]
            assert float(np.max(np.abs(a - b))) <= 1e-10 * (float(np.max(np.abs(b))) or 1.0), name


def test_unspring_rules_match_reference(ref):
    """UNSPRING countdowns, failure, activation and unload curves over eight
    DEM calls."""
    from test_unspring import hanging
    for kw in ({}, {"nfreq": 1, "unload": [0.0, 0.0, 1.0, 1e5]}, {"entity": "F", "operator": "MAX"}):
        mr, *_ = hanging(**kw)
        mo, *_ = hanging(**kw)
        run_reference(ref["plain"], mr, 2e-3, 1e-4, calls=8)
        run_oracle(mo, 2e-3, 1e-4, calls=8)
        assert list(mr.S.unspring[:mr.sprnum]) == list(mo.S.unspring[:mo.sprnum])
        assert_close_state(mr, mo, where=f"unspring {kw}: ")


def test_restraints_match_reference(ref):
    """RESTRAIN rows on colliding spheres over two DEM calls."""
    def make():
        m, dt = make_collision_scene(n_side=4)
        m.restrain(0, linear=[0.0, 0.0, 1.0])
        m.restrain(3, linear=[1.0, 1.0, 0.0, 0.0, 1.0, 1.0], angular=[0.0, 0.0, 1.0])
        m.restrain(3, angular=[1.0, 0.0, 0.0])
        m.restrain(7, angular=[1.0, 0.2, 0.0, 0.0, 1.0, 0.3, 0.1, 0.0, 1.0])
        return m, dt
    mr, dt = make()
    mo, _ = make()
    run_reference(ref["state"], mr, 25 * dt, dt, calls=2)
    run_oracle(mo, 25 * dt, dt, calls=2)
    assert_close_state(mr, mo)


def test_adaptive_steps_match_reference(ref):
    """forces(adaptive) + adaptive_timestep on colliding spheres: the chosen
    steps and the state.  The oracle fixes two adaptive defects (slave
    contacts read kcur/ecur that nothing sets, forces.ispc:554-557; the
    k-end spring arm rotated with the j particle, forces.ispc:1341); on this
    deck they move the chosen step by about 1e-11 relative."""
    from oracle.pyoracle import OracleEngine
    mr, dt = make_collision_scene(n_side=4)
    mo, _ = make_collision_scene(n_side=4)
    host = ispc_loop.Host(ref["state"], mr, orient=True)
    ispc_loop.dem(ref["state"], host, 40 * dt, dt, adaptive=0.6)
    mo.dem(40 * dt, dt, interval=1e9, adaptive=0.6, engine=OracleEngine())
    assert mr.curstep != dt
    assert abs(mr.curstep - mo.curstep) <= 1e-9 * mo.curstep
    assert_close_state(mr, mo, tol=1e-9)


def spheres_on_a_plane(n_side=6):
    """n_side^2 spheres resting apart on a plane: every contact a sphere
    masters (no slave records), normals along z."""
    from parmec_gb300.model import Model
    from parmec_gb300.scenes import critical_step
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    rng = np.random.default_rng(5)
    for i in range(n_side):
        for j in range(n_side):
            r = float(rng.uniform(0.01, 0.015))
            mass = (4.0 / 3.0) * np.pi * r ** 3 * 2500.0
            m.sphere((0.05 * i, 0.05 * j, r - mass * 9.81 / 1e6), r, mat, 1)   # the static overlap
    L = 1.0
    m.obstacle([(-L, -L, 0.0, L, -L, 0.0, L, L, 0.0), (-L, -L, 0.0, L, L, 0.0, -L, L, 0.0)], 2)
    m.granular(0, 0, 1e6, 0.2, 0.5)
    m.set_gravity(0.0, 0.0, -9.81)
    return m, 0.1 * critical_step(1e6, (4.0 / 3.0) * np.pi * 0.01 ** 3 * 2500.0, 0.2)


def test_critical_restatement_matches_reference(ref):
    """CRITICAL's host restatement (the checker of the device's) against the
    reference's critical_perparticle and critical_perspring: spheres on a
    plane (contact terms) and the MESH spring lattice (spring terms; its
    springs share one direction mode and lookup dashpots, so the reference's
    sprflg/dashidx indexing by particle reads the same kind)."""
    from oracle.critical_host import critical_perparticle, critical_perspring
    from parmec_gb300.scenes import spring_lattice
    for make, steps in ((spheres_on_a_plane, 30), (lambda: spring_lattice(12), 20)):
        mr, dt = make()
        mo, _ = make()
        host = run_reference(ref["plain"], mr, steps * dt - 0.5 * dt, dt)
        eng = run_oracle(mo, steps * dt - 0.5 * dt, dt)
        (hs, os_, rs), (hp, op, rp) = ispc_loop.critical(ref["plain"], host)
        h, o, r = critical_perparticle(mo, eng.contacts())
        touched = hp < 1e300
        assert touched.sum() >= 20
        assert np.array_equal(touched, h < 1e300)
        # rotational frequencies are eigenvalues of nearly double-rooted 3x3
        # matrices (one contact arm: rank two), where the reference's
        # acos/cos and the restatement's Newton root differ by ~sqrt(eps)
        # of the conditioning: 1e-7 relative
        for a, b in ((hp, h), (op, o), (rp, r)):
            assert np.allclose(a[touched], b[touched], rtol=1e-7, atol=0.0)
        if mo.sprnum:
            h2, o2, r2 = critical_perspring(mo)
            for a, b in ((hs, h2), (os_, o2), (rs, r2)):
                assert np.allclose(a, np.array(b), rtol=1e-10, atol=0.0)
