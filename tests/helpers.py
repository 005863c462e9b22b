"""Shared helpers of the test suite."""
import numpy as np

STATE = ("position", "linear", "angular", "rotation", "force", "torque")


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def assert_bitwise(ma, mb, names=STATE, where=""):
    """Particle state arrays equal bit for bit."""
    for name in names:
        a = getattr(ma.P, name)[..., :ma.parnum]
        b = getattr(mb.P, name)[..., :mb.parnum]
        if not np.array_equal(bits(a), bits(b)):
            diff = np.max(np.abs(a - b))
            bad = int(np.sum(bits(a) != bits(b)))
            raise AssertionError(f"{where}{name}: {bad} words differ, max abs diff {diff:.3e}")


def assert_spheres_bitwise(ma, mb):
    a = ma.E.center[0:3, :ma.ellnum]
    b = mb.E.center[0:3, :mb.ellnum]
    assert np.array_equal(bits(a), bits(b)), f"sphere centres differ (max {np.max(np.abs(a - b)):.3e})"


def assert_contacts_equal(ca, cb):
    """Same contact set in the same canonical order, bitwise equal records."""
    assert len(ca["mpart"]) == len(cb["mpart"]), f"contact counts {len(ca['mpart'])} vs {len(cb['mpart'])}"
    assert np.array_equal(ca["mpart"], cb["mpart"])
    assert np.array_equal(ca["code"], cb["code"])
    for k in ("force", "state", "point"):
        assert np.array_equal(bits(ca[k]), bits(cb[k])), f"contact {k} differs"


def make_collision_scene(n_side=5, seed=7, spacing=0.034, speed=0.5, moving=False, friction=0.5):
    """A dense jittered lattice in a box with fast random velocities and spins:
    many contacts form and break within tens of steps."""
    from parmec_gb300.scenes import box_triangles, critical_step
    from parmec_gb300.model import Model
    rng = np.random.default_rng(seed)
    m = Model()
    mat = m.material(2500.0, 1e9, 0.25)
    n = n_side ** 3
    g = np.stack(np.meshgrid(*(np.arange(n_side),) * 3, indexing="ij"), -1).reshape(-1, 3)[:, ::-1]
    centers = 0.1 + g * spacing + rng.uniform(-0.004, 0.004, size=(n, 3))
    radii = rng.uniform(0.012, 0.02, size=n)
    m.spheres(centers, radii, mat, 1)
    m.P.linear[:, :n] = rng.normal(0.0, speed, size=(3, n))
    for i in range(n):
        m.velocity(i, angular=tuple(rng.normal(0.0, 5.0, size=3)))
    hi = 0.2 + n_side * spacing
    if moving:
        m.obstacle(box_triangles((0.0, 0.0, 0.0), (hi, hi, hi)), 2, point=(0.5 * hi, 0.5 * hi, 0.5 * hi),
                   linear=lambda t: (0.0, 0.0, 0.3), angular=lambda t: (0.0, 2.0, 1.0))
    else:
        m.obstacle(box_triangles((0.0, 0.0, 0.0), (hi, hi, hi)), 2)
    m.granular(0, 0, 1e6, 0.2, friction)
    m.set_gravity(0.0, 0.0, -9.81)
    dt = 0.1 * critical_step(1e6, (4.0 / 3.0) * np.pi * 0.012 ** 3 * 2500.0, 0.2)
    return m, dt
