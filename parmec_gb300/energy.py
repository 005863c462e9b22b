"""Total mechanical energy of a scene (a diagnostic: the reference computes none).

E = sum 1/2 m |v|^2 + 1/2 Omega . (J Omega) - m g . x + sum_contacts 1/2 kn depth^2

Omega is the referential angular velocity and J the referential inertia, so
the rotational term equals 1/2 w . (L J L^T) w.  Spring energy is not
included (the sphere scenes this is used on have no springs).
"""
import numpy as np


def kinetic(m):
    P = m.P
    n = m.parnum
    mass = P.mass[:n]
    v = P.linear[:, :n]
    O = P.angular[0:3, :n]
    J = P.inertia[:, :n]
    JO = np.stack([J[0] * O[0] + J[3] * O[1] + J[6] * O[2],
                   J[1] * O[0] + J[4] * O[1] + J[7] * O[2],
                   J[2] * O[0] + J[5] * O[1] + J[8] * O[2]])
    return 0.5 * float(np.sum(mass * np.sum(v * v, axis=0))) + 0.5 * float(np.sum(O * JO))


def potential(m, gravity):
    n = m.parnum
    g = np.asarray(gravity, dtype=np.float64).reshape(3, 1)
    return -float(np.sum(m.P.mass[:n] * np.sum(g * m.P.position[0:3, :n], axis=0)))


def contact(m, contacts):
    """1/2 kn depth^2 over exported contacts (needs depths: FP64 session with recorded geometry)."""
    kn = m.iparam[0][0]
    d = contacts.get("depth")
    if d is None or len(d) == 0 or not np.all(np.isfinite(d)):
        return 0.0
    return 0.5 * kn * float(np.sum(d * d))


def total(m, gravity=None, contacts=None):
    g = m.gravity if gravity is None else gravity
    e = kinetic(m) + potential(m, g)
    if contacts is not None:
        e += contact(m, contacts)
    return e
