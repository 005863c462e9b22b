"""The library interface of parmec (parmec.h:291-310) over this package, for
callers that link a C library instead of running a deck: coupling codes that
drive the DEM from their own time loop (pg_coupling.cpp exports these as C
functions; include/parmec_coupling.h declares them).

The commands act on the process-wide Model of parmec_gb300.parmec, as the
reference's globals do, and DEM runs on the GPU session.
"""
from . import parmec as _commands


def init():
    """parmec::init (parmec.cpp:2227-2250): empty buffers and reset."""
    _commands.RESET()
    return 0


def reset():
    """parmec::reset (parmec.cpp:2253-2310)."""
    _commands.RESET()
    return 0


def input(path, argv):
    """parmec::input (parmec.h:300): interpret an input deck; 0 on success."""
    _commands.run_deck(path, list(argv))
    return 0


def dem(duration, step, interval, prefix, verbose, adaptive):
    """parmec::dem (parmec.h:303-310): interval None or (files, history);
    returns the run's wall time in seconds."""
    m = _commands.model()
    return float(m.dem(duration, step, interval, prefix, adaptive))


def declare_analytical(k):
    """declare_analytical (parmec.h:291)."""
    _commands.model().declare_analytical(k)
    return 0


def set_body_force(k, force, torque):
    """An entry of prescribed_body_forces (parmec.h:281-289): the outer force
    and torque added to particle k at every step; force None removes it."""
    _commands.model().set_body_force(k, force, torque)
    return 0


def get_body_force(k):
    """The inner force and torque of particle k at the last step (6 floats), or None."""
    v = _commands.model().body_force_inner(k)
    return None if v is None else tuple(v[0]) + tuple(v[1])


def parnum():
    return _commands.model().parnum


def particle(k):
    """Position, linear and spatial angular velocity of particle k (9 floats)."""
    m = _commands.model()
    if not (0 <= k < m.parnum):
        raise ValueError("particle index out of range")
    P = m.P
    return tuple(float(x) for x in P.position[0:3, k]) + tuple(float(x) for x in P.linear[:, k]) + \
        tuple(float(x) for x in P.angular[3:6, k])
