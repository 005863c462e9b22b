"""ctypes mirror of include/parmec_gb300.h (pg_scene, pg_steptab) and the loader
of libparmec_gb300.so.

The structures here must match the C header field for field; tests/test_abi.py
checks the sizes and that every symbol the header declares is exported.
"""
import ctypes
import os

import numpy as np

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)

NIPARAM = 7

PG_OK = 0
PG_ERR_CUDA = -1
PG_ERR_CAPACITY = -2
PG_ERR_ARGUMENT = -3
PG_ERR_UNSUPPORTED = -4
PG_ERR_TIMEOUT = -5

PG_COMPAT_EXPMAP = 1
PG_COMPAT_OBSIDX = 2
PG_COMPAT_TRIEDGE = 4

PG_FORM_FP64 = 0
PG_FORM_MIXED = 1

_ERRORS = {
    PG_ERR_CUDA: "CUDA runtime error",
    PG_ERR_CAPACITY: "per-particle list capacity exceeded",
    PG_ERR_ARGUMENT: "invalid argument",
    PG_ERR_UNSUPPORTED: "unsupported case (the reference asserts here)",
    PG_ERR_TIMEOUT: "bounded device wait gave up",
}


class PgScene(ctypes.Structure):
    """pg_scene (include/parmec_gb300.h)."""
    _fields_ = [
        ("parnum", ctypes.c_int),
        ("angular", D * 6), ("linear", D * 3), ("rotation", D * 9), ("position", D * 6),
        ("inertia", D * 9), ("inverse", D * 9), ("mass", D), ("invm", D),
        ("force", D * 3), ("torque", D * 3), ("flags", I), ("parmat", I),
        ("ellnum", ctypes.c_int),
        ("center", D * 6), ("radii", D * 3), ("ellcol", I), ("part", I),
        ("trinum", ctypes.c_int),
        ("tri", (D * 3) * 3), ("tricol", I), ("triobs", I),
        ("obsnum", ctypes.c_int),
        ("trirng", I), ("obspnt", D), ("obsang", D), ("obslin", D),
        ("pairnum", ctypes.c_int),
        ("pairs", I), ("ikind", I), ("iparam", D * NIPARAM),
        ("nodnum", ctypes.c_int),
        ("nodes", D * 6), ("nodpart", I),
        ("facnum", ctypes.c_int),
        ("facnod", I * 3), ("factri", I),
        ("sprnum", ctypes.c_int),
        ("sprtype", I), ("unspring", I), ("sprpart", I * 2), ("sprpnt", (D * 6) * 2),
        ("spring", D * 2), ("spridx", I), ("dashpot", D * 2), ("dashidx", I),
        ("unload", D * 2), ("unidx", I), ("yield_", D * 2), ("sprdir", D * 6),
        ("sprflg", I), ("sproffset", I), ("sprfric", D), ("sprkskn", D),
        ("sprsdsp", D * 3), ("stroke0", D), ("stroke", D * 3), ("sprfrc", D * 3),
        ("lcurve", D * 2), ("lcidx", I),
        ("prsnum", ctypes.c_int),
        ("prspart", I), ("prslin", I), ("prsang", I), ("linkind", I), ("angkind", I),
        ("compat", ctypes.c_int),
        ("nscene", ctypes.c_int),
        ("pscene", I), ("tscene", I), ("oscene", I), ("sactive", I),
        ("rstnum", ctypes.c_int),
        ("rstpart", I), ("rstlin", D * 9), ("rstang", D * 9),
        ("unsprnum", ctypes.c_int),
        ("tsprings", I), ("tspridx", I), ("msprings", I), ("mspridx", I), ("activate", I), ("actidx", I),
        ("unlim", D * 2), ("unent", I), ("unop", I), ("unabs", I), ("nsteps", I), ("nfreq", I),
        ("unaction", I), ("sprmap", I),
        ("trqsprnum", ctypes.c_int),
        ("trqsprpart", I * 2), ("trqzdir0", D * 3), ("trqxdir0", D * 3),
        ("krpy", (D * 2) * 3), ("krpyidx", I * 3), ("drpy", (D * 2) * 3), ("drpyidx", I * 3),
        ("trqcone", I), ("trqzdir1", D * 3), ("trqxdir1", D * 3),
        ("trqrpy", D * 3), ("trqrpytot", D * 3), ("trqrpyspr", D * 3),
        ("pbfnum", ctypes.c_int), ("pbfpart", I), ("pbfout", D * 6), ("pbfin", D * 6),
    ]


class PgStepTab(ctypes.Structure):
    """pg_steptab (include/parmec_gb300.h)."""
    _fields_ = [
        ("nsteps", ctypes.c_int),
        ("curtime", D), ("gravity", D), ("damping", D),
        ("prs_lin", D), ("prs_ang", D), ("obs_ang", D), ("obs_lin", D),
        ("stepnum", ctypes.c_int),
    ]


def dptr(a):
    """double* to a C-contiguous float64 array (or NULL)."""
    if a is None:
        return D()
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def iptr(a):
    """int* to a C-contiguous int32 array (or NULL)."""
    if a is None:
        return I()
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(I)


def rows(arr, n, ptype=D):
    """Array of per-component pointers of a (ncomp, cap) array."""
    out = (ptype * n)()
    for k in range(n):
        row = arr[k]
        assert row.flags.c_contiguous
        out[k] = row.ctypes.data_as(ptype)
    return out


def check(status, what="call"):
    """Raise RuntimeError for a negative pg_* status."""
    if status != PG_OK:
        raise RuntimeError(f"parmec_gb300: {what} failed: {_ERRORS.get(status, status)} ({status})")
    return status


_LIB = None


def library_path():
    here = os.path.dirname(os.path.abspath(__file__))
    return os.path.join(here, "_build", "libparmec_gb300.so")


def load_library():
    """Load libparmec_gb300.so (built in-tree by parmec_gb300.build).

    There is no CPU fallback: a missing library is an error.
    """
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"parmec_gb300: CUDA library {path} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    sig = {
        "pg_session_create": (ctypes.c_int, [ctypes.POINTER(PgScene), ctypes.c_int, ctypes.POINTER(P)]),
        "pg_session_destroy": (ctypes.c_int, [P]),
        "pg_session_first_half_step": (ctypes.c_int, [P, ctypes.c_double, D, D]),
        "pg_session_invert_inertia": (ctypes.c_int, [P]),
        "pg_session_run": (ctypes.c_int, [P, ctypes.POINTER(PgStepTab), ctypes.c_double]),
        "pg_session_run_async": (ctypes.c_int, [P, ctypes.POINTER(PgStepTab), ctypes.c_double]),
        "pg_session_run_adaptive": (ctypes.c_int, [P, ctypes.POINTER(PgStepTab), ctypes.c_double, ctypes.c_double, D]),
        "pg_session_restrain_velocities": (ctypes.c_int, [P]),
        "pg_session_critical": (ctypes.c_int, [P, ctypes.c_int, D, D, D]),
        "pg_session_mesh_contact": (ctypes.c_int, [P, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
        "pg_session_mesh_contact_stats": (ctypes.c_int, [P, I, I]),
        "pg_session_set_live": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "pg_session_download_particles": (ctypes.c_int, [P, ctypes.POINTER(PgScene), I, ctypes.c_int]),
        "pg_session_download_springs": (ctypes.c_int, [P, ctypes.POINTER(PgScene), I, ctypes.c_int]),
        "pg_session_sync": (ctypes.c_int, [P]),
        "pg_session_download": (ctypes.c_int, [P, ctypes.POINTER(PgScene)]),
        "pg_session_upload": (ctypes.c_int, [P, ctypes.POINTER(PgScene)]),
        "pg_session_contact_count": (ctypes.c_int, [P, I]),
        "pg_session_contacts": (ctypes.c_int, [P, ctypes.c_int, I, I, I, D, D, D, D, D]),
        "pg_session_stream": (ctypes.c_int, [P, ctypes.POINTER(P)]),
        "pg_session_kernel_launches": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_longlong)]),
        "pg_session_set_skin": (ctypes.c_int, [P, ctypes.c_double]),
        "pg_session_record_geometry": (ctypes.c_int, [P, ctypes.c_int]),
        "pg_session_profile": (ctypes.c_int, [P, ctypes.c_int]),
        "pg_session_set_grid": (ctypes.c_int, [P, ctypes.c_double, I]),
        "pg_session_set_capacity": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "pg_session_scene": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, D, D, ctypes.c_longlong]),
        "pg_session_upload_range": (ctypes.c_int, [P, ctypes.POINTER(PgScene), I]),
        "pg_session_download_range": (ctypes.c_int, [P, ctypes.POINTER(PgScene), I]),
        "pg_session_download_range_motion": (ctypes.c_int, [P, ctypes.POINTER(PgScene), I]),
        "pg_session_release_range": (ctypes.c_int, [P, I]),
        "pg_session_global_step": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_longlong)]),
        "pg_session_use_graph": (ctypes.c_int, [P, ctypes.c_int]),
        "pg_session_use_fused": (ctypes.c_int, [P, ctypes.c_int]),
        "pg_session_autotune": (ctypes.c_int, [P, ctypes.c_int]),
        "pg_session_fused_config": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int)]),
        "pg_session_barrier_selftest": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_double)]),
        "pg_host_register": (ctypes.c_int, [P, ctypes.c_size_t]),
        "pg_host_unregister": (ctypes.c_int, [P]),
        "pg_session_profile_read": (ctypes.c_int, [P, D, ctypes.POINTER(ctypes.c_longlong)]),
        "pg_session_diagnostics": (ctypes.c_int, [P, I]),
        "pg_cell_order": (ctypes.c_int, [P, P, P, ctypes.c_int, D, ctypes.c_double, I, P, P, P]),
        "pg_cell_order_static": (ctypes.c_int, [P, P, P, ctypes.c_int, D, ctypes.c_double, I, P, P, P]),
        "pg_version": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib
