"""The C ABI: ctypes mirrors match the header's layout, and the library
exports every function include/parmec_gb300.h declares (CPU only: nothing is
computed)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "parmec_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(pg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_session_api():
    names = declared_functions()
    for n in ("pg_session_create", "pg_session_run", "pg_session_download", "pg_cell_order", "pg_version"):
        assert n in names


def test_library_exports_every_declared_symbol():
    import __graft_entry__
    __graft_entry__.build()
    from parmec_gb300 import abi
    lib = abi.load_library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", abi.library_path()], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    assert not [n for n in declared_functions() if n not in exported]
    assert lib.pg_version().decode().startswith("parmec_gb300")


def c_layout(tmp_path):
    src = tmp_path / "layout.c"
    fields = ["parnum", "angular", "mass", "ellnum", "center", "trinum", "tri", "obsnum", "obslin", "pairnum",
              "iparam", "nodnum", "facnum", "factri", "sprnum", "sprpnt", "lcidx", "prsnum", "angkind", "compat"]
    body = "".join(f'  printf("{f} %zu\\n", offsetof(pg_scene, {f}));\n' for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "parmec_gb300.h"\nint main(void){\n'
                   '  printf("size %zu\\n", sizeof(pg_scene));\n  printf("tabsize %zu\\n", sizeof(pg_steptab));\n'
                   + body + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return {l.split()[0]: int(l.split()[1]) for l in out.splitlines()}


def test_ctypes_scene_layout_matches_c(tmp_path):
    from parmec_gb300 import abi
    lay = c_layout(tmp_path)
    assert lay["size"] == ctypes.sizeof(abi.PgScene)
    assert lay["tabsize"] == ctypes.sizeof(abi.PgStepTab)
    for name, off in lay.items():
        if name in ("size", "tabsize"):
            continue
        assert getattr(abi.PgScene, name).offset == off, name


def test_session_create_without_gpu_fails_loudly():
    """No CPU fallback: without a device the session cannot be created."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import hopper_fill
    m, dt = hopper_fill(n_side=2)
    with pytest.raises(RuntimeError):
        m.dem(dt, dt, engine=GpuEngine())


# ---------------------------------------------------------------- drop-in ISPC surface
ISPC_HEADER = os.path.join(ROOT, "include", "parmec_ispc.h")


def ispc_functions():
    text = open(ISPC_HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"#.*", "", text)
    return sorted(set(re.findall(r"(?:^|;|\})\s*(?:struct\s+)?\w+\s*\*?\s*(\w+)\s*\(", text)))


def test_ispc_header_declares_the_reference_exports():
    names = ispc_functions()
    for n in ("condet", "forces", "dynamics", "euler", "invert_inertia", "shapes", "obstacles",
              "partitioning_create", "partitioning_store", "partitioning_destroy", "master_alloc", "master_free",
              "slave_alloc", "slave_free", "aligned_real_alloc", "aligned_int_alloc", "ispc_num_cores"):
        assert n in names, n


def test_library_exports_every_ispc_symbol():
    from parmec_gb300 import abi
    out = subprocess.run(["nm", "-D", "--defined-only", abi.library_path()], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    assert not [n for n in ispc_functions() if n not in exported]


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_ispc_header_compiles(tmp_path, lang):
    """parmec.cpp includes the header as C++ (namespace ispc); C hosts can use it too."""
    src = tmp_path / ("use.cpp" if lang == "c++" else "use.c")
    pre = "using namespace ispc;\n" if lang == "c++" else ""
    src.write_text('#include "parmec_ispc.h"\n' + pre +
                   "int main(void){ return (int)sizeof(struct master_conpnt) - 1464 + "
                   "(int)sizeof(struct slave_conpnt) - 600; }\n")
    exe = tmp_path / "use"
    cc = "g++" if lang == "c++" else "gcc"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    assert subprocess.run([str(exe)]).returncode == 0


def test_ispc_host_side_functions_without_gpu():
    """Allocation, grid handles and the empty restraint call need no device."""
    from parmec_gb300 import abi
    lib = abi.load_library()
    lib.aligned_real_alloc.restype = ctypes.POINTER(ctypes.c_double)
    lib.partitioning_create.restype = ctypes.c_void_p
    lib.master_alloc.restype = ctypes.c_void_p
    lib.master_alloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.master_free.argtypes = [ctypes.c_void_p, ctypes.c_int]
    p = lib.aligned_real_alloc(1000)
    assert all(p[i] == 0.0 for i in range(1000))
    lib.aligned_real_free(p)
    assert lib.ispc_num_cores() >= 1
    assert lib.partitioning_create(1, 0, None) is None
    t = lib.partitioning_create(1, 10, None)
    assert t and lib.partitioning_store(1, ctypes.c_void_p(t), 10, None, None, None, None, None) == 0
    lib.partitioning_destroy(ctypes.c_void_p(t))
    m = lib.master_alloc(None, 0, 16)
    m2 = lib.master_alloc(m, 16, 32)
    lib.master_free(m2, 32)
    lib.pg_compat_exit_on_error(0)
    lib.restrain_forces(1, 0, None, None, None, None, None)
    assert lib.pg_compat_status() == 0
    # a restraint runs on the device: without one the call reports PG_ERR_CUDA
    import numpy as np
    part = np.zeros(1, dtype=np.int32)
    dirs = np.zeros((9, 1))
    dirs[2, 0] = 1.0
    vec = np.ones((3, 1))
    lib.restrain_forces(1, 1, abi.iptr(part), abi.rows(dirs, 9), abi.rows(np.zeros((9, 1)), 9),
                        abi.rows(vec, 3), abi.rows(vec.copy(), 3))
    st = lib.pg_compat_status()
    assert st in (abi.PG_OK, abi.PG_ERR_CUDA)
    if st == abi.PG_OK:
        assert list(vec[:, 0]) == [1.0, 1.0, 0.0]
    lib.pg_compat_exit_on_error(1)
