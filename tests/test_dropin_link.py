"""The unmodified reference host code compiles and links against the drop-in.

parmec.cpp and input.cpp include the headers ISPC generates from the
kernels (parmec_ispc.h, partition_ispc.h, forces_ispc.h, ...; parmec.cpp:46-52,
input.cpp:43-49).  Here include/parmec_ispc.h stands in for all of them: the
reference's own parmec_ispc.h include finds it on the include path, and
each other generated header is a one-line shim that includes it.  Both
files compile with REAL = double, so every call site type-checks against
the declarations; every ISPC entry point their objects leave undefined must
be exported by libparmec_gb300.so.  Runs where the reference's sources are
(skipped elsewhere); needs no GPU.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("PARMEC_REFERENCE", "/root/reference")
SHIMS = ("partition", "condet", "forces", "dynamics", "shapes", "obstacles", "restrain")


def symbols(path, *flags):
    out = subprocess.run(["nm", *flags, path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


@pytest.fixture(scope="module")
def objects(tmp_path_factory):
    if not os.path.exists(os.path.join(REFERENCE, "parmec.cpp")):
        pytest.skip("the reference's sources are not on this host")
    if not shutil.which("g++") or not shutil.which("python3-config") or not shutil.which("nm"):
        pytest.skip("g++, python3-config or nm missing")
    d = tmp_path_factory.mktemp("dropin")
    shim = d / "shim"
    shim.mkdir()
    for f in SHIMS:
        (shim / f"{f}_ispc.h").write_text('#include "parmec_ispc.h"\n')
    pyinc = subprocess.run(["python3-config", "--includes"], capture_output=True, text=True,
                           check=True).stdout.split()
    objs = []
    for src in ("parmec", "input"):
        o = str(d / f"{src}.o")
        r = subprocess.run(["g++", "-std=c++11", "-DREAL=8", "-fopenmp", "-w", "-I", os.path.join(ROOT, "include"),
                            "-I", str(shim), "-I", REFERENCE, *pyinc, "-c", os.path.join(REFERENCE, f"{src}.cpp"),
                            "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, f"{src}.cpp does not compile against include/parmec_ispc.h:\n{r.stderr[-3000:]}"
        objs.append(o)
    return objs


def test_reference_host_calls_are_exported(objects):
    from oracle import ispc_ref
    from parmec_gb300 import abi
    lib = abi.library_path()
    if not os.path.exists(lib):
        pytest.skip("libparmec_gb300.so is not built")
    entry_points = ispc_ref.exported_names(REFERENCE)
    undefined = set()
    for o in objects:
        undefined |= symbols(o, "-u")
    needed = undefined & entry_points
    assert {"condet", "forces", "dynamics", "eqm", "critical_perparticle", "critical_perspring"} <= needed
    missing = sorted(needed - symbols(lib, "-D", "--defined-only"))
    assert not missing, f"entry points the reference calls but libparmec_gb300.so does not export: {missing}"
