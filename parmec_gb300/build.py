"""Build libparmec_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel; the FP64 kernels are compiled with
-fmad=false so that no multiply-add is contracted (the results then agree bit
for bit with the CPU restatement used as the parity oracle).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
SOURCES = ["pg_step.cu", "pg_rebuild.cu", "pg_sort.cu", "pg_partition.cu", "pg_mixed.cu", "pg_session.cu",
           "pg_compat.cu", "pg_meshcontact.cu"]
# the FP64 form must not contract multiply-adds (bit parity with the oracle);
# the mixed form is FP32 arithmetic with explicit error-free transformations
FMAD = {"pg_mixed.cu": "true"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--prec-div=true", "--prec-sqrt=true",
                    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"] + list(extra)
    if verbose:
        flags += ["-Xptxas", "-v"]
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc()] + flags + ["-fmad=" + FMAD.get(src, "false"), "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = False
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(f"--- {src}\n{out}")
        failed |= p.returncode != 0
    if failed:
        raise RuntimeError("nvcc failed")
    lib = os.path.join(OUT, "libparmec_gb300.so")
    cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
    subprocess.run(cmd, check=True)
    if build_coupling() is None:
        sys.stderr.write("note: libparmec_gb300_coupling.so not built (Python headers or library missing)\n")
    return lib


def build_coupling():
    """libparmec_gb300_coupling.so: the C library interface (pg_coupling.cpp,
    include/parmec_coupling.h), linked against this interpreter's libpython.
    Returns the path, or None when the Python headers or library are absent."""
    import sysconfig
    inc = sysconfig.get_paths().get("include")
    libdir = sysconfig.get_config_var("LIBDIR")
    ver = sysconfig.get_config_var("LDVERSION") or sysconfig.get_config_var("VERSION")
    if not inc or not os.path.exists(os.path.join(inc, "Python.h")):
        return None
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libparmec_gb300_coupling.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", inc, os.path.join(CSRC, "pg_coupling.cpp"),
           "-o", lib, "-L", libdir, "-Wl,-rpath," + libdir, "-lpython" + ver, "-ldl"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout[-3000:])
        return None
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
