"""Build the reference's own ISPC hot path as a CPU library (TEST INFRASTRUCTURE ONLY).

`ispc` is not installed, so the reference's *.ispc sources cannot be compiled
as they are.  This recipe translates them mechanically into C++ at gang size
one and compiles the result with g++:

    python -m oracle.ispc_ref [--reference DIR]

It reads condet, forces, dynamics, parmec, partition, restrain, shapes and
obstacles .ispc, and the reference headers they include, from the reference
tree where they lie, writes one self-contained translation unit per file to
oracle/_ref/src/ and links oracle/_ref/libparmec_ref.so.  Nothing of the
reference is committed: oracle/_ref/ is git-ignored.  When the reference tree
is absent (the GPU host), build() compiles the translation units already in
oracle/_ref/src/ if they are there, and otherwise reports that the library
cannot be built.

The library exports the reference's own ISPC entry points (condet, forces,
dynamics, euler, shapes, obstacles, partitioning_*, master_alloc, ...), with
the signatures of the header ISPC would generate, so tests/ispc_loop.py drives
it with the same dem() call sequence as the GPU drop-in.

Translation rules (text to text; every rule is listed here, nothing else is
changed):

  1. `#include "x.h"` of a header in the reference tree is replaced by the
     header's translated text, so each unit compiles without the tree;
  2. `export` -> `extern "C"`; a prototype in an included header of a function
     that some file exports gets `extern "C"` too (ISPC links exported
     functions by their C names);
  3. `task` -> `static`;
  4. `foreach (v = a ... b)` -> `for (int v = a; v < b; v ++)`;
  5. `launch [n] f (args);` -> `ISPC_LAUNCH(n, f (args));` and `sync;` ->
     `ISPC_SYNC;` (oracle/ispc_gang1.h runs the n tasks and returns when all
     are done);
  6. `new T` / `new T [n]` (with any uniform qualifiers) -> `ispc_new<T>(1)` /
     `ispc_new<T>(n)`, and `delete p` / `delete[] p` -> `ispc_delete(p)`;
  7. `print (` -> `ispc_print (`;
  8. `X->lock = -1;`, `X.lock = -1;`, `lock[k] = -1;` -> `ispc_unlock(&...);`
     (a release store; see oracle/ispc_gang1.h);
  9. a function definition whose signature, once uniform and varying are
     dropped, repeats an earlier definition of the same unit is kept out with
     `#if 0` (ISPC overloads on uniform versus varying arguments; at gang
     size one both overloads compute the same thing);
 10. a function with a return value whose body does not end in a return
     statement gets `return 0;` before its closing brace (ISPC returns an
     undefined value there; C++ makes falling off the end undefined
     behaviour, which g++ compiles to a trap).

One variant adds two edits, and only to the library it names
(libparmec_ref_state.so), for the reference defect it targets: the
tangential friction state of a contact is never initialised and is not moved
when forces() compacts a list (condet.ispc:229-260, forces.ispc:339-357), so
a new contact starts from whatever state its slot last held.  The variant
zeroes the state where condet creates a contact and moves it with the
contact in the compaction, which is the position the oracle takes.  The plain
library is the reference as written.

Uniform, varying, cif, cfor and the ISPC standard-library calls are defined
by oracle/ispc_gang1.h.  The units are compiled with -DREAL=8 (the reference's
FP64 build), -ffp-contract=off (every expression evaluated as written) and
-fno-operator-names (the reference names a parameter `or`).
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libparmec_ref.so")
LIB_STATE = os.path.join(OUT, "libparmec_ref_state.so")
DEFAULT_REFERENCE = "/root/reference"
UNITS = ["partition", "condet", "forces", "dynamics", "parmec", "restrain", "shapes", "obstacles"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
            "-fno-operator-names", "-DREAL=8", "-w"]


def _match_paren(text, i):
    """Index just past the parenthesis group that opens at text[i] == '('."""
    assert text[i] == "("
    depth = 0
    for k in range(i, len(text)):
        c = text[k]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return k + 1
    raise ValueError("unbalanced parentheses")


def _foreach(text):
    out, pos = [], 0
    for m in re.finditer(r"\bforeach\s*\(", text):
        if m.start() < pos:
            continue
        open_ = m.end() - 1
        close = _match_paren(text, open_)
        inner = text[open_ + 1:close - 1]
        var, rng = inner.split("=", 1)
        lo, hi = rng.split("...", 1)
        var, lo, hi = var.strip(), lo.strip(), hi.strip()
        out.append(text[pos:m.start()])
        out.append(f"for (int {var} = {lo}; {var} < ({hi}); {var} ++)")
        pos = close
    out.append(text[pos:])
    return "".join(out)


def _launch(text):
    out, pos = [], 0
    for m in re.finditer(r"\blaunch\s*\[([^\]]+)\]\s*(\w+)\s*\(", text):
        if m.start() < pos:
            continue
        open_ = m.end() - 1
        close = _match_paren(text, open_)
        out.append(text[pos:m.start()])
        out.append(f"ISPC_LAUNCH(({m.group(1)}), {m.group(2)} {text[open_:close]})")
        pos = close
    out.append(text[pos:])
    return "".join(out)


def _new_delete(text):
    q = r"(?:uniform\s+|varying\s+)*"
    text = re.sub(q + r"\bnew\s+" + q + r"(?:struct\s+)?(\w+)\s*\[([^\]]+)\]",
                  lambda m: f"ispc_new<{m.group(1)}>({m.group(2)})", text)
    text = re.sub(q + r"\bnew\s+" + q + r"(?:struct\s+)?(\w+)",
                  lambda m: f"ispc_new<{m.group(1)}>(1)", text)
    text = re.sub(r"\bdelete\s*(?:\[\s*\])?\s*([\w\->\.\[\]]+)\s*;", lambda m: f"ispc_delete({m.group(1)});", text)
    return text


def _unlock(text):
    return re.sub(r"([\w\->\.\[\]]*(?:->|\.)lock|\block\s*\[[^\]]+\])\s*=\s*-1\s*;",
                  lambda m: f"ispc_unlock(&({m.group(1)}));", text)


def _strip_comments(text):
    return re.sub(r"/\*.*?\*/|//[^\n]*", lambda m: re.sub(r"[^\n]", " ", m.group(0)), text, flags=re.S)


def _dedupe_definitions(text):
    """Rule 9: keep out a definition whose uniform-free signature repeats."""
    bare = _strip_comments(text)
    seen, cuts = set(), []
    depth, stmt_start = 0, 0
    i = 0
    while i < len(bare):
        c = bare[i]
        if c == "{":
            if depth == 0:
                head = bare[stmt_start:i]
                if re.search(r"\)\s*$", head) and "=" not in head.split("(")[0]:
                    sig = re.sub(r"\b(uniform|varying|inline|static)\b", " ", head)
                    sig = re.sub(r"\s+", " ", sig).strip()
                    sig = re.sub(r"\s*([(),\[\]*])\s*", r"\1", sig)
                    # the name and the parameter list identify the definition
                    if sig in seen:
                        # find the end of the body
                        d, k = 0, i
                        while k < len(bare):
                            if bare[k] == "{":
                                d += 1
                            elif bare[k] == "}":
                                d -= 1
                                if d == 0:
                                    break
                            k += 1
                        # start of the definition: after the previous line break
                        s = bare.rfind("\n", 0, stmt_start + len(bare[stmt_start:i]) - len(bare[stmt_start:i].lstrip()))
                        cuts.append((s + 1, k + 1))
                    else:
                        seen.add(sig)
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                stmt_start = i + 1
        elif c in ";" and depth == 0:
            stmt_start = i + 1
        elif c == "#" and depth == 0:
            # preprocessor lines end a top-level statement
            e = bare.find("\n", i)
            stmt_start = e + 1 if e >= 0 else len(bare)
            i = stmt_start
            continue
        i += 1
    for s, e in reversed(cuts):
        text = text[:s] + "#if 0 /* repeats an earlier definition once uniform/varying are dropped */\n" + \
               text[s:e] + "\n#endif\n" + text[e:]
    return text


def _terminate_returns(text):
    """Rule 10: `return 0;` at the end of a value-returning body without one."""
    bare = _strip_comments(text)
    inserts = []
    depth, stmt_start, open_at, head = 0, 0, -1, ""
    i = 0
    while i < len(bare):
        c = bare[i]
        if c == "{":
            if depth == 0:
                head = bare[stmt_start:i]
                open_at = i
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                h = re.sub(r"\s+", " ", head).strip()
                m = re.match(r"(?:(?:extern \"C\"|static|inline|uniform|varying)\s+)*(.+?)\b(\w+)\s*\(", h)
                if m and re.search(r"\)\s*$", h) and "=" not in h.split("(")[0]:
                    rtype = m.group(1).strip()
                    body = bare[open_at + 1:i].rstrip()
                    if rtype not in ("void", "") and not re.search(r"\breturn\b[^;]*;\s*$", body):
                        inserts.append(i)
                stmt_start = i + 1
        elif c == ";" and depth == 0:
            stmt_start = i + 1
        elif c == "#" and depth == 0:
            e = bare.find("\n", i)
            stmt_start = e + 1 if e >= 0 else len(bare)
            i = stmt_start
            continue
        i += 1
    for k in reversed(inserts):
        text = text[:k] + "  return 0; /* the reference leaves the value unset */\n" + text[k:]
    return text


def translate_text(text):
    text = re.sub(r"\bexport\b", 'extern "C"', text)
    text = re.sub(r"\btask\b(?=\s+void\b)", "static", text)
    text = _foreach(text)
    text = _launch(text)
    text = re.sub(r"\bsync\s*;", "ISPC_SYNC;", text)
    text = _new_delete(text)
    text = re.sub(r"\bprint\s*\(", "ispc_print (", text)
    text = _unlock(text)
    return text


def exported_names(ref):
    names = set()
    for u in UNITS:
        with open(os.path.join(ref, u + ".ispc")) as f:
            src = _strip_comments(f.read())
        for m in re.finditer(r"\bexport\b[^;{(]*?\b(\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def _inline_headers(text, ref, exports, seen):
    def repl(m):
        name = m.group(1)
        path = os.path.join(ref, name)
        if not os.path.exists(path):
            return m.group(0)
        if name in seen:
            return f"/* {name} already included */"
        seen.add(name)
        with open(path) as f:
            h = f.read()
        h = _inline_headers(h, ref, exports, seen)
        h = translate_text(h)
        # rule 2: prototypes of exported functions take C linkage
        for e in exports:
            h = re.sub(r"(^|\n)(\s*)((?:uniform\s+)?\w+[\s\*]+(?:uniform\s+)?" + e + r"\s*\([^;{]*\)\s*;)",
                       lambda mm: f"{mm.group(1)}{mm.group(2)}extern \"C\" {mm.group(3)}", h)
        return f"/* ---- {name} (reference header, translated) ---- */\n{h}\n/* ---- end {name} ---- */"
    return re.sub(r'^\s*#\s*include\s+"([^"]+)"', repl, text, flags=re.M)


def _state_variant(unit, text):
    """The friction-state variant's two edits (see the module docstring)."""
    if unit == "condet":
        text, n = re.subn(r"(con->depth\[k\] = depth\[j\];)",
                          r"\1 for (int s_ = 0; s_ < NSTATE; s_ ++) con->state[s_][k] = 0.0;", text)
        assert n == 3, "condet: expected three sphere-contact creations"
    elif unit == "forces":
        text, n = re.subn(r"(con->ecur\[k\] = con->ecur\[j\];)",
                          r"\1 for (int s_ = 0; s_ < NSTATE; s_ ++) con->state[s_][k] = con->state[s_][j];", text)
        assert n == 1, "forces: expected one list compaction"
    return text


def translate(ref=DEFAULT_REFERENCE):
    """Write oracle/_ref/src/<unit>.cpp (and the friction-state variant's
    oracle/_ref/src/state_<unit>.cpp) from the reference tree at `ref`."""
    os.makedirs(SRC_OUT, exist_ok=True)
    exports = exported_names(ref)
    for u in UNITS:
        with open(os.path.join(ref, u + ".ispc")) as f:
            src = f.read()
        body = _inline_headers(src, ref, exports, set())
        body = translate_text(body)
        body = _dedupe_definitions(body)
        body = _terminate_returns(body)
        for name, text in ((u, body), ("state_" + u, _state_variant(u, body))):
            with open(os.path.join(SRC_OUT, name + ".cpp"), "w") as f:
                f.write(f"/* generated by oracle/ispc_ref.py from the reference's {u}.ispc; not for commit */\n")
                f.write('#include "ispc_gang1.h"\n')
                f.write(text)
    return [os.path.join(SRC_OUT, u + ".cpp") for u in UNITS]


def _sources(variant):
    return [os.path.join(SRC_OUT, (variant + u) + ".cpp") for u in UNITS]


def compile_units(sources, lib, cxx="g++"):
    objs, procs = [], []
    for s in sources:
        o = s[:-4] + ".o"
        objs.append(o)
        procs.append((s, subprocess.Popen([cxx] + CXXFLAGS + ["-I", HERE, "-c", s, "-o", o],
                                          stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    bad = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            bad.append(f"--- {os.path.basename(s)}\n{out}")
    if bad:
        raise RuntimeError("compiling the translated reference failed:\n" + "\n".join(bad)[-6000:])
    # -Bsymbolic: calls between the units (forces -> eqm) bind inside this
    # library even when another library with the same entry points is loaded
    subprocess.run([cxx, "-shared", "-fopenmp", "-Wl,-Bsymbolic", "-o", lib] + objs, check=True)
    return lib


def build(ref=None):
    """Translate (when the reference tree is present) and compile.  Returns the
    library path, or None when neither the tree nor translated units exist."""
    ref = ref or os.environ.get("PARMEC_REFERENCE", DEFAULT_REFERENCE)
    if os.path.isdir(ref) and os.path.exists(os.path.join(ref, "condet.ispc")):
        translate(ref)
    if not all(os.path.exists(s) for s in _sources("") + _sources("state_")):
        return None
    compile_units(_sources("state_"), LIB_STATE)
    return compile_units(_sources(""), LIB)


def available():
    return os.path.exists(LIB)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    lib = build(a.reference)
    print(lib or "reference sources not found; nothing built")
    sys.exit(0 if lib else 1)
