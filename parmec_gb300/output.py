"""File output: the OUTPUT command (input.cpp:3560-3955) and output_files
(output.cpp:5127-5140) in the DUMP and VTK formats.

Files are named as the reference names them: <path><j>.vtk.<frame> for
triangles, <path><j>rb.vtk.<frame> for rigid bodies, <path><j>sl.vtk.<frame>
and <path><j>st.vtk.<frame> for linear and torsional springs, and
<path><j>.dump (appended frame after frame) for spheres, where j = 0 is the
particles no OUTPUT subset selected and j = 1, 2, ... the subsets in command
order.  Numbers are printed as C++ streams print doubles by default (%g).

The XDMF (the reference's default) and MED formats need the HDF5 and MED
libraries, which this build does not have: a DEM with only those formats
selected writes no files and says so once.  Positions taken:
* the unselected-spring test reads flags & OUTREST (the reference writes
  flags && OUTREST, output.cpp:4553, 4625, selecting every spring);
* OUTPUT's RB/CD/SL/ST/JT modes without a subset set the unselected
  particles' modes (the reference writes outmode[1] or outmode[i] there,
  input.cpp:3654-3669, 3701-3721).
"""
import os
import sys

import numpy as np

OUT_FORMAT_DUMP, OUT_FORMAT_VTK, OUT_FORMAT_XDMF, OUT_FORMAT_MED = 1, 2, 4, 8
OUT_MODE = {"SPH": 1, "MESH": 2, "RB": 4, "CD": 8, "SL": 16, "ST": 32, "JT": 64}
OUT_MODE_ALL = 127
OUT_ENT = {"NUMBER": 1, "COLOR": 2, "DISPL": 4, "ORIENT": 8, "ORIENT1": 16, "ORIENT2": 32, "ORIENT3": 64,
           "LINVEL": 128, "ANGVEL": 256, "FORCE": 512, "TORQUE": 1024, "F": 2048, "FN": 4096, "FT": 8192,
           "SF": 16384, "AREA": 32768, "PAIR": 65536, "LENGTH": 131072, "SS": 262144, "FF": 524288,
           "XDIR": 1048576, "YDIR": 2097152, "ZDIR": 4194304, "TRQROT": 8388608, "TRQTOT": 16777216,
           "TRQSPR": 33554432, "JREAC": 67108864}
OUT_FORMATS = {"DUMP": OUT_FORMAT_DUMP, "VTK": OUT_FORMAT_VTK, "XDMF": OUT_FORMAT_XDMF, "MED": OUT_FORMAT_MED}
E = OUT_ENT


class OutputState:
    """outnum/outidx/outpart/outent/outmode/outrest/outformat/output_frame/output_path."""

    def __init__(self):
        self.subsets = []                  # (particles, entity mask, mode mask) per OUTPUT with a subset
        self.rest = [0xffffffff, OUT_MODE_ALL]
        self.format = OUT_FORMAT_XDMF
        self.frame = 0
        self.path = None
        self.warned = False


def default_path():
    p = sys.argv[0] if sys.argv and sys.argv[0] else ""
    return p[:-3] if p.endswith(".py") else os.path.join(os.getcwd(), "parmec")


def output_command(m, entities=None, subset=None, mode=None, format=None):
    """OUTPUT (input.cpp:3560-3955)."""
    from .model import OUTREST
    if entities is not None and not isinstance(entities, list):
        raise TypeError("'entities' must be a list")
    if subset is not None and not isinstance(subset, (list, int)):
        raise TypeError("'subset' must be a list or a number")
    for v, n in ((mode, "mode"), (format, "format")):
        if v is not None and not isinstance(v, (str, list)):
            raise TypeError(f"'{n}' must be a string or a list")
    parts = None
    if subset is not None:
        parts = [subset] if isinstance(subset, int) else list(subset)
        for k in parts:
            if not (0 <= int(k) < m.parnum):
                raise ValueError("Invalid particle number")
    mmask = OUT_MODE_ALL
    if mode is not None:
        items = [mode] if isinstance(mode, str) else mode
        mmask = 0
        for it in items:
            if not isinstance(it, str):
                raise TypeError("mode list item is not a string")
            if it not in OUT_MODE:
                raise ValueError("Invalid mode")
            mmask |= OUT_MODE[it]
    emask = 0xffffffff
    if entities is not None:
        emask = 0
        for it in entities:
            if it not in OUT_ENT:
                raise ValueError("Invalid entity")
            emask |= OUT_ENT[it]
    fmask = None
    if format is not None:
        items = [format] if isinstance(format, str) else format
        fmask = 0
        for it in items:
            if it not in OUT_FORMATS:
                raise ValueError("Invalid format")
            fmask |= OUT_FORMATS[it]
    o = m.out
    if parts is not None:
        for k in parts:
            m.P.flags[int(k)] &= ~OUTREST
        o.subsets.append(([int(k) for k in parts], emask, mmask))
    else:
        o.rest = [emask, mmask]
    if fmask is not None:
        o.format = fmask
    return None


def _rows(f, cols):
    """Rows of space-separated %g numbers (C++ stream defaults)."""
    if cols and len(cols[0]):
        np.savetxt(f, np.column_stack(cols), fmt="%g", delimiter=" ")


def _ints(f, vals):
    if len(vals):
        np.savetxt(f, np.asarray(vals, dtype=np.int64).reshape(-1, 1), fmt="%d")


def _header(f, what, t):
    f.write("# vtk DataFile Version 2.0\n")
    f.write(f"PARMEC {what} output at time {t:g}\n")
    f.write("ASCII\n")


def _triangles(m, f, s, ent):
    """vtk_triangle_dataset (output.cpp:1709-1978)."""
    P, Tr, O = m.P, m.Tr, m.O
    s = np.asarray(s, dtype=np.int64)
    n = len(s)
    tri = Tr.tri[:, s]
    f.write("DATASET UNSTRUCTURED_GRID\n")
    f.write(f"POINTS {3 * n} float\n")
    _rows(f, [tri[k] for k in range(9)])
    f.write(f"CELLS {n} {4 * n}\n")
    i = np.arange(n)
    if n:
        np.savetxt(f, np.column_stack([np.full(n, 3), 3 * i, 3 * i + 1, 3 * i + 2]), fmt="%d")
    f.write(f"CELL_TYPES {n}\n")
    if n:
        np.savetxt(f, np.full((n, 1), 5), fmt="%d")
    obs = Tr.triobs[s]
    pts = [tri[0:3], tri[3:6], tri[6:9]]
    if ent & (E["DISPL"] | E["LINVEL"]):
        f.write(f"POINT_DATA {3 * n}\n")
    if ent & E["DISPL"]:
        f.write("VECTORS displ float\n")
        out = np.zeros((n, 9))
        for r in range(n):
            j = obs[r]
            for v in range(3):
                p = pts[v][:, r]
                if j >= 0:
                    L = P.rotation[:, j]
                    x, X = P.position[0:3, j], P.position[3:6, j]
                    d = p - x
                    Pp = [X[0] + (L[0] * d[0] + L[1] * d[1] + L[2] * d[2]),
                          X[1] + (L[3] * d[0] + L[4] * d[1] + L[5] * d[2]),
                          X[2] + (L[6] * d[0] + L[7] * d[1] + L[8] * d[2])]
                    out[r, 3 * v:3 * v + 3] = [p[0] - Pp[0], p[1] - Pp[1], p[2] - Pp[2]]
                elif j < -1:
                    q = -j - 2
                    out[r, 3 * v:3 * v + 3] = p - O.obspnt[:, q]
        _rows(f, [out.reshape(-1, 3)[:, k] for k in range(3)])
    if ent & E["LINVEL"]:
        f.write("VECTORS linvel float\n")
        out = np.zeros((n, 9))
        for r in range(n):
            j = obs[r]
            if j == -1:
                continue
            if j >= 0:
                x, o, v0 = P.position[0:3, j], P.angular[3:6, j], P.linear[:, j]
            else:
                q = -j - 2
                x, o, v0 = O.obspnt[:, q], O.obsang[:, q], O.obslin[:, q]
            for v in range(3):
                a = pts[v][:, r] - x
                out[r, 3 * v:3 * v + 3] = [v0[0] + (o[1] * a[2] - o[2] * a[1]), v0[1] + (o[2] * a[0] - o[0] * a[2]),
                                           v0[2] + (o[0] * a[1] - o[1] * a[0])]
        _rows(f, [out.reshape(-1, 3)[:, k] for k in range(3)])
    if ent & (E["NUMBER"] | E["COLOR"] | E["ANGVEL"] | E["FORCE"] | E["TORQUE"]):
        f.write(f"CELL_DATA {n}\n")
    if ent & E["NUMBER"]:
        f.write("SCALARS number int\nLOOKUP_TABLE default\n")
        _ints(f, obs)
    if ent & E["COLOR"]:
        f.write("SCALARS colors int\nLOOKUP_TABLE default\n")
        _ints(f, Tr.tricol[s])
    for key, name in (("ANGVEL", "angvel"), ("FORCE", "force"), ("TORQUE", "torque")):
        if not ent & E[key]:
            continue
        f.write(f"VECTORS {name} float\n")
        out = np.zeros((n, 3))
        for r in range(n):
            j = obs[r]
            if j >= 0:
                out[r] = {"ANGVEL": P.angular[3:6, j], "FORCE": P.force[:, j], "TORQUE": P.torque[:, j]}[key]
            elif j < -1 and key == "ANGVEL":
                out[r] = O.obsang[:, -j - 2]
        _rows(f, [out[:, k] for k in range(3)])


def _rigid(m, f, s, ent):
    """output_rb_dataset (output.cpp:146-268)."""
    P = m.P
    s = np.asarray(s, dtype=np.int64)
    n = len(s)
    f.write("DATASET UNSTRUCTURED_GRID\n")
    f.write(f"POINTS {n} float\n")
    _rows(f, [P.position[k, s] for k in range(3)])
    if ent & (E["NUMBER"] | E["DISPL"] | E["ORIENT1"] | E["ORIENT2"] | E["ORIENT3"] | E["LINVEL"] | E["ANGVEL"]
              | E["FORCE"] | E["TORQUE"]):
        f.write(f"POINT_DATA {n}\n")
    if ent & E["NUMBER"]:
        f.write("SCALARS NUMBER int\nLOOKUP_TABLE default\n")
        _ints(f, s)
    if ent & E["DISPL"]:
        f.write("VECTORS DISPL float\n")
        _rows(f, [P.position[k, s] - P.position[3 + k, s] for k in range(3)])
    for key, rows in (("ORIENT1", (0, 1, 2)), ("ORIENT2", (3, 4, 5)), ("ORIENT3", (6, 7, 8))):
        if ent & E[key]:
            f.write(f"VECTORS {key} float\n")
            _rows(f, [P.rotation[k, s] for k in rows])
    for key, arr in (("LINVEL", P.linear), ("ANGVEL", P.angular), ("FORCE", P.force), ("TORQUE", P.torque)):
        if ent & E[key]:
            f.write(f"VECTORS {key} float\n")
            _rows(f, [arr[k, s] for k in range(3)])


def _linear_springs(m, f, s, ent):
    """vtk_linear_spring_dataset (output.cpp:2855-2967)."""
    S = m.S
    s = np.asarray(s, dtype=np.int64)
    n = len(s)
    f.write("DATASET UNSTRUCTURED_GRID\n")
    f.write(f"POINTS {n} float\n")
    _rows(f, [0.5 * (S.sprpnt[k, s] + S.sprpnt[6 + k, s]) for k in range(3)])
    if ent & (E["NUMBER"] | E["DISPL"] | E["F"] | E["SF"] | E["PAIR"] | E["SS"] | E["FF"]):
        f.write(f"POINT_DATA {n}\n")
    if ent & E["NUMBER"]:
        f.write("SCALARS number int\nLOOKUP_TABLE default\n")
        _ints(f, S.sprid[s])
    if ent & E["DISPL"]:
        f.write("SCALARS displ float\nLOOKUP_TABLE default\n")
        _rows(f, [S.stroke[0, s]])
    if ent & E["LENGTH"]:
        f.write("SCALARS length float\nLOOKUP_TABLE default\n")
        q = S.sprpnt[6:9, s] - S.sprpnt[0:3, s]
        _rows(f, [np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2])])
    if ent & E["ORIENT"]:
        f.write("VECTORS orient float\n")
        _rows(f, [S.sprdir[k, s] for k in range(3)])
    for key, row in (("F", 0), ("SF", 1), ("FF", 2)):
        if ent & E[key]:
            f.write(f"SCALARS {key} float\nLOOKUP_TABLE default\n")
            _rows(f, [S.sprfrc[row, s]])
    if ent & E["SS"]:
        f.write("SCALARS SS float\nLOOKUP_TABLE default\n")
        _rows(f, [S.unspring[s].astype(np.float32).astype(np.float64)])


def _torsion_springs(m, f, s, ent):
    """vtk_torsional_spring_dataset (output.cpp:2969-3143)."""
    from .model import REAL_MAX
    P, Q = m.P, m.Q
    s = np.asarray(s, dtype=np.int64)
    n = len(s)
    f.write("DATASET UNSTRUCTURED_GRID\n")
    f.write(f"POINTS {n} float\n")
    pts = np.zeros((n, 3))
    for r, j in enumerate(s):
        k, l = int(Q.tsprpart[0, j]), int(Q.tsprpart[1, j])
        ref = Q.refpnt[:, j]
        if ref[0] != REAL_MAX:
            L = P.rotation[:, k]
            d = ref - P.position[3:6, k]
            x = P.position[0:3, k]
            pts[r] = [x[0] + (L[0] * d[0] + L[3] * d[1] + L[6] * d[2]), x[1] + (L[1] * d[0] + L[4] * d[1] + L[7] * d[2]),
                      x[2] + (L[2] * d[0] + L[5] * d[1] + L[8] * d[2])]
        elif l == -1:
            pts[r] = P.position[0:3, k]
        else:
            pts[r] = 0.5 * (P.position[0:3, k] + P.position[0:3, l])
    _rows(f, [pts[:, k] for k in range(3)])
    if ent & (E["NUMBER"] | E["ZDIR"] | E["XDIR"] | E["YDIR"] | E["TRQROT"] | E["TRQTOT"] | E["TRQSPR"]):
        f.write(f"POINT_DATA {n}\n")
    if ent & E["NUMBER"]:
        f.write("SCALARS number int\nLOOKUP_TABLE default\n")
        _ints(f, Q.tsprid[s])
    z, x = Q.zdir1[:, s], Q.xdir1[:, s]
    y = np.stack([z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]])
    if ent & E["ZDIR"]:
        f.write("VECTORS ZDIR float\n")
        _rows(f, [z[k] for k in range(3)])
    if ent & E["XDIR"]:
        f.write("VECTORS XDIR float\n")
        _rows(f, [x[k] for k in range(3)])
    if ent & E["YDIR"]:
        f.write("VECTORS YDIR float\n")
        _rows(f, [y[k] for k in range(3)])
    for key, arr in (("TRQROT", Q.rpy), ("TRQTOT", Q.rpytot), ("TRQSPR", Q.rpyspr)):
        if ent & E[key]:
            f.write(f"VECTORS {key} float\n")
            a = arr[:, s]
            _rows(f, [x[k] * a[0] + y[k] * a[1] + z[k] * a[2] for k in range(3)])


def _dump(m, f, s, ent, t):
    """output_dump_dataset (output.cpp:54-144), spheres."""
    P, Es = m.P, m.E
    s = np.asarray(s, dtype=np.int64)
    k = Es.part[s]
    f.write("ITEM: TIMESTEP\n")
    f.write(f"{t:g}\n")
    f.write("ITEM: NUMBER OF ATOMS\n")
    f.write(f"{len(s)}\n")
    f.write("ITEM: BOX BOUNDS\n0 1\n0 1\n0 1\n")
    head = "ITEM: ATOMS id x y z radius"
    cols = [Es.center[0, s], Es.center[1, s], Es.center[2, s], Es.radii[0, s]]
    for key, name, arr in (("LINVEL", " vx vy vz", P.linear), ("ANGVEL", " omegax omegay omegaz", P.angular),
                           ("FORCE", " fx fy fz", P.force), ("TORQUE", " tqx tqy tqz", P.torque)):
        if ent & E[key]:
            head += name
            cols += [arr[c, k] for c in range(3)]
    f.write(head + "\n")
    if len(s):
        body = np.column_stack(cols)
        for r in range(len(s)):
            f.write(f"{s[r] + 1} " + " ".join(f"{v:g}" for v in body[r]) + "\n")


def _springs_of(n_parts, part0, part1, parts):
    """The springs attached to each listed particle, in index order (MAP order)."""
    out = []
    for p in parts:
        out += [int(i) for i in range(n_parts) if part0[i] == p or part1[i] == p]
    return out


def output_files(m, t):
    """output_files (output.cpp:5127-5140) at time t: DUMP and VTK files of the
    unselected particles (j = 0) and of each OUTPUT subset (j = 1, ...)."""
    from .model import OUTREST
    o = m.out
    if o.path is None:
        o.path = default_path()
    fmt = o.format
    if fmt & (OUT_FORMAT_XDMF | OUT_FORMAT_MED) and not o.warned:
        print("parmec_gb300: XDMF and MED output need HDF5 and MED, which this build lacks; "
              "OUTPUT(format='VTK') or 'DUMP' writes files", file=sys.stderr)
        o.warned = True
    flags = m.P.flags
    groups = [(None, o.rest[0], o.rest[1])] + [(p, e, md) for p, e, md in o.subsets]
    path = o.path
    if fmt & OUT_FORMAT_DUMP and m.ellnum:
        for j, (parts, ent, mode) in enumerate(groups):
            if not mode & OUT_MODE["SPH"]:
                continue
            if parts is None:
                s = [i for i in range(m.ellnum) if flags[m.E.part[i]] & OUTREST]
            else:
                s = [i for p in parts for i in range(m.ellnum) if m.E.part[i] == p]
            with open(f"{path}{j}.dump", "a" if o.frame else "w") as f:
                _dump(m, f, s, ent, t)
    if fmt & OUT_FORMAT_VTK:
        tr = m.Tr.triobs[:m.trinum]
        for j, (parts, ent, mode) in enumerate(groups):
            if m.trinum and mode & OUT_MODE["MESH"]:
                if parts is None:
                    s = [i for i in range(m.trinum) if tr[i] < 0 or flags[tr[i]] & OUTREST]
                else:
                    s = [i for p in parts for i in range(m.trinum) if tr[i] == p]
                with open(f"{path}{j}.vtk.{o.frame}", "w") as f:
                    _header(f, "triangles", t)
                    if parts is None or s:
                        _triangles(m, f, s, ent)
            if m.parnum and mode & OUT_MODE["RB"]:
                s = [i for i in range(m.parnum) if flags[i] & OUTREST] if parts is None else parts
                with open(f"{path}{j}rb.vtk.{o.frame}", "w") as f:
                    _header(f, "rigid bodies", t)
                    _rigid(m, f, s, ent)
            for num, part, tag, what, writer in (
                    (m.sprnum, m.S.sprpart, "sl", "linear springs", _linear_springs),
                    (m.trqsprnum, m.Q.tsprpart, "st", "torsional springs", _torsion_springs)):
                if not num or not mode & OUT_MODE[tag.upper()]:
                    continue
                p0, p1 = part[0, :num], part[1, :num]
                if parts is None:
                    s = [i for i in range(num) if flags[p0[i]] & OUTREST or (p1[i] >= 0 and flags[p1[i]] & OUTREST)]
                else:
                    s = _springs_of(num, p0, p1, parts)
                with open(f"{path}{j}{tag}.vtk.{o.frame}", "w") as f:
                    _header(f, what, t)
                    if parts is None or s:
                        writer(m, f, s, ent)
    o.frame += 1
