"""TORSION_SPRING command, ordering and lookup tables (host side).

Restates input.cpp:1791-2080 (TORSION_SPRING) and parmec.cpp:1968-2090
(sort_trqspr).  The per-step torque (trqspr_task, forces.ispc:1415-2057) runs
on the device.  Positions taken where the command is defective:

* the reference takes the length of zdir for xdir too and scales zdir twice
  (input.cpp:1881-1895), leaving xdir unnormalised and zdir scaled by 1/|z|^2
  for non-unit input; here each is normalised by its own length (unit input,
  the documented use, is unaffected).
"""
import math

import numpy as np

from .model import REAL_MAX

TRQCONE_ROLL, TRQCONE_PITCH, TRQCONE_YAW = 1, 2, 4        # constants.h:66-68
REAL_EPS = 2.220446049250313e-16


def _table(lst, name):
    if not isinstance(lst, list) or len(lst) < 4 or len(lst) % 2:
        raise ValueError(f"Invalid {name} lookup table list length")
    return [(float(lst[2 * j]), float(lst[2 * j + 1])) for j in range(len(lst) // 2)]


def torsion_command(m, part1, part2, zdir, xdir, kroll=None, kpitch=None, kyaw=None, droll=None, dpitch=None,
                    dyaw=None, cone=None, refpnt=None):
    if part1 < 0:
        raise ValueError("'part1' must be non-negative")
    for v, n in ((zdir, "zdir"), (xdir, "xdir")):
        if not (isinstance(v, tuple) and len(v) == 3):
            raise TypeError(f"'{n}' must be a tuple of size 3")
    if refpnt is not None and not (isinstance(refpnt, tuple) and len(refpnt) == 3):
        raise TypeError("'refpnt' must be a tuple of size 3")
    if cone is not None and not isinstance(cone, tuple):
        raise TypeError("'cone' must be a tuple")
    if part2 < -1:
        raise ValueError("Particle two index is out of range [-1, 0, ...]")
    names = ("roll", "pitch", "yaw")
    springs, dashpots = (kroll, kpitch, kyaw), (droll, dpitch, dyaw)
    ktab, dtab = [], []
    for o in range(3):
        if springs[o] is not None:
            if not isinstance(springs[o], list):
                raise TypeError(f"'k{names[o]}' must be a list")
            t = _table(springs[o], "k" + names[o])
            for j in range(1, len(t)):
                if t[j][0] <= t[j - 1][0]:
                    raise ValueError("Torsion spring angle values must increase")
        else:
            t = [(-REAL_MAX, 0.0), (REAL_MAX, 0.0)]             # zero torque
        ktab.append(t)
        d = dashpots[o]
        if isinstance(d, list):
            t = _table(d, "d" + names[o])
            for j in range(1, len(t)):
                if t[j][0] <= t[j - 1][0]:
                    raise ValueError("Torsion damper angular velocity values must increase")
        elif isinstance(d, (int, float)) and not isinstance(d, bool):
            if d < 0.0:
                raise ValueError("Critical damping ratio not in [0.0, +Inf) interval")
            t = [(float(d), float(d))]                          # critical damping ratio
        elif d is None:
            t = [(-REAL_MAX, 0.0), (REAL_MAX, 0.0)]
        else:
            raise TypeError(f"'d{names[o]}' must be a list or a number")
        dtab.append(t)
    z = [float(x) for x in zdir]
    x = [float(v) for v in xdir]
    zl = math.sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2])
    xl = math.sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2])
    if zl == 0.0:
        raise ValueError("Zero zdir length")
    if xl == 0.0:
        raise ValueError("Zero xdir length")
    iz, ix = 1.0 / zl, 1.0 / xl
    z = [z[0] * iz, z[1] * iz, z[2] * iz]
    x = [x[0] * ix, x[1] * ix, x[2] * ix]
    if z[0] * x[0] + z[1] * x[1] + z[2] * x[2] > REAL_EPS * REAL_EPS:
        raise ValueError("Directions zdir and xdir do not seem orthogonal")
    flags = 0
    if cone is not None:
        if not 2 <= len(cone) <= 3:
            raise ValueError("Invalid cone tuple size: neither 2 nor 3")
        for c in cone:
            if not isinstance(c, str):
                raise ValueError("Invalid cone tuple component: not a string")
            if c not in names:
                raise ValueError("Invalid cone tuple component name")
            flags |= (TRQCONE_ROLL, TRQCONE_PITCH, TRQCONE_YAW)[names.index(c)]
        need = {3: (0, "('roll', 'pitch')"), 5: (0, "('roll', 'yaw')"), 6: (1, "('pitch', 'yaw')"),
                7: (0, "('roll', 'pitch', 'yaw')")}
        if flags not in need:
            raise ValueError("Invalid cone tuple: components repeat")
        o, what = need[flags]
        if springs[o] is None and dashpots[o] is None:
            raise ValueError(f"A {names[o]} curve not defined for cone = {what}")
    m._touch()
    m.torsion_changed = True
    Q = m.Q
    i = m.trqsprnum
    Q.ensure(i + 1)
    m.trqsprnum += 1
    Q.tsprid[i] = i
    Q.tsprmap[i] = i
    Q.tsprpart[:, i] = (part1, part2)
    Q.zdir0[:, i] = z
    Q.xdir0[:, i] = x
    Q.zdir1[:, i] = 0.0
    Q.xdir1[:, i] = 0.0
    Q.rpy[:, i] = 0.0
    Q.rpytot[:, i] = 0.0
    Q.rpyspr[:, i] = 0.0
    Q.refpnt[:, i] = [float(v) for v in refpnt] if refpnt is not None else [REAL_MAX] * 3
    Q.cone[i] = flags
    m.krpy_tab.append(ktab)
    m.drpy_tab.append(dtab)
    return i


def sort_torsion(m):
    """sort_trqspr (parmec.cpp:1968-2090): order by (part0, part1), stably."""
    n = m.trqsprnum
    if n == 0:
        return
    Q = m.Q
    order = sorted(range(n), key=lambda i: (int(Q.tsprpart[0, i]), int(Q.tsprpart[1, i])))
    for name, (ncomp, _) in Q.spec.items():
        arr = getattr(Q, name)
        if ncomp:
            arr[:, :n] = arr[:, order]
        else:
            arr[:n] = arr[order]
    m.krpy_tab = [m.krpy_tab[i] for i in order]
    m.drpy_tab = [m.drpy_tab[i] for i in order]
    for i in range(n):
        Q.tsprmap[Q.tsprid[i]] = i


def torsion_tables(m):
    """krpy[3][2]/krpyidx[3] and drpy[3][2]/drpyidx[3] in the current order."""
    n = m.trqsprnum
    out = {}
    for key, tabs in (("krpy", m.krpy_tab), ("drpy", m.drpy_tab)):
        for o in range(3):
            idx = np.zeros(n + 1, dtype=np.int32)
            xs, ys = [], []
            for i in range(n):
                t = tabs[i][o]
                idx[i + 1] = idx[i] + len(t)
                xs += [p[0] for p in t]
                ys += [p[1] for p in t]
            arr = np.zeros((2, max(1, len(xs))))
            arr[0, :len(xs)] = xs
            arr[1, :len(ys)] = ys
            out[f"{key}{o}"] = arr
            out[f"{key}idx{o}"] = idx
    return out
