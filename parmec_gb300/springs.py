"""SPRING command, spring ordering and spring tables (host side).

Restates input.cpp:1440-1788 (SPRING), parmec.cpp:1683-1965 (sort_springs),
parmec.cpp:1239-1269 (lcurve_from_time_series) and parmec.ispc:423-482 (eqm,
for the EQM command) for the host.  The per-step spring force and CRITICAL
run on the device.
"""
import math

import numpy as np

from .model import (REAL_MAX, SPRDIR_CONSTANT, SPRDIR_FOLLOWER, SPRDIR_PLANAR, SPRDIR_PROJECT,
                    SPRING_GENERAL_NONLINEAR, SPRING_NONLINEAR_ELASTIC)


def _pairs(lst, what):
    if not isinstance(lst, list) or len(lst) < 4 or len(lst) % 2:
        raise ValueError(f"Invalid {what} lookup table list length")
    return [(float(lst[2 * j]), float(lst[2 * j + 1])) for j in range(len(lst) // 2)]


def spring_command(m, part1, point1, part2, geom2, spring, dashpot, direction, planar,
                   unload, ylim, inactive, offset, friction, kskn):
    if part1 < 0:
        raise ValueError("'part1' must be non-negative")
    if not (isinstance(point1, tuple) and len(point1) == 3):
        raise TypeError("'point1' must be a tuple of size 3")
    if friction < 0 or kskn < 0:
        raise ValueError("'friction' and 'kskn' must be non-negative")
    if offset < -1 or offset >= len(m.tms):
        raise ValueError("offset TSERIES index is out of range")
    if part2 < -1:
        raise ValueError("Particle two index is out of range [-1, 0, ...]")
    sp = _pairs(spring, "spring")
    for j in range(1, len(sp)):
        if sp[j][0] <= sp[j - 1][0]:
            raise ValueError("Spring stroke values must increase")
    if isinstance(dashpot, list):
        dp = _pairs(dashpot, "dashpot")
        for j in range(1, len(dp)):
            if dp[j][0] <= dp[j - 1][0]:
                raise ValueError("Dashpot velocity values must increase")
    elif dashpot is not None:
        ratio = float(dashpot)
        if ratio < 0.0:
            raise ValueError("Critical damping ratio not in [0.0, +Inf) interval")
        dp = [(ratio, ratio)]
    else:
        dp = [(-REAL_MAX, 0.0), (REAL_MAX, 0.0)]
    ul = None
    if unload is not None:
        ul = _pairs(unload, "unload")
        for j in range(1, len(ul)):
            slope = (ul[j][1] - ul[j - 1][1]) / (ul[j][0] - ul[j - 1][0])
            if slope <= 0.0:
                raise ValueError("Unloading curve must be monotonically increasing")

    S = m.S
    i = m.sprnum
    S.ensure(i + 1)
    m.sprnum += 1
    S.sprid[i] = i
    S.sprmap[i] = i
    S.sprpart[:, i] = (part1, part2)
    p1 = [float(x) for x in point1]
    S.sprpnt[0:3, i] = p1
    S.sprpnt[3:6, i] = p1
    S.sprdir[:, i] = 0.0
    if isinstance(geom2, tuple):
        if len(geom2) != 3:
            raise TypeError("'geom2' must be a tuple of size 3 or a [point, normal] list")
        q = [float(x) for x in geom2]
        S.sprpnt[6:9, i] = q
        S.sprpnt[9:12, i] = q
    else:
        point, normal = geom2[0], geom2[1]
        q = [float(x) for x in point]
        d = [float(x) for x in normal]
        ln = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])     # NORMALIZE (macros.h:427)
        d = [d[0] / ln, d[1] / ln, d[2] / ln]
        S.sprdir[0:3, i] = d
        S.sprdir[3:6, i] = d
        w = [p1[0] - q[0], p1[1] - q[1], p1[2] - q[2]]
        ln = d[0] * w[0] + d[1] * w[1] + d[2] * w[2]
        q = [p1[0] - ln * d[0], p1[1] - ln * d[1], p1[2] - ln * d[2]]   # SUBMUL
        S.sprpnt[6:9, i] = q
        S.sprpnt[9:12, i] = q
    S.sprflg[i] = 0
    S.sproffset[i] = -1 if offset < 0 else _lcurve_from_time_series(m, offset)
    S.sprfric[i] = float(friction)
    S.sprkskn[i] = float(kskn)
    S.sprsdsp[:, i] = 0.0
    S.stroke[:, i] = 0.0
    S.sprfrc[:, i] = 0.0
    m.spring_tab.append(sp)
    m.dashpot_tab.append(dp)
    m.unload_tab.append(ul)
    S.sprtype[i] = SPRING_GENERAL_NONLINEAR if ul is not None else SPRING_NONLINEAR_ELASTIC
    S.unspring[i] = -1 if inactive is True else -3
    if not isinstance(geom2, tuple):
        S.sprflg[i] |= SPRDIR_PROJECT
        S.stroke0[i] = 0.0
    else:
        if direction is not None:
            d = [float(x) for x in direction]
            ln = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
            if ln == 0.0:
                raise ValueError("Invalid zero direction")
            inv = 1.0 / ln
            d = [d[0] * inv, d[1] * inv, d[2] * inv]
            S.sprdir[0:3, i] = d
            S.sprdir[3:6, i] = d
            if planar is not None:
                if planar == "ON":
                    S.sprflg[i] |= SPRDIR_PLANAR
                elif planar == "OFF":
                    S.sprflg[i] |= SPRDIR_CONSTANT
                else:
                    raise ValueError("Invalid planar switch")
            else:
                S.sprflg[i] |= SPRDIR_CONSTANT
            dif = [q[0] - p1[0], q[1] - p1[1], q[2] - p1[2]]
            if S.sprflg[i] & SPRDIR_CONSTANT:
                S.stroke0[i] = dif[0] * d[0] + dif[1] * d[1] + dif[2] * d[2]
            else:
                dot = dif[0] * d[0] + dif[1] * d[1] + dif[2] * d[2]
                dif = [dif[0] - dot * d[0], dif[1] - dot * d[1], dif[2] - dot * d[2]]
                S.stroke0[i] = math.sqrt(dif[0] * dif[0] + dif[1] * dif[1] + dif[2] * dif[2])
        else:
            S.sprflg[i] |= SPRDIR_FOLLOWER
            dif = [q[0] - p1[0], q[1] - p1[1], q[2] - p1[2]]
            S.stroke0[i] = math.sqrt(dif[0] * dif[0] + dif[1] * dif[1] + dif[2] * dif[2])
    if ylim is not None:
        y0, y1 = float(ylim[0]), float(ylim[1])
        if y0 > 0.0:
            raise ValueError("Compressive yield limit must be <= 0.0")
        if y1 < 0.0:
            raise ValueError("Tensile yield limit must be >= 0.0")
        S.yield_[:, i] = (y0, y1)
    else:
        S.yield_[:, i] = (0.0, 0.0)
    return i


def _lcurve_from_time_series(m, ts):
    """lcurve_from_time_series (parmec.cpp:1239-1269): copy a TSERIES into the lookup curves once."""
    for k, t in enumerate(m.lcurves):
        if t == ts:
            return k
    m.lcurves.append(ts)
    return len(m.lcurves) - 1


def sort_springs(m):
    """sort_springs (parmec.cpp:1683-1965): order springs by (part0, part1).

    Springs with equal keys keep their creation order (stable sort)."""
    n = m.sprnum
    if n == 0:
        return
    S = m.S
    order = sorted(range(n), key=lambda i: (int(S.sprpart[0, i]), int(S.sprpart[1, i])))
    for name, (ncomp, _) in S.spec.items():
        arr = getattr(S, name)
        if ncomp:
            arr[:, :n] = arr[:, order]
        else:
            arr[:n] = arr[order]
    m.spring_tab = [m.spring_tab[i] for i in order]
    m.dashpot_tab = [m.dashpot_tab[i] for i in order]
    m.unload_tab = [m.unload_tab[i] for i in order]
    for i in range(n):
        S.sprmap[S.sprid[i]] = i


def spring_tables(m):
    """Flat lookup tables (spring[2][*], spridx, ...) in the current spring order."""
    n = m.sprnum

    def flat(tabs):
        idx = np.zeros(n + 1, dtype=np.int32)
        xs, ys = [], []
        for i, t in enumerate(tabs):
            t = t or []
            idx[i + 1] = idx[i] + len(t)
            xs += [p[0] for p in t]
            ys += [p[1] for p in t]
        arr = np.zeros((2, max(1, len(xs))), dtype=np.float64)
        arr[0, :len(xs)] = xs
        arr[1, :len(ys)] = ys
        return arr, idx

    spring, spridx = flat(m.spring_tab)
    dashpot, dashidx = flat(m.dashpot_tab)
    unload, unidx = flat(m.unload_tab)
    lcidx = np.zeros(len(m.lcurves) + 1, dtype=np.int32)
    xs, ys = [], []
    for k, ts in enumerate(m.lcurves):
        pts = m.tms[ts].points
        lcidx[k + 1] = lcidx[k] + len(pts)
        xs += [p[0] for p in pts]
        ys += [p[1] for p in pts]
    lcurve = np.zeros((2, max(1, len(xs))), dtype=np.float64)
    lcurve[0, :len(xs)] = xs
    lcurve[1, :len(ys)] = ys
    return {"spring": spring, "spridx": spridx, "dashpot": dashpot, "dashidx": dashidx,
            "unload": unload, "unidx": unidx, "lcurve": lcurve, "lcidx": lcidx}


def _eqm(m, part1, point1, part2, point2, direction):
    """eqm (parmec.ispc:423-482) on the host model."""
    P = m.P

    def block(part, point):
        Jiv = P.inverse[:, part]
        A = [P.position[3, part] - point[0], P.position[4, part] - point[1], P.position[5, part] - point[2]]
        Ask = np.array([0, A[2], -A[1], -A[2], 0, A[0], A[1], -A[0], 0], dtype=float).reshape(3, 3).T
        J = np.array(Jiv, dtype=float).reshape(3, 3).T
        return Ask.T @ J @ Ask + P.invm[part] * np.eye(3)

    Miv = block(part1, point1)
    if part2 >= 0:
        Miv = Miv + block(part2, point2)
    d = np.array(direction, dtype=float)
    if d @ d > 0.0:
        return 1.0 / float(d @ (Miv @ d))
    return 1.0 / _extremum_eigenvalue([float(x) for x in Miv.T.reshape(-1)], 1)


def _triple_angle_root(r, largest):
    """cos(acos(r)/3) (largest) or cos(acos(r)/3 + 2 pi/3) as roots of the
    triple-angle identity 4c^3 - 3c = r, by Newton's method from c = 1 (or -1),
    monotone on [1/2, 1] (and [-1, -1/2]); the device and the CPU restatement
    run the same operations."""
    r = -1.0 if r < -1.0 else (1.0 if r > 1.0 else r)
    c = 1.0 if largest else -1.0
    for _ in range(100):
        f = (4.0 * c * c - 3.0) * c - r
        den = 12.0 * c * c - 3.0
        if den == 0.0:
            break
        cn = c - f / den
        if (largest and not cn < c) or (not largest and not cn > c):
            break
        c = cn
    return c


def _extremum_eigenvalue(A, minimum):
    """extremum_eigenvalue (macros.h:1539-1588) of a symmetric column-major 3x3;
    its diagonal branch returns the largest entry whichever is asked for."""
    p1 = A[3] * A[3] + A[6] * A[6] + A[7] * A[7]
    if p1 == 0.0:
        r = A[0] if A[0] > A[4] else A[4]
        return r if r > A[8] else A[8]
    q = (A[0] + A[4] + A[8]) / 3.0
    p2 = (A[0] - q) * (A[0] - q) + (A[4] - q) * (A[4] - q) + (A[8] - q) * (A[8] - q) + 2 * p1
    p = math.sqrt(p2 / 6.0)
    invp = 1.0 / p
    B = [invp * (A[0] - q), invp * A[1], invp * A[2], invp * A[3], invp * (A[4] - q), invp * A[5],
         invp * A[6], invp * A[7], invp * (A[8] - q)]
    det = (B[0] * (B[4] * B[8] - B[5] * B[7]) + B[3] * (B[2] * B[7] - B[1] * B[8])
           + B[6] * (B[1] * B[5] - B[2] * B[4]))
    return q + 2.0 * p * _triple_angle_root(0.5 * det, not minimum)
