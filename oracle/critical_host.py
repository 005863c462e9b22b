"""CRITICAL restated on the host (TEST INFRASTRUCTURE ONLY; input.cpp:3034-3154,
parmec.ispc:275-383, 485-900).

The oracle engine's CRITICAL and the checker of the device's
(pg_session_critical).  The per-particle critical step estimate of the
reference, over the current contacts and springs:

* critical_perparticle_contacts (parmec.ispc:547-650): per particle, the
  contacts it takes part in add the absolute contact-normal components to
  kact, their normal stiffness and damping to kmax/emax, and the rotational
  stiffness terms of the contact arm to krot;
* critical_perparticle_springs (parmec.ispc:653-857): springs add their
  direction (or an in-plane pair for PLANAR springs), largest curve slope,
  damping and arm terms;
* time_step_task (parmec.ispc:275-383): translational frequency
  sqrt(n k / m), rotational frequency from the generalised eigenproblem
  K x = lambda J x through a Cholesky factor of J, and the damped step
  (2/w)(sqrt(1+ksi^2) - ksi) of each, the smaller taken.

Positions taken (the device takes the same):
* the slave side of a contact uses the contact's own normal stiffness and
  damping; the reference reads them from slave records it never sets
  (the slave copy, forces.ispc:383-405, copies point and force only);
* springs are classified by their own dashpot and flags; the reference
  indexes dashidx and sprflg with the particle index there
  (parmec.ispc:728, 759);
* extremum_eigenvalue returns the largest eigenvalue of a diagonal matrix
  even when the smallest is asked for (macros.h:1545-1553), as in the
  reference (spheres are unaffected: their J is a multiple of I).
"""
import math

import numpy as np

from parmec_gb300.springs import _eqm, _extremum_eigenvalue, _triple_angle_root  # noqa: F401

REAL_MAX = 1.7976931348623157E+308


def pairing(m, i, j):
    """pairing (forces.ispc:98-122) over the model's sorted colour pairs."""
    p0, p1 = (i, j) if i <= j else (j, i)
    start, end = 1, len(m.pairs)
    while start < end:
        mid = ((end - start) >> 1) + start
        a, b = m.pairs[mid]
        if p0 > a or (p0 == a and p1 > b):
            if start == mid:
                break
            start = mid
        elif p0 == a and p1 == b:
            return mid
        else:
            end = mid
    return 0


def _invert(F):
    det = F[0] * (F[4] * F[8] - F[5] * F[7]) + F[3] * (F[2] * F[7] - F[1] * F[8]) + (F[1] * F[5] - F[2] * F[4]) * F[6]
    if det == 0.0:
        return [0.0] * 9
    det = 1.0 / det
    return [(F[4] * F[8] - F[5] * F[7]) * det, (F[2] * F[7] - F[1] * F[8]) * det, (F[1] * F[5] - F[2] * F[4]) * det,
            (F[5] * F[6] - F[3] * F[8]) * det, (F[0] * F[8] - F[2] * F[6]) * det, (F[2] * F[3] - F[0] * F[5]) * det,
            (F[3] * F[7] - F[4] * F[6]) * det, (F[1] * F[6] - F[0] * F[7]) * det, (F[0] * F[4] - F[1] * F[3]) * det]


def _nnmul(A, B):
    C = [0.0] * 9
    for c in range(3):
        for r in range(3):
            C[3 * c + r] = A[r] * B[3 * c] + A[3 + r] * B[3 * c + 1] + A[6 + r] * B[3 * c + 2]
    return C


def _ntmul(A, B):
    """NTMUL: A * B^T (column-major)."""
    Bt = [B[0], B[3], B[6], B[1], B[4], B[7], B[2], B[5], B[8]]
    return _nnmul(A, Bt)


def _add_arm(krot, p, L, a, transpose):
    """krot terms of an arm a (body frame: L a for contacts, L^T a for springs)."""
    if transpose:
        A = np.stack([
            L[0] * a[0] + L[1] * a[1] + L[2] * a[2],
            L[3] * a[0] + L[4] * a[1] + L[5] * a[2],
            L[6] * a[0] + L[7] * a[1] + L[8] * a[2]])
    else:
        A = np.stack([L[0] * a[0] + L[3] * a[1] + L[6] * a[2],
                      L[1] * a[0] + L[4] * a[1] + L[7] * a[2],
                      L[2] * a[0] + L[5] * a[1] + L[8] * a[2]])
    dot = A[0] * A[0] + A[1] * A[1] + A[2] * A[2]
    for k, v in enumerate((dot - A[0] * A[0], dot - A[1] * A[1], dot - A[2] * A[2],
                           -A[0] * A[1], -A[0] * A[2], -A[1] * A[2])):
        np.add.at(krot[k], p, v)


def _contact_terms(m, contacts, kact, kmax, emax, krot):
    n = len(contacts["mpart"])
    if n == 0:
        return
    P, E = m.P, m.E
    pell = np.full(m.parnum, -1, dtype=np.int64)
    pell[E.part[:m.ellnum]] = np.arange(m.ellnum)
    mp = contacts["mpart"].astype(np.int64)
    code = contacts["code"].astype(np.int64)
    pnt = contacts["point"].T
    frc = contacts["force"].T
    ci = E.center[0:3, pell[mp]]
    sph = code >= 0
    pj = np.where(sph, E.part[np.maximum(code, 0)], m.Tr.triobs[np.maximum(-code - 1, 0)]).astype(np.int64)
    # normal: the recorded one, else from the partner centre (sphere) or the
    # contact point (triangle) to the master centre
    nrm = contacts["normal"].T if "normal" in contacts else None
    if nrm is None or not np.all(np.isfinite(nrm)):
        other = np.where(sph, E.center[0:3, np.maximum(code, 0)], pnt)
        q = ci - other
        ln = np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2])
        nrm = q / np.where(ln > 0.0, ln, 1.0)
    # normal stiffness and damping of each contact (forces.ispc:125-147)
    coli = E.ellcol[pell[mp]]
    colj = np.where(sph, E.ellcol[np.maximum(code, 0)], m.Tr.tricol[np.maximum(-code - 1, 0)])
    uniq, inv = np.unique(np.stack([coli, colj]), axis=1, return_inverse=True)
    pair = np.array([pairing(m, int(a), int(b)) for a, b in uniq.T], dtype=np.int64)[inv.reshape(-1)]
    ipar = np.array(m.iparam, dtype=np.float64)
    kc = ipar[pair, 0]
    with np.errstate(divide="ignore"):
        ma = np.where(pj >= 0, 1.0 / (P.invm[mp] + P.invm[np.maximum(pj, 0)]), P.mass[mp])
    ec = ipar[pair, 1] * 2.0 * np.sqrt(kc * ma)
    L = P.rotation[:, mp]
    for k in range(3):
        np.add.at(kact[k], mp, np.abs(nrm[k]))
    np.maximum.at(kmax, mp, kc)
    np.maximum.at(emax, mp, ec)
    _add_arm(krot, mp, L, pnt - P.position[0:3, mp], False)
    # the partner particle (slave side): the force direction of -f
    s = pj >= 0
    if np.any(s):
        ps = pj[s]
        f = -frc[:, s]
        fl = np.sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
        f = np.where(fl != 0.0, f / np.where(fl != 0.0, fl, 1.0), 0.0)
        for k in range(3):
            np.add.at(kact[k], ps, np.abs(f[k]))
        np.maximum.at(kmax, ps, kc[s])
        np.maximum.at(emax, ps, ec[s])
        _add_arm(krot, ps, P.rotation[:, ps], pnt[:, s] - P.position[0:3, ps], False)


def _spring_terms(m, kact, kmax, emax, krot):
    from parmec_gb300.springs import SPRDIR_PLANAR, _eqm
    S, P = m.S, m.P
    for j in range(m.sprnum):
        i, k = int(S.sprpart[0, j]), int(S.sprpart[1, j])
        sp = m.spring_tab[j]
        kspr = 0.0
        for a in range(len(sp) - 1):
            kspr = max(abs((sp[a + 1][1] - sp[a][1]) / (sp[a + 1][0] - sp[a][0])), kspr)
        dp = m.dashpot_tab[j]
        espr = 0.0
        if len(dp) == 1:                      # critical damping ratio
            mass = _eqm(m, i, S.sprpnt[3:6, j], k, S.sprpnt[9:12, j], S.sprdir[0:3, j])
            espr = dp[0][0] * 2.0 * math.sqrt(kspr * mass)
        else:
            for a in range(len(dp) - 1):
                espr = max(abs((dp[a + 1][1] - dp[a][1]) / (dp[a + 1][0] - dp[a][0])), espr)
        d = S.sprdir[0:3, j]
        for p, pnt in ((i, S.sprpnt[0:3, j]), (k, S.sprpnt[6:9, j])):
            if p < 0:
                continue
            if d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > 0.0:
                if S.sprflg[j] & SPRDIR_PLANAR:
                    t1 = d + np.array([0.123, 0.346, 0.789])
                    t2 = np.cross(d, t1)
                    t2 = t2 * (1.0 / math.sqrt(float(np.dot(t2, t2))))
                    t1 = np.cross(t2, d)
                    for c in range(3):
                        kact[c][p] += abs(t1[c]) + abs(t2[c])
                else:
                    for c in range(3):
                        kact[c][p] += abs(d[c])
            else:
                for c in range(3):
                    kact[c][p] += 1.0
            L = P.rotation[:, p][:, None]
            a = (pnt - P.position[0:3, p])[:, None]
            _add_arm(krot, np.array([p]), L, a, True)
            kmax[p] = max(kmax[p], kspr)
            emax[p] = max(emax[p], espr)


def _triple_angle_root_v(r, largest):
    """_triple_angle_root over arrays, element by element the same operations."""
    r = np.clip(r, -1.0, 1.0)
    c = np.full(r.shape, 1.0 if largest else -1.0)
    live = np.ones(r.shape, dtype=bool)
    for _ in range(100):
        if not live.any():
            break
        f = (4.0 * c * c - 3.0) * c - r
        den = 12.0 * c * c - 3.0
        with np.errstate(divide="ignore", invalid="ignore"):
            cn = c - f / den
        step = (cn < c) if largest else (cn > c)
        live &= step & (den != 0.0)
        c = np.where(live, cn, c)
    return c


def _extremum_eigenvalue_v(A, minimum):
    """_extremum_eigenvalue over arrays A[9][n]."""
    p1 = A[3] * A[3] + A[6] * A[6] + A[7] * A[7]
    diag = np.maximum(np.maximum(A[0], A[4]), A[8])
    q = (A[0] + A[4] + A[8]) / 3.0
    p2 = (A[0] - q) * (A[0] - q) + (A[4] - q) * (A[4] - q) + (A[8] - q) * (A[8] - q) + 2 * p1
    with np.errstate(divide="ignore", invalid="ignore"):
        p = np.sqrt(p2 / 6.0)
        invp = 1.0 / p
        B = [invp * (A[0] - q), invp * A[1], invp * A[2], invp * A[3], invp * (A[4] - q), invp * A[5],
             invp * A[6], invp * A[7], invp * (A[8] - q)]
        det = (B[0] * (B[4] * B[8] - B[5] * B[7]) + B[3] * (B[2] * B[7] - B[1] * B[8])
               + B[6] * (B[1] * B[5] - B[2] * B[4]))
        gen = q + 2.0 * p * _triple_angle_root_v(np.where(p1 == 0.0, 0.0, 0.5 * det), not minimum)
    return np.where(p1 == 0.0, diag, gen)


def _time_steps(m, kact, kmax, emax, krot):
    """time_step_task (parmec.ispc:275-383) for every particle, over arrays."""
    P = m.P
    n = m.parnum
    nxyz = np.maximum(np.maximum(kact[0], kact[1]), kact[2])
    live = nxyz > 0.0
    h = np.full(n, REAL_MAX)
    om = np.zeros(n)
    ra = np.zeros(n)
    if not live.any():
        return h, om, ra
    ix = np.nonzero(live)[0]
    k = kmax[ix]
    mxyz = P.mass[ix]
    omegaxyz = np.sqrt(nxyz[ix] * k / mxyz)
    K = [k * krot[0][ix], k * krot[3][ix], k * krot[4][ix], None, k * krot[1][ix], k * krot[5][ix], None, None,
         k * krot[2][ix]]
    K[3], K[6], K[7] = K[1], K[2], K[5]
    J = [P.inertia[c, ix] for c in range(9)]
    mrot = _extremum_eigenvalue_v(J, 1)
    z = np.zeros(len(ix))
    L = [z] * 9
    L[0] = np.sqrt(J[0])
    inv = 1.0 / L[0]
    L[1] = inv * J[1]
    L[2] = inv * J[2]
    L[4] = np.sqrt(J[4] - L[1] * L[1])
    inv = 1.0 / L[4]
    L[5] = inv * (J[5] - L[2] * L[1])
    L[8] = np.sqrt(J[8] - (L[2] * L[2] + L[5] * L[5]))
    invL = _invert_v(L)
    A = _nnmul_v(invL, _ntmul_v(K, invL))
    lam = _extremum_eigenvalue_v(A, 0)
    omegarot = np.where(lam > 0.0, np.sqrt(np.maximum(lam, 0.0)), 0.0)
    damping = emax[ix]
    ratioxyz = damping / (2.0 * mxyz * omegaxyz)
    hxyz = (2.0 / omegaxyz) * (np.sqrt(1.0 + ratioxyz * ratioxyz) - ratioxyz)
    rot = omegarot > 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        ratiorot = np.where(rot, damping / (2.0 * mrot * omegarot), 0.0)
        hrot = np.where(rot, (2.0 / omegarot) * (np.sqrt(1.0 + ratiorot * ratiorot) - ratiorot), REAL_MAX)
    h[ix] = np.minimum(hxyz, hrot)
    om[ix] = np.maximum(omegaxyz, omegarot)
    ra[ix] = np.maximum(ratioxyz, ratiorot)
    return h, om, ra


def _invert_v(F):
    det = F[0] * (F[4] * F[8] - F[5] * F[7]) + F[3] * (F[2] * F[7] - F[1] * F[8]) + (F[1] * F[5] - F[2] * F[4]) * F[6]
    ok = det != 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        det = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
    return [(F[4] * F[8] - F[5] * F[7]) * det, (F[2] * F[7] - F[1] * F[8]) * det, (F[1] * F[5] - F[2] * F[4]) * det,
            (F[5] * F[6] - F[3] * F[8]) * det, (F[0] * F[8] - F[2] * F[6]) * det, (F[2] * F[3] - F[0] * F[5]) * det,
            (F[3] * F[7] - F[4] * F[6]) * det, (F[1] * F[6] - F[0] * F[7]) * det, (F[0] * F[4] - F[1] * F[3]) * det]


def _nnmul_v(A, B):
    C = [None] * 9
    for c in range(3):
        for r in range(3):
            C[3 * c + r] = A[r] * B[3 * c] + A[3 + r] * B[3 * c + 1] + A[6 + r] * B[3 * c + 2]
    return C


def _ntmul_v(A, B):
    return _nnmul_v(A, [B[0], B[3], B[6], B[1], B[4], B[7], B[2], B[5], B[8]])


def critical_perparticle(m, contacts=None):
    """Per-particle (step, omega, ratio) arrays; 'contacts' is the session's
    contact export (None or empty before any DEM step: no contacts yet)."""
    n = m.parnum
    kact = [np.zeros(n) for _ in range(3)]
    krot = [np.zeros(n) for _ in range(6)]
    kmax = np.zeros(n)
    emax = np.zeros(n)
    if contacts is not None:
        _contact_terms(m, contacts, kact, kmax, emax, krot)
    _spring_terms(m, kact, kmax, emax, krot)
    return _time_steps(m, kact, kmax, emax, krot)


def critical_perspring(m):
    """critical_perspring (parmec.ispc:485-544): per-spring critical step, omega, damping ratio."""
    S = m.S
    h, o, r = [], [], []
    for j in range(m.sprnum):
        i, k = int(S.sprpart[0, j]), int(S.sprpart[1, j])
        sp = m.spring_tab[j]
        kspr = 0.0
        for a in range(len(sp) - 1):
            kk = (sp[a + 1][1] - sp[a][1]) / (sp[a + 1][0] - sp[a][0])
            kspr = max(abs(kk), kspr)
        mspr = _eqm(m, i, S.sprpnt[3:6, j], k, S.sprpnt[9:12, j], S.sprdir[0:3, j])
        omega = math.sqrt(kspr / mspr)
        ksi = 0.0
        dp = m.dashpot_tab[j]
        if len(dp) == 1:
            ksi = dp[0][0]
        else:
            espr = 0.0
            for a in range(len(dp) - 1):
                e = (dp[a + 1][1] - dp[a][1]) / (dp[a + 1][0] - dp[a][0])
                espr = max(abs(e), espr)
            if omega > 0.0:
                ksi = espr / (2 * mspr * omega)
        h.append((2.0 / omega) * (math.sqrt(1.0 + ksi * ksi) - ksi) if omega > 0.0 else 1.0)
        o.append(omega)
        r.append(ksi)
    return h, o, r
