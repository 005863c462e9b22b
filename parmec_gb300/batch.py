"""Many independent scenes advanced together in one session.

`pool(models)` concatenates single-scene Models into one Model whose
particles, spheres, triangles and obstacles carry a scene index.  On the
device every scene keeps its own grid (cells never shared between scenes),
its own triangles and its own base excitation, so each scene's arithmetic is
the same as when it runs alone; one launch per kernel steps all of them.
"""
import numpy as np

from . import abi
from .model import Model


def pool(models, capacity=None):
    """One Model holding every scene of `models` (all with the same surface pairing).

    capacity: optional (particles, spheres, triangles, obstacles) to reserve
    room for scenes loaded later (serving)."""
    P = Model()
    P.mparam = [list(x) for x in models[0].mparam] if models else []
    if models:
        P.pairs, P.ikind, P.iparam = list(models[0].pairs), list(models[0].ikind), [list(x) for x in models[0].iparam]
    ranges = []
    for m in models:
        if (m.pairs, m.ikind, m.iparam) != (P.pairs, P.ikind, P.iparam):
            raise ValueError("every scene of a pool must use the same surface pairing (GRANULAR) table")
        if m.prescribe or m.sprnum or m.nodnum:
            raise ValueError("pooled scenes support spheres, obstacles and base excitation only")
        ranges.append(append_scene(P, m))
    P.nscene = len(models)
    P.compat = models[0].compat if models else P.compat
    P.gravity = list(models[0].gravity) if models else P.gravity
    if capacity is not None:
        reserve(P, *capacity)
    return P, ranges


def _grow_to(soa, n):
    soa.ensure(max(n, 1))


def append_scene(P, m):
    """Append scene m to pool P; returns its ranges (p0,p1,e0,e1,t0,t1,o0,o1)."""
    p0, e0, t0, o0 = P.parnum, P.ellnum, P.trinum, P.obsnum
    n, ne, nt, no = m.parnum, m.ellnum, m.trinum, m.obsnum
    for dst, src, cnt, base in ((P.P, m.P, n, p0), (P.E, m.E, ne, e0), (P.Tr, m.Tr, nt, t0), (P.O, m.O, no, o0)):
        _grow_to(dst, base + cnt)
        for name in dst.spec:
            getattr(dst, name)[..., base:base + cnt] = getattr(src, name)[..., :cnt]
    P.E.part[e0:e0 + ne] += p0
    tob = P.Tr.triobs[t0:t0 + nt]
    moving = tob <= -2
    tob[moving] = -((-tob[moving] - 2) + o0) - 2
    tob[tob >= 0] += p0
    P.O.trirng[:, o0:o0 + no] += t0
    P.linhis += list(m.linhis)
    P.anghis += list(m.anghis)
    P.parnum += n
    P.ellnum += ne
    P.trinum += nt
    P.obsnum += no
    k = len(P.scene_ranges) if hasattr(P, "scene_ranges") else 0
    _set_scene_ids(P, k, (p0, p0 + n, e0, e0 + ne, t0, t0 + nt, o0, o0 + no))
    return (p0, p0 + n, e0, e0 + ne, t0, t0 + nt, o0, o0 + no)


def _set_scene_ids(P, k, r):
    for name, size in (("pscene", P.P.cap), ("tscene", P.Tr.cap), ("oscene", P.O.cap)):
        arr = getattr(P, name, None)
        if arr is None or len(arr) < size:
            new = np.zeros(max(size, 1), dtype=np.int32)
            if arr is not None:
                new[:len(arr)] = arr
            setattr(P, name, new)
    P.pscene[r[0]:r[1]] = k
    P.tscene[r[4]:r[5]] = k
    P.oscene[r[6]:r[7]] = k
    if not hasattr(P, "scene_ranges"):
        P.scene_ranges = []
    P.scene_ranges.append(r)
    P.sactive = np.ones(len(P.scene_ranges), dtype=np.int32)


def reserve(P, particles, spheres, triangles, obstacles):
    P.P.ensure(particles)
    P.E.ensure(spheres)
    P.Tr.ensure(triangles)
    P.O.ensure(obstacles)
    for name, size in (("pscene", P.P.cap), ("tscene", P.Tr.cap), ("oscene", P.O.cap)):
        arr = getattr(P, name, None)
        new = np.zeros(max(size, 1), dtype=np.int32)
        if arr is not None:
            new[:len(arr)] = arr[:len(new)]
        setattr(P, name, new)


EXC_LEN = 32


def excitation(g0, direction, components):
    """Excitation record: g(t) = g0 + direction * sum_k amp_k sin(2 pi freq_k t + phase_k).

    components: up to 8 (amp, freq, phase) triples."""
    comps = list(components)
    if len(comps) > 8:
        raise ValueError("at most 8 sinusoid components")
    rec = np.zeros(EXC_LEN, dtype=np.float64)
    rec[0:3] = g0
    rec[3:6] = direction
    rec[6] = len(comps)
    for k, (a, f, ph) in enumerate(comps):
        rec[8 + 3 * k:11 + 3 * k] = (a, f, ph)
    return rec


def sinusoid(g0, amplitude_vector, frequency, phase=0.0):
    """A single sinusoid a*sin(2 pi f t + phase) added to g0."""
    a = np.asarray(amplitude_vector, dtype=np.float64)
    n = float(np.linalg.norm(a))
    d = a / n if n > 0 else np.array([1.0, 0.0, 0.0])
    return excitation(g0, d, [(n, frequency, phase)])


def band_noise(g0, direction, rms, fmin, fmax, seed, ncomp=8):
    """Seeded band-limited noise: ncomp sinusoids with random frequencies in
    [fmin, fmax] and phases, scaled to the given RMS acceleration."""
    rng = np.random.default_rng(seed)
    f = rng.uniform(fmin, fmax, size=ncomp)
    ph = rng.uniform(0.0, 2.0 * np.pi, size=ncomp)
    a = np.full(ncomp, rms * np.sqrt(2.0 / ncomp))
    return excitation(g0, direction, list(zip(a, f, ph)))


def extract(P, k, m):
    """Copy scene k's dynamic state from pool P back into its own Model m."""
    p0, p1, e0, e1, t0, t1, o0, o1 = P.scene_ranges[k]
    for dst, src, b, e in ((m.P, P.P, p0, p1), (m.E, P.E, e0, e1), (m.Tr, P.Tr, t0, t1), (m.O, P.O, o0, o1)):
        for name in dst.spec:
            getattr(dst, name)[..., :e - b] = getattr(src, name)[..., b:e]
    m.E.part[:e1 - e0] -= p0
    m.O.trirng[:, :o1 - o0] -= t0
    tob = m.Tr.triobs[:t1 - t0]
    moving = tob <= -2
    tob[moving] = -((-tob[moving] - 2) - o0) - 2
    tob[tob >= 0] -= p0
