"""Seeded synthetic scenes with the shapes, sizes and value distributions of the
benchmark configurations (the reference publishes no benchmark decks).

hopper_fill  4,096 spheres on a jittered 16^3 lattice in a 1 m box of 12
             triangles; GRANULAR spring 1e6, damping 0.2, friction 0.5;
             dt = 0.1 of the single-contact critical step (CPU-runnable case).
drum         N spheres (1,048,576 for the full case), radii log-uniform in
             [0.5, 2] mm, a bed in the lower part of a rotating cylinder of
             4,096 triangles (R = 0.5 m, L = 0.3 m, 2 rad/s about x);
             friction 0.3.
"""
import math

import numpy as np

from .model import Model


_LN2_HI = 6.93147180369123816490e-01     # ln 2 split so that k * _LN2_HI is exact for |k| < 2^20
_LN2_LO = 1.90821492927058770002e-10


def exp_ieee(x):
    """exp of a float64 array from +, -, *, / and ldexp only, so that scene
    inputs are the same bits on every IEEE-754 host (vectorised libm exp
    differs in the last bit between x86 and Arm builds of numpy).  Cody-Waite
    reduction x = k ln 2 + r, |r| <= ln(2)/2, then the Taylor series of e^r to
    the 20th power in Horner form (truncation below 1e-28)."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x / 0.6931471805599453)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.ones_like(r)
    for n in range(20, 0, -1):
        p = 1.0 + p * r / n
    return np.ldexp(p, k.astype(np.int64))


def log_ieee(x):
    """Natural log of a positive float (scalar) from basic operations only:
    x = m 2^e with m in [1/sqrt 2, sqrt 2), ln x = e ln 2 + 2 atanh((m-1)/(m+1))."""
    m, e = math.frexp(float(x))
    if m < 0.7071067811865476:
        m, e = 2.0 * m, e - 1
    t = (m - 1.0) / (m + 1.0)
    t2, term, acc = t * t, t, 0.0
    for n in range(1, 60, 2):
        acc += term / n
        term *= t2
    return (e * _LN2_HI + 2.0 * acc) + e * _LN2_LO


def log_uniform(rng, lo, hi, size):
    """Log-uniform draws in [lo, hi] with exp_ieee/log_ieee (host-independent bits)."""
    return exp_ieee(rng.uniform(log_ieee(lo), log_ieee(hi), size=size))


def critical_step(kn, m_min, xi):
    """Single-contact critical step h = (2/w)(sqrt(1+xi^2) - xi), w = sqrt(kn/m)
    (the LS-DYNA form used by parmec.ispc:300-379)."""
    w = math.sqrt(kn / m_min)
    return (2.0 / w) * (math.sqrt(1.0 + xi * xi) - xi)


def box_triangles(lo, hi):
    """12 triangles of an axis-aligned box."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),
         (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]
    quads = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (3, 2, 6, 7), (0, 3, 7, 4), (1, 2, 6, 5)]
    tris = []
    for a, b, c, d in quads:
        tris.append(v[a] + v[b] + v[c])
        tris.append(v[a] + v[c] + v[d])
    return [tuple(float(x) for x in t) for t in tris]


def hopper_fill(n_side=16, seed=0, spacing=0.045, jitter=0.005, rmin=0.01, rmax=0.02, density=2500.0,
                kn=1e6, damper=0.2, friction=0.5, box=1.0):
    """Config 0: returns (model, dt)."""
    rng = np.random.default_rng(seed)
    m = Model()
    mat = m.material(density, 1e9, 0.25)
    n = n_side ** 3
    g = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), np.arange(n_side), indexing="ij"), -1)
    g = g.reshape(-1, 3)[:, ::-1].astype(np.float64)          # x fastest
    extent = (n_side - 1) * spacing
    org = 0.5 * (box - extent)
    centers = org + g * spacing + rng.uniform(-jitter, jitter, size=(n, 3))
    radii = rng.uniform(rmin, rmax, size=n)
    parts = m.spheres(centers, radii, mat, 1)
    v0 = rng.normal(0.0, 0.05, size=(n, 3))
    m.P.linear[:, parts[0]:parts[-1] + 1] = v0.T
    m.obstacle(box_triangles((0.0, 0.0, 0.0), (box, box, box)), 2)
    m.granular(0, 0, kn, damper, friction)
    m.set_gravity(0.0, 0.0, -9.81)
    m_min = (4.0 / 3.0) * math.pi * rmin ** 3 * density
    dt = 0.1 * critical_step(kn, m_min, damper)
    return m, dt


def cylinder_triangles(radius=0.5, length=0.3, n_theta=128, n_x=13):
    """Cylinder along x with capped ends: 2*n_theta*n_x side triangles plus two
    caps of n_theta fan + 2*n_theta ring triangles (4,096 for the defaults)."""
    tris = []
    th = np.linspace(0.0, 2.0 * math.pi, n_theta + 1)
    xs = np.linspace(-0.5 * length, 0.5 * length, n_x + 1)
    def p(x, r, t):
        return (float(x), float(r * math.cos(t)), float(r * math.sin(t)))
    for a in range(n_x):
        for b in range(n_theta):
            p0, p1 = p(xs[a], radius, th[b]), p(xs[a + 1], radius, th[b])
            p2, p3 = p(xs[a + 1], radius, th[b + 1]), p(xs[a], radius, th[b + 1])
            tris.append(p0 + p1 + p2)
            tris.append(p0 + p2 + p3)
    for x in (-0.5 * length, 0.5 * length):
        rin = 0.5 * radius
        for b in range(n_theta):
            tris.append((float(x), 0.0, 0.0) + p(x, rin, th[b]) + p(x, rin, th[b + 1]))
            q0, q1 = p(x, rin, th[b]), p(x, radius, th[b])
            q2, q3 = p(x, radius, th[b + 1]), p(x, rin, th[b + 1])
            tris.append(q0 + q1 + q2)
            tris.append(q0 + q2 + q3)
    return tris


def drum(n=1048576, seed=1, radius=0.5, length=0.3, rmin=0.5e-3, rmax=2e-3, density=2500.0,
         kn=1e6, damper=0.2, friction=0.3, omega=2.0, overlap=1e-6):
    """Config 1: returns (model, dt, info).

    Placement (random sequential addition cannot reach a dense bed, so the bed
    is built directly): radii are drawn log-uniform and sorted by size; the
    spheres are laid along rows parallel to the drum axis, each touching its
    row neighbour with a relative overlap of `overlap`; rows of one layer are
    spaced by the row's largest diameter and layers by the layer's largest
    diameter, filling the drum from the bottom up.  The achieved solid
    fraction of the bed and the initial contact count are reported in `info`.
    """
    rng = np.random.default_rng(seed)
    r = log_uniform(rng, rmin, rmax, n)
    r = np.sort(r)[::-1]
    centers = np.zeros((n, 3))
    half = 0.5 * length - rmax
    k = 0
    z = -radius + 1.2 * rmax
    bed_volume = 0.0
    while k < n:
        rlay = r[k]
        zc = z + rlay
        if zc + rlay > radius - rmax:
            raise ValueError("drum is too small for the requested sphere count")
        ychord = math.sqrt(max(0.0, (radius - 1.5 * rmax) ** 2 - zc ** 2))
        y = -ychord
        while k < n and y + 2 * r[k] <= ychord:
            rrow = r[k]
            yc = y + rrow
            # one row along x: consecutive spheres touch
            x = -half
            start = k
            while k < n:
                xc = x + r[k] if k == start else centers[k - 1, 0] + (r[k - 1] + r[k]) * (1.0 - overlap)
                if xc + r[k] > half:
                    break
                centers[k] = (xc, yc, zc)
                k += 1
            if k == start:
                break
            y += 2.0 * rrow
        bed_volume += 2 * half * 2 * ychord * 2 * rlay
        z += 2.0 * rlay
    # transverse jitter of 1e-3 r: exactly collinear rows would give contacts with
    # exactly zero tangential velocity, for which the reference's friction cap
    # divides 0 by 0 whenever the normal force turns tensile (forces.ispc:172-178)
    centers[:, 1:] += rng.uniform(-1e-3, 1e-3, size=(n, 2)) * r[:, None]
    m = Model()
    mat = m.material(density, 1e9, 0.25)
    m.spheres(centers, r, mat, 1)
    m.obstacle(cylinder_triangles(radius, length), 2, point=(0.0, 0.0, 0.0),
               angular=lambda t: (omega, 0.0, 0.0))
    m.granular(0, 0, kn, damper, friction)
    m.set_gravity(0.0, 0.0, -9.81)
    m_min = (4.0 / 3.0) * math.pi * rmin ** 3 * density
    dt = 0.1 * critical_step(kn, m_min, damper)
    solid = float(np.sum((4.0 / 3.0) * math.pi * r ** 3))
    info = {"spheres": n, "solid_volume": solid, "bed_volume": bed_volume,
            "solid_fraction": solid / bed_volume if bed_volume > 0 else 0.0,
            "drum_fill_fraction": solid / (math.pi * radius ** 2 * length), "dt": dt}
    return m, dt, info


def shaken_box(n, seed, frequency, amplitude_g):
    """A config-0 scene scaled to about n spheres (lattice side round(n^(1/3)),
    box side 1 m per 16 lattice sites) with its base excitation:
    g(t) = (A sin(2 pi f t), 0, -9.81).  Returns (model, dt, excitation)."""
    from .batch import sinusoid
    side = max(2, int(round(n ** (1.0 / 3.0))))
    m, dt = hopper_fill(n_side=side, seed=seed, box=max(1.0, side / 16.0))
    exc = sinusoid((0.0, 0.0, -9.81), (amplitude_g * 9.81, 0.0, 0.0), frequency)
    return m, dt, exc


def batch_scenes(count=512, seed=3, nmin=2048, nmax=65536):
    """Config 3: `count` shaken boxes with sphere counts log-uniform in
    [nmin, nmax], base excitation f ~ U[1,20] Hz, amplitude ~ U[0.1,1] g."""
    rng = np.random.default_rng(seed)
    ns = log_uniform(rng, nmin, nmax, count)
    fs = rng.uniform(1.0, 20.0, size=count)
    amps = rng.uniform(0.1, 1.0, size=count)
    out = []
    for k in range(count):
        out.append(shaken_box(int(ns[k]), seed * 100003 + k, float(fs[k]), float(amps[k])))
    return out


def critical_spring_step(kmax, m_eff, emax):
    """Critical step of a spring with largest curve slope kmax, effective mass
    m_eff and largest dashpot slope emax: (2/w)(sqrt(1+ksi^2) - ksi) with
    w = sqrt(kmax/m_eff), ksi = emax/(2 m_eff w) (the formula of
    critical_perspring, parmec.ispc:485-544)."""
    w = math.sqrt(kmax / m_eff)
    ksi = emax / (2.0 * m_eff * w)
    return (2.0 / w) * (math.sqrt(1.0 + ksi * ksi) - ksi)


def spring_lattice(n_side=256, seed=2, edge=0.01, gap=0.002, density=2500.0, contact_radius=0.0):
    """Config 2, the spring-lattice shaking table: n_side x n_side rigid
    hexahedral MESH particles (12 triangles each) joined to their right and
    upper neighbours by SPRINGs with 8-point random monotone force-stroke
    curves (segment slopes in [1e4, 1e6] N/m) and lookup dashpots; each cube
    hangs on one more spring from a base plate MESH particle whose motion is a
    PRESCRIBEd acceleration 0.5 g sin(2 pi 5 t) along x.  Gravity -9.81 z.
    contact_radius > 0 turns mesh-mesh contact on (Model.mesh_contact) with
    GRANULAR spring 1e4 N/m per triangle pair, damping 0.2, friction 0.3
    between the cubes and the plate: with the radius at half the gap, faces
    touch as soon as a gap closes (a cube face meets its neighbour through
    tens of triangle pairs, so the pair stiffness is kept low enough for the
    springs' step).  Returns (model, dt) with dt = 0.1 of the critical spring step."""
    from .model import Model
    from . import mesh
    rng = np.random.default_rng(seed)
    m = Model()
    mat = m.material(density, 1e9, 0.25)
    h = edge + gap
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij"), axis=-1).reshape(-1, 2)
    origins = np.zeros((len(ij), 3))
    origins[:, 0] = ij[:, 0] * h
    origins[:, 1] = ij[:, 1] * h
    parts = mesh.hex_grid(m, origins, edge, mat, 1)
    # the base plate: one flat hexahedron under the grid
    L = n_side * h
    z0 = -gap - edge
    bx = [(-gap, -gap, z0), (L, -gap, z0), (L, L, z0), (-gap, L, z0),
          (-gap, -gap, -gap), (L, -gap, -gap), (L, L, -gap), (-gap, L, -gap)]
    base = m.mesh([v for p in bx for v in p], [8, 0, 1, 2, 3, 4, 5, 6, 7, mat], mat, 1)
    idx = {(int(a), int(b)): int(p) for (a, b), p in zip(ij, parts)}
    half = 0.5 * edge
    kmax = emax = 0.0

    def curve():
        nonlocal kmax
        s = np.linspace(-0.75 * gap, 0.75 * gap, 8)
        k = rng.uniform(1e4, 1e6, 7)
        kmax = max(kmax, float(k.max()))
        f = np.concatenate([[0.0], np.cumsum(k * np.diff(s))])
        f -= np.interp(0.0, s, f)
        return [float(v) for pair in zip(s, f) for v in pair]

    m_cube = density * edge ** 3
    c = 2.0 * 0.1 * math.sqrt(5e5 * 0.5 * m_cube)
    dash = [-1.0, -c, 1.0, c]
    emax = c
    for (a, b), p in idx.items():
        cx, cy = a * h + half, b * h + half
        for da, db in ((1, 0), (0, 1)):
            q = idx.get((a + da, b + db))
            if q is None:
                continue
            pa = (cx + half * da, cy + half * db, half)
            pb = (cx + (h - half) * da, cy + (h - half) * db, half)
            m.spring(p, pa, q, pb, curve(), dashpot=dash)
        m.spring(base, (cx, cy, -gap), p, (cx, cy, 0.0), curve(), dashpot=dash)
    m.prescribe_motion(base, linear=lambda t: (0.5 * 9.81 * math.sin(2.0 * math.pi * 5.0 * t), 0.0, 0.0),
                       kind="av")
    m.set_gravity(0.0, 0.0, -9.81)
    if contact_radius > 0.0:
        m.granular(0, 0, 1e4, 0.2, 0.3)
        m.mesh_contact(contact_radius)
    dt = 0.1 * critical_spring_step(kmax, 0.5 * m_cube, emax)
    return m, dt
