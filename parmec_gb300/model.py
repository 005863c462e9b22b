"""Host-side scene model and the Parmec input commands.

The reference embeds CPython and defines the commands of its `parmec` module in
C++ (input.cpp:4093-4119).  Each command validates its arguments and appends to
global structure-of-arrays buffers (parmec.cpp:61-285).  Here the same commands
append to numpy SoA buffers of a `Model`; `DEM` hands the buffers to a compute
engine through the C ABI of libparmec_gb300.so (include/parmec_gb300.h) and
copies the advanced state back, so after `DEM` returns the host arrays hold the
same data the reference's globals would.

Only the spec commands are implemented in full: MATERIAL, SPHERE, MESH,
OBSTACLE, GRANULAR, SPRING, PRESCRIBE, HISTORY, DEM, plus GRAVITY, TSERIES,
VELOCITY, DAMPING, ANALYTICAL, RESET and CRITICAL(perspring=...), which decks
built from them need.
"""
import math
import os
import time as _time

import numpy as np

from . import abi
from .timeseries import TimeSeries

# constants.h:33-64
DENSITY, YOUNG, POISSON = 0, 1, 2
SPRING, DAMPER, FRISTAT, FRIDYN, FRIROL, FRIDRIL, KSKN = range(7)
ANALYTICAL_FLAG, OUTREST, SKIP = 1, 2, 4
SPRING_NONLINEAR_ELASTIC, SPRING_GENERAL_NONLINEAR = 0, 1
SPRING_YIELDED, SPRING_UNLOADING = 1, 2
SPRDIR_CONSTANT, SPRDIR_PLANAR, SPRDIR_FOLLOWER, SPRDIR_PROJECT = 4, 8, 16, 32
REAL_MAX = 1.7976931348623157E+308

HISTORY_ENTITIES = {
    "TIME": ("TIME", 0), "PX": ("PX", 0), "PY": ("PY", 0), "PZ": ("PZ", 0), "|P|": ("PL", 0),
    "DX": ("DX", 0), "DY": ("DY", 0), "DZ": ("DZ", 0), "|D|": ("DL", 0),
    "VX": ("VX", 0), "VY": ("VY", 0), "VZ": ("VZ", 0), "|V|": ("VL", 0),
    "OX": ("OX", 0), "OY": ("OY", 0), "OZ": ("OZ", 0), "|O|": ("OL", 0),
    "FX": ("FX", 0), "FY": ("FY", 0), "FZ": ("FZ", 0), "|F|": ("FL", 0),
    "TX": ("TX", 0), "TY": ("TY", 0), "TZ": ("TZ", 0), "|T|": ("TL", 0),
    "LENGTH": ("LENGTH", 1), "STROKE": ("STROKE", 1), "F": ("F", 1), "SF": ("SF", 1), "FF": ("FF", 1),
}


class _SoA:
    """A growable set of (ncomp, capacity) arrays sharing one count."""

    def __init__(self, spec, cap):
        self.spec = dict(spec)
        self.cap = cap
        for name, (ncomp, dtype) in self.spec.items():
            shape = (ncomp, cap) if ncomp else (cap,)
            setattr(self, name, np.zeros(shape, dtype=dtype))

    def ensure(self, n):
        if n <= self.cap:
            return False
        cap = self.cap
        while cap < n:
            cap *= 2
        for name, (ncomp, dtype) in self.spec.items():
            old = getattr(self, name)
            shape = (ncomp, cap) if ncomp else (cap,)
            new = np.zeros(shape, dtype=dtype)
            new[..., :self.cap] = old
            setattr(self, name, new)
        self.cap = cap
        return True


def _is_tuple(x, n):
    return isinstance(x, tuple) and len(x) == n


class Model:
    """One Parmec scene: the reference's global state, as numpy SoA buffers."""

    def __init__(self):
        self.reset()

    # ------------------------------------------------------------------ RESET
    def reset(self):
        """RESET (input.cpp:610-623): drop all data, contacts and time."""
        f8, i4 = np.float64, np.int32
        self.P = _SoA({"angular": (6, f8), "linear": (3, f8), "rotation": (9, f8), "position": (6, f8),
                       "inertia": (9, f8), "inverse": (9, f8), "mass": (0, f8), "invm": (0, f8),
                       "force": (3, f8), "torque": (3, f8), "flags": (0, i4), "parmat": (0, i4)}, 256)
        self.E = _SoA({"center": (6, f8), "radii": (3, f8), "ellcol": (0, i4), "part": (0, i4)}, 256)
        self.tt_radius = 0.0                  # mesh-mesh contact (mesh_contact); 0: off
        self.Tr = _SoA({"tri": (9, f8), "tricol": (0, i4), "triobs": (0, i4)}, 256)
        self.O = _SoA({"trirng": (2, i4), "obspnt": (3, f8), "obsang": (3, f8), "obslin": (3, f8)}, 16)
        self.N = _SoA({"nodes": (6, f8), "nodpart": (0, i4)}, 256)
        self.F = _SoA({"facnod": (3, i4), "factri": (0, i4)}, 256)
        self.S = _SoA({"sprtype": (0, i4), "unspring": (0, i4), "sprpart": (2, i4), "sprpnt": (12, f8),
                       "spridx": (0, i4), "dashidx": (0, i4), "unidx": (0, i4), "yield_": (2, f8),
                       "sprdir": (6, f8), "sprflg": (0, i4), "sproffset": (0, i4), "sprfric": (0, f8),
                       "sprkskn": (0, f8), "sprsdsp": (3, f8), "stroke0": (0, f8), "stroke": (3, f8),
                       "sprfrc": (3, f8), "sprid": (0, i4), "sprmap": (0, i4)}, 64)
        self.Q = _SoA({"tsprpart": (2, i4), "zdir0": (3, f8), "xdir0": (3, f8), "zdir1": (3, f8),
                       "xdir1": (3, f8), "rpy": (3, f8), "rpytot": (3, f8), "rpyspr": (3, f8),
                       "refpnt": (3, f8), "cone": (0, i4), "tsprid": (0, i4), "tsprmap": (0, i4)}, 16)
        self.parnum = self.ellnum = self.trinum = self.obsnum = 0
        self.nodnum = self.facnum = self.sprnum = self.trqsprnum = 0
        # spheres, mesh faces and triangles of analytical particles sit in
        # front of the arrays, out of contact detection and the shape
        # updates (ellcon, faccon, tricon, parmec.cpp:87-93, 1401-1592)
        self.ellcon = self.faccon = self.tricon = 0
        self.krpy_tab, self.drpy_tab = [], []   # per torsion spring: three (angle|rate, torque) tables
        self.torsion_changed = False
        self.mparam = []                    # [density, young, poisson]
        self.pairs = [(0, 0)]               # pair_reset (parmec.cpp:375-388)
        self.ikind = [0]
        self.iparam = [[0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.5]]
        self.linhis, self.anghis = [], []   # obstacle callbacks
        self.spring_tab = []                # per spring (stroke,force) pairs
        self.dashpot_tab = []
        self.unload_tab = []
        self.tms = []                       # TSERIES objects
        self.lcurves = []                   # time series copied as lookup curves (sproffset)
        self.prescribe = []                 # dicts: part, lin, ang, linkind, angkind
        self.restraints = []                # (part, lin[9], ang[9]) orthonormal direction rows
        self.body_forces = {}               # particle -> outer force xyz, torque xyz (coupling import)
        self.body_forces_inner = {}         # particle -> inner force xyz, torque xyz (coupling export)
        self.unsprings = []                 # UNSPRING rules (dicts); failure countdowns in unspring_nfreq
        self.unspring_nfreq = np.zeros(1, dtype=np.int32)
        self.gravity = [0.0, 0.0, 0.0]
        self.gravfunc = [None, None, None]
        self.gravtms = [-1, -1, -1]
        self.lindamp = self.angdamp = None
        self.lindamptms = [-1, -1, -1]
        self.angdamptms = [-1, -1, -1]
        self.damping = [0.0] * 6
        self.histories = []
        from .output import OutputState
        self.out = OutputState()            # OUTPUT settings and frame counter
        self.curtime = 0.0
        self.curstep = 0.0
        self.curtime_history = 0.0
        self.curtime_output = 0.0
        self.stepnum = 0
        self.springs_changed = False
        # reference defects: expmap typo and triangle edge parameter reproduced,
        # moving-obstacle index fixed
        self.compat = abi.PG_COMPAT_EXPMAP | abi.PG_COMPAT_TRIEDGE
        self.engine = None                  # compute engine holding device state
        self.last_engine = None             # engine of the latest DEM (owned or passed in)
        self._dirty = True                  # host arrays changed since the engine last saw them

    def _touch(self):
        self._dirty = True

    # ---------------------------------------------------------------- TSERIES
    def tseries(self, points):
        """TSERIES (input.cpp:626-725): constant, file path, [t,v,...], [[t,v]...] or [(t,v)...]."""
        if isinstance(points, (int, float)) and not isinstance(points, bool):
            ts = TimeSeries.constant(float(points))
        elif isinstance(points, str):
            ts = TimeSeries.from_file(points)
        elif isinstance(points, list) and points:
            if isinstance(points[0], (list, tuple)):
                ts = TimeSeries([float(p[0]) for p in points], [float(p[1]) for p in points])
            else:
                if len(points) < 4:
                    raise ValueError("Time series must have at least two points")
                n = len(points) // 2
                ts = TimeSeries([float(points[2 * i]) for i in range(n)],
                                [float(points[2 * i + 1]) for i in range(n)])
        else:
            raise TypeError("Invalid points format")
        self.tms.append(ts)
        return len(self.tms) - 1

    # --------------------------------------------------------------- MATERIAL
    def material(self, density, young, poisson):
        """MATERIAL (input.cpp:728-746)."""
        for v, n in ((density, "density"), (young, "young"), (poisson, "poisson")):
            if v <= 0:
                raise ValueError(f"'{n}' must be positive")
        self.mparam.append([float(density), float(young), float(poisson)])
        return len(self.mparam) - 1

    # ------------------------------------------------------------ particles
    def _new_particle(self):
        i = self.parnum
        if self.P.ensure(i + 1):
            pass
        self.parnum += 1
        P = self.P
        P.angular[:, i] = 0.0
        P.linear[:, i] = 0.0
        P.force[:, i] = 0.0
        P.torque[:, i] = 0.0
        return i

    def sphere(self, center, radius, material, color):
        """SPHERE (input.cpp:749-837): a one-sphere particle; returns the particle index."""
        if not _is_tuple(center, 3):
            raise TypeError("'center' must be a tuple of size 3")
        if radius <= 0:
            raise ValueError("'radius' must be positive")
        if not (0 <= material < len(self.mparam)):
            raise ValueError("'material' out of range")
        if color <= 0:
            raise ValueError("'color' must be positive")
        self._touch()
        j = self.ellnum
        self.E.ensure(j + 1)
        self.ellnum += 1
        i = self._new_particle()
        P, E = self.P, self.E
        P.parmat[i] = material
        E.part[j] = i
        c = [float(center[0]), float(center[1]), float(center[2])]
        E.center[0:3, j] = c
        E.center[3:6, j] = c
        P.position[0:3, i] = c
        P.position[3:6, i] = c
        rad = float(radius)
        E.radii[0, j] = rad
        E.radii[1, j] = -1.0
        E.radii[2, j] = -1.0
        E.ellcol[j] = color
        volume = (4. / 3.) * math.pi * rad * rad * rad
        mass = volume * self.mparam[material][DENSITY]
        P.mass[i] = mass
        P.invm[i] = 1.0 / mass
        P.rotation[:, i] = (1, 0, 0, 0, 1, 0, 0, 0, 1)
        ine = 0.4 * mass * rad * rad
        P.inertia[:, i] = (ine, 0, 0, 0, ine, 0, 0, 0, ine)
        P.inverse[:, i] = _invert(P.inertia[:, i])
        P.flags[i] = OUTREST
        return i

    def spheres(self, centers, radii, material, color):
        """Many SPHERE commands at once (same arithmetic per sphere as `sphere`).

        centers: (n, 3), radii: (n,); returns the particle indices."""
        centers = np.asarray(centers, dtype=np.float64).reshape(-1, 3)
        rad = np.asarray(radii, dtype=np.float64).reshape(-1)
        n = len(rad)
        if n == 0:
            return np.zeros(0, dtype=np.int64)
        if np.any(rad <= 0):
            raise ValueError("'radius' must be positive")
        if not (0 <= material < len(self.mparam)):
            raise ValueError("'material' out of range")
        if color <= 0:
            raise ValueError("'color' must be positive")
        self._touch()
        j0, i0 = self.ellnum, self.parnum
        self.E.ensure(j0 + n)
        self.P.ensure(i0 + n)
        self.ellnum += n
        self.parnum += n
        P, E = self.P, self.E
        js = slice(j0, j0 + n)
        ps = slice(i0, i0 + n)
        P.angular[:, ps] = 0.0
        P.linear[:, ps] = 0.0
        P.force[:, ps] = 0.0
        P.torque[:, ps] = 0.0
        P.parmat[ps] = material
        E.part[js] = np.arange(i0, i0 + n, dtype=np.int32)
        E.center[0:3, js] = centers.T
        E.center[3:6, js] = centers.T
        P.position[0:3, ps] = centers.T
        P.position[3:6, ps] = centers.T
        E.radii[0, js] = rad
        E.radii[1, js] = -1.0
        E.radii[2, js] = -1.0
        E.ellcol[js] = color
        volume = (4. / 3.) * math.pi * rad * rad * rad
        mass = volume * self.mparam[material][DENSITY]
        P.mass[ps] = mass
        P.invm[ps] = 1.0 / mass
        P.rotation[:, ps] = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)[:, None]
        ine = 0.4 * mass * rad * rad
        P.inertia[:, ps] = 0.0
        P.inertia[0, ps] = ine
        P.inertia[4, ps] = ine
        P.inertia[8, ps] = ine
        P.inverse[:, ps] = _invert_diag(ine)
        P.flags[ps] = OUTREST
        return np.arange(i0, i0 + n)

    def analytical(self, inertia=None, mass=0.0, rotation=None, position=None, material=0, particle=-1):
        """ANALYTICAL (input.cpp:1159-1364) for new particles (particle < 0), or to
        redefine the mass properties of an existing particle."""
        vin = [float(x) for x in inertia] if inertia is not None else [1.0, 1.0, 1.0, 0.0, 0.0, 0.0]
        if inertia is not None and len(vin) != 6:
            raise TypeError("'inertia' must be a list of size 6")
        vrot = [float(x) for x in rotation] if rotation is not None else [1, 0, 0, 0, 1, 0, 0, 0, 1]
        vpos = [float(x) for x in position] if position is not None else [0.0, 0.0, 0.0]
        if mass < 0:
            raise ValueError("'mass' must be non-negative")
        self._touch()
        P = self.P

        def set_inertia(i):
            J = np.zeros(9)
            J[0], J[4], J[8] = vin[0], vin[1], vin[2]
            J[1] = J[3] = vin[3]
            J[2] = J[6] = vin[4]
            J[5] = J[7] = vin[5]
            P.inertia[:, i] = J
            P.inverse[:, i] = _invert(J)

        if particle < 0:
            i = self._new_particle()
            P.parmat[i] = material
            P.position[0:3, i] = vpos
            P.position[3:6, i] = vpos
            P.rotation[:, i] = vrot
            P.mass[i] = 1.0 if mass == 0.0 else float(mass)
            P.invm[i] = 1.0 / P.mass[i]
            set_inertia(i)
        else:
            if particle >= self.parnum:
                raise ValueError("Particle index is out of range")
            self.declare_analytical(particle)
            i = particle
            if position is not None:
                P.position[0:3, i] = vpos
                P.position[3:6, i] = vpos
            if rotation is not None:
                P.rotation[:, i] = vrot
            if mass > 0.0:
                P.mass[i] = mass
                P.invm[i] = 1.0 / mass
            if inertia is not None:
                set_inertia(i)
        P.flags[i] = ANALYTICAL_FLAG | OUTREST
        return i

    def declare_analytical(self, k):
        """declare_analytical (parmec.cpp:1585-1592): particle k's spheres, or
        if it has none its mesh faces and their triangles, leave contact
        detection and the shape updates.  They move in front of the ranges
        the engines see (ellcon, faccon, tricon grow), the others keeping
        their order; obstacle triangle ranges and face-triangle indices follow
        the moved triangles.  The reference's shuffles swap every earlier
        entry with one fixed position and include one entry of the preceding
        particle in the range (parmec.cpp:1419-1423, 1515-1519), and its
        triangle swap leaves factri and the obstacles' triangle ranges
        pointing at the old positions (parmec.cpp:1541-1577); here the
        entries are moved as a stable partition instead."""
        k = int(k)
        if not (0 <= k < self.parnum):
            raise ValueError("Particle index is out of range")
        self._touch()
        c, n = self.ellcon, self.ellnum
        part = self.E.part[c:n]
        sel = np.nonzero(part == k)[0]
        if len(sel):
            order = np.concatenate([sel, np.nonzero(part != k)[0]]) + c
            for name in self.E.spec:
                a = getattr(self.E, name)
                a[..., c:n] = a[..., order]
            self.ellcon += len(sel)
            return
        f0, nf = self.faccon, self.facnum
        if nf <= f0:
            return
        owner = self.N.nodpart[self.F.facnod[0, f0:nf]]
        fsel = np.nonzero(owner == k)[0]
        if not len(fsel):
            return
        forder = np.concatenate([fsel, np.nonzero(owner != k)[0]]) + f0
        for name in self.F.spec:
            a = getattr(self.F, name)
            a[..., f0:nf] = a[..., forder]
        t0, nt = self.tricon, self.trinum
        moved = self.F.factri[f0:f0 + len(fsel)].astype(np.int64)
        mask = np.zeros(nt, dtype=bool)
        mask[moved] = True
        rest = np.nonzero(~mask[t0:nt])[0] + t0
        torder = np.concatenate([moved, rest])
        where = np.arange(nt, dtype=np.int64)              # old index -> new index
        where[torder] = np.arange(t0, nt)
        for name in self.Tr.spec:
            a = getattr(self.Tr, name)
            a[..., t0:nt] = a[..., torder]
        self.F.factri[:nf] = where[self.F.factri[:nf]]
        for o in range(self.obsnum):
            b, e = int(self.O.trirng[0, o]), int(self.O.trirng[1, o])
            if e > b:
                self.O.trirng[0, o] = where[b]
                self.O.trirng[1, o] = where[e - 1] + 1
        self.tricon += len(moved)
        self.faccon += len(fsel)

    # ---------------------------------------------------------------- MESH
    def mesh(self, nodes, elements, material, colors):
        """MESH (input.cpp:840-1156)."""
        from .mesh import mesh_command
        self._touch()
        return mesh_command(self, nodes, elements, material, colors)

    # ------------------------------------------------------------- OBSTACLE
    def obstacle(self, triangles, color, point=None, linear=None, angular=None):
        """OBSTACLE (input.cpp:1367-1437)."""
        if not isinstance(triangles, list) or not all(_is_tuple(t, 9) for t in triangles):
            raise TypeError("'triangles' must be a list of 9-tuples")
        m = len(triangles)
        if isinstance(color, list):
            if len(color) != m:
                raise ValueError("'color' list size must match the triangles")
        elif color <= 0:
            raise ValueError("'color' must be positive")
        if point is not None and not _is_tuple(point, 3):
            raise TypeError("'point' must be a tuple of size 3")
        for f, n in ((linear, "linear"), (angular, "angular")):
            if f is not None and not callable(f):
                raise TypeError(f"'{n}' must be callable")
        self._touch()
        haveobs = False
        if point is not None and (linear is not None or angular is not None):
            i = self.obsnum
            self.O.ensure(i + 1)
            self.obsnum += 1
            self.O.trirng[:, i] = (self.trinum, self.trinum + m)
            self.O.obspnt[:, i] = [float(point[0]), float(point[1]), float(point[2])]
            self.linhis.append(linear)
            self.anghis.append(angular)
            haveobs = True
        for n, t in enumerate(triangles):
            i = self.trinum
            self.Tr.ensure(i + 1)
            self.trinum += 1
            self.Tr.tri[:, i] = [float(x) for x in t]
            self.Tr.tricol[i] = color[n] if isinstance(color, list) else color
            # -k-2 for moving obstacle k; the reference writes -obsnum-2 after
            # incrementing obsnum (input.cpp:1391,1433), i.e. -k-3; the contact
            # kernel decodes -j-2 (forces.ispc:265).  The product stores -k-2;
            # PG_COMPAT_OBSIDX restores the reference's off-by-one decode.
            self.Tr.triobs[i] = -(self.obsnum - 1) - 2 if haveobs else -1

    # ------------------------------------------------------------- GRANULAR
    def granular(self, color1, color2, spring, damper=1.0, friction=None, rolling=0.0, drilling=0.0, kskn=0.5):
        """GRANULAR (input.cpp:2384-2455).  Colours > 0 create a new pair (the
        reference writes that pair's parameters to index -1 because an inner
        `int i` shadows the outer one, input.cpp:2424-2445; the product stores
        them in the new pair)."""
        if spring <= 0:
            raise ValueError("'spring' must be positive")
        if damper < 0 or rolling < 0 or drilling < 0:
            raise ValueError("'damper', 'rolling' and 'drilling' must be non-negative")
        if kskn <= 0:
            raise ValueError("'kskn' must be positive")
        if friction is None:
            raise TypeError("'friction' must be given")
        if isinstance(friction, tuple):
            if len(friction) != 2:
                raise TypeError("'friction' must be a number or a tuple of size 2")
            fri = (float(friction[0]), float(friction[1]))
        else:
            fri = (float(friction), float(friction))
        if fri[0] < 0 or fri[1] < 0:
            raise ValueError("'friction' must be non-negative")
        self._touch()
        if color1 == 0 and color2 == 0:
            i = 0
        elif color1 > 0 and color2 > 0:
            self.pairs.append((min(color1, color2), max(color1, color2)))
            self.ikind.append(0)
            self.iparam.append([0.0] * 7)
            i = len(self.pairs) - 1
        else:
            raise ValueError("Invalid color values")
        self.ikind[i] = 0
        self.iparam[i] = [float(spring), float(damper), fri[0], fri[1], float(rolling), float(drilling), float(kskn)]

    # --------------------------------------------------------------- SPRING
    def spring(self, part1, point1, part2, geom2, spring, dashpot=None, direction=None, planar=None,
               unload=None, ylim=None, inactive=False, offset=-1, friction=0.0, kskn=0.0):
        """SPRING (input.cpp:1440-1788): nonlinear translational spring; returns its id."""
        from .springs import spring_command
        self._touch()
        self.springs_changed = True
        return spring_command(self, part1, point1, part2, geom2, spring, dashpot, direction, planar,
                              unload, ylim, inactive, offset, friction, kskn)

    def torsion_spring(self, part1, part2, zdir, xdir, kroll=None, kpitch=None, kyaw=None, droll=None,
                       dpitch=None, dyaw=None, cone=None, refpnt=None):
        """TORSION_SPRING (input.cpp:1791-2080): roll/pitch/yaw torsion spring
        between two particles (or a particle and the ground); returns its id."""
        from .torsion import torsion_command
        return torsion_command(self, part1, part2, zdir, xdir, kroll, kpitch, kyaw, droll, dpitch, dyaw,
                               cone, refpnt)

    # ------------------------------------------------------------ PRESCRIBE
    def prescribe_motion(self, parnum, linear=None, angular=None, kind=None):
        """PRESCRIBE (input.cpp:2647-2795): callables or TSERIES triples; kind in vv/va/av/aa."""
        if not (0 <= parnum < self.parnum):
            raise ValueError("'parnum' out of range")
        for v, n in ((linear, "linear"), (angular, "angular")):
            if v is None or callable(v):
                continue
            if isinstance(v, tuple):
                if len(v) != 3:
                    raise ValueError(f"'{n}' tuple size != 3")
                if any(not (0 <= int(k) < len(self.tms)) for k in v):
                    raise ValueError(f"'{n}' time series number out of range")
            else:
                raise ValueError(f"'{n}' is neither a tuple nor a callback")
        if kind is None:
            kind = "vv"
        if kind not in ("vv", "va", "av", "aa"):
            raise ValueError("Invalid time history kind")
        if linear is None and angular is None:
            return
        self._touch()
        self.prescribe.append({"part": parnum, "lin": linear, "ang": angular,
                               "linkind": 0 if kind[0] == "v" else 1,
                               "angkind": 0 if kind[1] == "v" else 1})

    # ---------------------------------------------------- coupling interface
    def set_body_force(self, particle, force=(0.0, 0.0, 0.0), torque=(0.0, 0.0, 0.0)):
        """A prescribed body force (struct prescribed_body_force, parmec.h:281-289):
        each step of the next DEM calls adds 'force' and 'torque' to the
        particle's after the contact and spring forces, and records the
        particle's own force and torque before that addition (body_force_inner).
        None removes the record."""
        if not (0 <= particle < self.parnum):
            raise ValueError("'particle' out of range")
        self._touch()
        if force is None:
            self.body_forces.pop(int(particle), None)
            self.body_forces_inner.pop(int(particle), None)
            return
        self.body_forces[int(particle)] = [float(x) for x in force] + [float(x) for x in torque]

    def body_force_inner(self, particle):
        """(force, torque) of the particle exported at the latest step
        (prescribe_body_forces, parmec.cpp:2202-2224)."""
        v = self.body_forces_inner.get(int(particle))
        return None if v is None else (tuple(v[:3]), tuple(v[3:]))

    # ------------------------------------------------------------------ EQM
    def eqm(self, part1, point1, part2=-1, point2=None, direction=None):
        """EQM (input.cpp:2336-2381): the equivalent point mass of one particle
        (or of a particle pair) at the given points, along 'direction' or, with
        none, from the smallest eigenvalue of the inverse mass matrix
        (eqm, parmec.ispc:423-482)."""
        from .springs import _eqm
        if not (0 <= part1 < self.parnum):
            raise ValueError("'part1' out of range")
        for v, n in ((point1, "point1"), (point2, "point2"), (direction, "direction")):
            if v is not None and not _is_tuple(v, 3):
                raise TypeError(f"'{n}' must be a tuple of size 3")
        if part2 >= self.parnum:
            raise ValueError("Particle number 'part2' is out of range")
        if part2 >= 0 and point2 is None:
            raise TypeError("'point2' must be a tuple of size 3")
        p1 = [float(x) for x in point1]
        p2 = [float(x) for x in point2] if part2 >= 0 else [0.0, 0.0, 0.0]
        d = [float(x) for x in direction] if direction is not None else [0.0, 0.0, 0.0]
        return float(_eqm(self, part1, p1, part2 if part2 >= 0 else -1, p2, d))

    # ------------------------------------------------------------- RESTRAIN
    def restrain(self, parnum, linear=None, angular=None):
        """RESTRAIN (input.cpp:2458-2644): up to three linear and three angular
        directions along which the particle's motion is removed; lists of 3, 6
        or 9 numbers, orthonormalised in order (Gram-Schmidt, NORMALIZE divides
        by the length as macros.h:427 does)."""
        if not (0 <= parnum < self.parnum):
            raise ValueError("'parnum' out of range")
        for v, n in ((linear, "linear"), (angular, "angular")):
            if v is not None and not isinstance(v, list):
                raise TypeError(f"'{n}' must be a list")

        def dirs(v, what):
            if v is None:
                return [0.0] * 9
            if len(v) not in (3, 6, 9):
                raise ValueError(f"Invalid {what} constrained directions list")
            d = [[0.0] * 3 for _ in range(3)]
            for k in range(len(v) // 3):
                d[k] = [float(v[3 * k]), float(v[3 * k + 1]), float(v[3 * k + 2])]

            def normalize(a):
                ln = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
                return [a[0] / ln, a[1] / ln, a[2] / ln]

            def submul(a, dot, b):
                return [a[0] - dot * b[0], a[1] - dot * b[1], a[2] - dot * b[2]]

            def dot3(a, b):
                return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
            d[0] = normalize(d[0])
            if len(v) >= 6:
                d[1] = normalize(submul(d[1], dot3(d[0], d[1]), d[0]))
            if len(v) == 9:
                d[2] = submul(d[2], dot3(d[0], d[2]), d[0])
                d[2] = normalize(submul(d[2], dot3(d[1], d[2]), d[1]))
            return d[0] + d[1] + d[2]
        lin = dirs(linear, "linear")
        ang = dirs(angular, "angular")
        if linear is None and angular is None:
            return
        self._touch()
        self.restraints.append((int(parnum), lin, ang))

    # ------------------------------------------------------------- UNSPRING
    UNSPRING_ENTITIES = {"STROKE": 25, "F": 26, "SF": 27, "FF": 28}   # HIS_* codes (constants.h:43-46)
    UNSPRING_OPERATORS = {"SUM": 0, "MAX": 1, "MIN": 2}             # OP_* codes (constants.h:70)

    def unspring(self, tsprings, msprings, limits, entity=None, operator=None, abs=False, nsteps=1, nfreq=1,
                 unload=-1, activate=None):
        """UNSPRING (input.cpp:2083-2295): when the SUM/MIN/MAX of an entity over
        the tested springs leaves 'limits' nfreq times (checked every nsteps),
        the monitored springs fail (zero force, or unload along a TSERIES
        curve) and the springs in 'activate' switch on; returns the rule index."""
        from .springs import _lcurve_from_time_series
        if not isinstance(tsprings, list) or not isinstance(msprings, list):
            raise TypeError("'tsprings' and 'msprings' must be lists")
        if not (isinstance(limits, tuple) and len(limits) == 2):
            raise TypeError("'limits' must be a tuple of size 2")
        if activate is not None and not isinstance(activate, list):
            raise TypeError("'activate' must be a list")
        if not isinstance(abs, bool):
            raise TypeError("'abs' must be a boolean")
        if nsteps <= 0 or nfreq <= 0:
            raise ValueError("'nsteps' and 'nfreq' must be positive")
        if unload < -1 or unload >= len(self.tms):
            raise ValueError("unload TSERIES index is out of range")
        if unload >= 0:
            pts = self.tms[unload].points
            for j in range(1, len(pts)):
                if (pts[j][1] - pts[j - 1][1]) / (pts[j][0] - pts[j - 1][0]) <= 0.0:
                    raise ValueError("Unloading curve must be monotonically increasing")
        S = self.S
        for j in tsprings:
            if not (0 <= j < self.sprnum):
                raise ValueError("tsprings SPRING index is out of range")
        for j in msprings:
            if not (0 <= j < self.sprnum):
                raise ValueError("msprings SPRING index is out of range")
            u = S.unspring[S.sprmap[j]]
            if u == -2:
                raise ValueError(f"in msprings, spring index {j} already in use by an earlier UNSPRING call")
            if u == -1:
                raise ValueError(f"in msprings, trying to use an inactive SPRING with index {j}")
        lim = []
        for k, v in enumerate(limits):
            if v is None:
                lim.append(-REAL_MAX if k == 0 else REAL_MAX)
            elif isinstance(v, (int, float)) and not isinstance(v, bool):
                lim.append(float(v))
            else:
                raise ValueError("Invalid lower limit" if k == 0 else "Invalid upper limit")
        if lim[0] >= lim[1]:
            raise ValueError("Lower limit >= upper limit")
        ent = self.UNSPRING_ENTITIES.get(entity if entity is not None else "SF")
        if ent is None:
            raise ValueError("Invalid entity")
        op = self.UNSPRING_OPERATORS.get(operator if operator is not None else "SUM")
        if op is None:
            raise ValueError("Invalid operator")
        for j in (activate or []):
            if not (0 <= j < self.sprnum) or S.unspring[S.sprmap[j]] != -1:
                raise ValueError(f"in activate list: SPRING {j} is already active")
        self._touch()
        for j in msprings:
            S.unspring[S.sprmap[j]] = -2                # in use by UNSPRING
        action = unload if unload < 0 else _lcurve_from_time_series(self, unload)
        self.unsprings.append({"tsprings": [int(j) for j in tsprings], "msprings": [int(j) for j in msprings],
                               "activate": [int(j) for j in (activate or [])], "limits": lim, "entity": ent,
                               "op": op, "abs": 1 if abs else 0, "nsteps": int(nsteps), "action": int(action)})
        nf = np.zeros(len(self.unsprings), dtype=np.int32)
        nf[:len(self.unsprings) - 1] = self.unspring_nfreq[:len(self.unsprings) - 1]
        nf[-1] = int(nfreq)
        self.unspring_nfreq = nf
        return len(self.unsprings) - 1

    # ------------------------------------------------------------- VELOCITY
    def velocity(self, parnum, linear=None, angular=None):
        """VELOCITY (input.cpp:2798-2837)."""
        if not (0 <= parnum < self.parnum):
            raise ValueError("'parnum' out of range")
        self._touch()
        P = self.P
        i = parnum
        if linear is not None:
            if not _is_tuple(linear, 3):
                raise TypeError("'linear' must be a tuple of size 3")
            P.linear[:, i] = [float(x) for x in linear]
        if angular is not None:
            if not _is_tuple(angular, 3):
                raise TypeError("'angular' must be a tuple of size 3")
            o = [float(x) for x in angular]
            P.angular[3:6, i] = o
            L = P.rotation[:, i]
            P.angular[0, i] = L[0] * o[0] + L[1] * o[1] + L[2] * o[2]   # TVMUL (macros.h:966)
            P.angular[1, i] = L[3] * o[0] + L[4] * o[1] + L[5] * o[2]
            P.angular[2, i] = L[6] * o[0] + L[7] * o[1] + L[8] * o[2]

    # -------------------------------------------------------------- GRAVITY
    def set_gravity(self, gx, gy, gz):
        """GRAVITY (input.cpp:2840-2933): float, callable or TSERIES number per component."""
        for k, g in enumerate((gx, gy, gz)):
            if callable(g):
                self.gravfunc[k] = g
                self.gravtms[k] = -1
            elif isinstance(g, float):
                self.gravity[k] = g
            elif isinstance(g, int) and not isinstance(g, bool):
                if not (0 <= g < len(self.tms)):
                    raise ValueError(f"Invalid TSERIES number for g{'xyz'[k]}")
                self.gravtms[k] = g
                self.gravfunc[k] = None
            else:
                raise ValueError(f"Invalid g{'xyz'[k]} component")

    # -------------------------------------------------------------- DAMPING
    def set_damping(self, linear, angular):
        """DAMPING (input.cpp:2936-3031): callables or TSERIES triples."""
        for v, n in ((linear, "linear"), (angular, "angular")):
            if callable(v):
                continue
            if isinstance(v, tuple):
                if len(v) != 3:
                    raise ValueError(f"Invalid {n} damping tuple size")
                if any(not (0 <= int(k) < len(self.tms)) for k in v):
                    raise ValueError(f"Invalid TSERIES number in {n} damping tuple")
            else:
                raise ValueError(f"Invalid {n} damping argument type")
        if callable(linear):
            self.lindamp, self.lindamptms = linear, [-1, -1, -1]
        else:
            self.lindamp, self.lindamptms = None, [int(k) for k in linear]
        if callable(angular):
            self.angdamp, self.angdamptms = angular, [-1, -1, -1]
        else:
            self.angdamp, self.angdamptms = None, [int(k) for k in angular]

    # -------------------------------------------------------------- HISTORY
    def history(self, entity, source=None, point=None):
        """HISTORY (input.cpp:3157-3557) for particle and linear-spring entities with
        list or single-index sources (optionally a body point); returns the list
        that DEM appends to (output.cpp:5143-5533)."""
        if entity not in HISTORY_ENTITIES:
            raise ValueError("Invalid entity")
        ent, srckind = HISTORY_ENTITIES[entity]
        if source is None:
            if not self.parnum:
                raise ValueError("No particle has been defined")
            lst = [0]
        elif isinstance(source, int):
            lst = [source]
        elif isinstance(source, list):
            lst = [int(x) for x in source]
        else:
            raise ValueError("sphere and box history sources are not supported")
        for k in lst:
            if srckind == 0 and ent != "TIME" and not (0 <= k < self.parnum):
                raise ValueError("Particle index out of range")
            if srckind == 1 and not (0 <= k < self.sprnum):
                raise ValueError("Spring index out of range")
        pnt = None
        if point is not None:
            if not _is_tuple(point, 3):
                raise TypeError("'point' must be a tuple of size 3")
            if len(lst) == 1:
                pnt = [float(x) for x in point]
        out = []
        self.histories.append({"ent": ent, "list": lst, "point": pnt, "out": out})
        return out

    # ------------------------------------------------------------- CRITICAL
    def mesh_contact(self, radius):
        """Mesh-mesh contact, an extension with no counterpart in the
        reference (its contact detection holds spheres only, so MESH
        particles meet spheres but never each other): every triangle of a
        MESH particle is swept by a sphere of 'radius', and triangles of
        different particles closer than 2 * radius touch, under the GRANULAR
        law of their colours.  0 (the default) turns it off."""
        r = float(radius)
        if not (r >= 0.0) or r != r:
            raise ValueError("'radius' must be non-negative")
        self.tt_radius = r

    def critical(self, perspring=-1, perparticle=-1, engine=None):
        """CRITICAL (input.cpp:3034-3154): per-spring and per-particle critical
        step estimates.  perspring=N returns the N smallest spring steps as
        (step, index, omega, ratio), perparticle=N the N smallest particle steps
        likewise, both a tuple of the two lists, and no argument the smallest
        particle step (REAL_MAX while no contact or spring restrains anything,
        as in the reference).  The estimates run on the device
        (pg_session_critical) of 'engine', else of the session the last DEM
        call stepped this model with (its contacts), else of a session opened
        for the query (springs only: no contact exists before DEM)."""
        if perspring < -1 or perspring > self.sprnum:
            raise ValueError("Parameter 'perspring' is out of range")
        if perparticle < -1 or perparticle > self.parnum:
            raise ValueError("Parameter 'perparticle' is out of range")
        if self.springs_changed:
            from .springs import sort_springs
            self.sort_materials()
            sort_springs(self)
            self.springs_changed = False
        eng, temp = engine, None
        if eng is None:
            last = self.last_engine
            if last is not None and last.model is self and not last.stale() and hasattr(last, "critical"):
                eng = last
        if eng is None:
            from .engine import GpuEngine
            self.sort_materials()
            eng = temp = GpuEngine()
            eng.attach(self)
        try:
            out_s = out_p = None
            if perspring >= 0:
                h, o, r = eng.critical(1)
                order = sorted(range(self.sprnum), key=lambda i: (h[i], i))
                out_s = [(float(h[i]), i, float(o[i]), float(r[i])) for i in order[:perspring]]
            if perparticle >= 0 or out_s is None:
                h, o, r = eng.critical(0)
                order = sorted(range(self.parnum), key=lambda i: (h[i], i))
                if perparticle >= 0:
                    out_p = [(float(h[i]), i, float(o[i]), float(r[i])) for i in order[:perparticle]]
        finally:
            if temp is not None:
                temp.close()
        if out_s is not None and out_p is not None:
            return (out_s, out_p)
        if out_s is not None:
            return out_s
        if out_p is not None:
            return out_p
        return float(h[order[0]]) if order else REAL_MAX

    # ------------------------------------------------------------ scene ABI
    def sort_materials(self):
        """sort_materials (parmec.cpp:1636-1663): pairs sorted by colour pair."""
        order = sorted(range(len(self.pairs)), key=lambda i: self.pairs[i])
        self.pairs = [self.pairs[i] for i in order]
        self.ikind = [self.ikind[i] for i in order]
        self.iparam = [self.iparam[i] for i in order]

    def scene(self):
        """A pg_scene whose pointers view this model's arrays (valid until the next append)."""
        from .springs import spring_tables
        s = abi.PgScene()
        P, E, Tr, O, N, F, S = self.P, self.E, self.Tr, self.O, self.N, self.F, self.S
        keep = []
        s.parnum = self.parnum
        s.angular = abi.rows(P.angular, 6)
        s.linear = abi.rows(P.linear, 3)
        s.rotation = abi.rows(P.rotation, 9)
        s.position = abi.rows(P.position, 6)
        s.inertia = abi.rows(P.inertia, 9)
        s.inverse = abi.rows(P.inverse, 9)
        s.mass = abi.dptr(P.mass)
        s.invm = abi.dptr(P.invm)
        s.force = abi.rows(P.force, 3)
        s.torque = abi.rows(P.torque, 3)
        s.flags = abi.iptr(P.flags)
        s.parmat = abi.iptr(P.parmat)
        # the engines see the spheres, triangles and faces from the contact
        # offsets on (parmec.cpp:2353-2357 passes icenter = center + ellcon)
        ec, tc, fc = self.ellcon, self.tricon, self.faccon
        s.ellnum = self.ellnum - ec
        s.center = abi.rows(E.center[:, ec:], 6)
        s.radii = abi.rows(E.radii[:, ec:], 3)
        s.ellcol = abi.iptr(E.ellcol[ec:])
        s.part = abi.iptr(E.part[ec:])
        s.trinum = self.trinum - tc
        for v in range(3):
            for d in range(3):
                s.tri[v][d] = Tr.tri[3 * v + d, tc:].ctypes.data_as(abi.D)
        s.tricol = abi.iptr(Tr.tricol[tc:])
        s.triobs = abi.iptr(Tr.triobs[tc:])
        s.obsnum = self.obsnum
        trirng = np.ascontiguousarray(O.trirng.T.reshape(-1)[:2 * max(1, O.cap)] - tc)
        obspnt = np.ascontiguousarray(O.obspnt.T.reshape(-1))
        obsang = np.ascontiguousarray(O.obsang.T.reshape(-1))
        obslin = np.ascontiguousarray(O.obslin.T.reshape(-1))
        keep += [trirng, obspnt, obsang, obslin]
        s.trirng = abi.iptr(trirng)
        s.obspnt = abi.dptr(obspnt)
        s.obsang = abi.dptr(obsang)
        s.obslin = abi.dptr(obslin)
        self._obs_views = (obspnt, obsang, obslin)
        pairs = np.array([c for p in self.pairs for c in p], dtype=np.int32)
        ikind = np.array(self.ikind, dtype=np.int32)
        iparam = np.ascontiguousarray(np.array(self.iparam, dtype=np.float64).T)
        keep += [pairs, ikind, iparam]
        s.pairnum = len(self.pairs)
        s.pairs = abi.iptr(pairs)
        s.ikind = abi.iptr(ikind)
        s.iparam = abi.rows(iparam, 7)
        s.nodnum = self.nodnum
        s.nodes = abi.rows(N.nodes, 6)
        s.nodpart = abi.iptr(N.nodpart)
        s.facnum = self.facnum - fc
        s.facnod = abi.rows(F.facnod[:, fc:], 3, abi.I)
        factri = np.ascontiguousarray(F.factri[fc:] - tc) if tc else F.factri[fc:]
        keep.append(factri)
        s.factri = abi.iptr(factri)
        s.sprnum = self.sprnum
        tabs = spring_tables(self)
        keep.append(tabs)
        s.sprtype = abi.iptr(S.sprtype)
        s.unspring = abi.iptr(S.unspring)
        s.sprpart = abi.rows(S.sprpart, 2, abi.I)
        for a in range(2):
            for k in range(6):
                s.sprpnt[a][k] = S.sprpnt[6 * a + k].ctypes.data_as(abi.D)
        s.spring = abi.rows(tabs["spring"], 2)
        s.spridx = abi.iptr(tabs["spridx"])
        s.dashpot = abi.rows(tabs["dashpot"], 2)
        s.dashidx = abi.iptr(tabs["dashidx"])
        s.unload = abi.rows(tabs["unload"], 2)
        s.unidx = abi.iptr(tabs["unidx"])
        s.yield_ = abi.rows(S.yield_, 2)
        s.sprdir = abi.rows(S.sprdir, 6)
        s.sprflg = abi.iptr(S.sprflg)
        s.sproffset = abi.iptr(S.sproffset)
        s.sprfric = abi.dptr(S.sprfric)
        s.sprkskn = abi.dptr(S.sprkskn)
        s.sprsdsp = abi.rows(S.sprsdsp, 3)
        s.stroke0 = abi.dptr(S.stroke0)
        s.stroke = abi.rows(S.stroke, 3)
        s.sprfrc = abi.rows(S.sprfrc, 3)
        s.lcurve = abi.rows(tabs["lcurve"], 2)
        s.lcidx = abi.iptr(tabs["lcidx"])
        npr = len(self.prescribe)
        prspart = np.array([p["part"] for p in self.prescribe] or [0], dtype=np.int32)
        prslin = np.array([1 if p["lin"] is not None else 0 for p in self.prescribe] or [0], dtype=np.int32)
        prsang = np.array([1 if p["ang"] is not None else 0 for p in self.prescribe] or [0], dtype=np.int32)
        linkind = np.array([p["linkind"] for p in self.prescribe] or [0], dtype=np.int32)
        angkind = np.array([p["angkind"] for p in self.prescribe] or [0], dtype=np.int32)
        keep += [prspart, prslin, prsang, linkind, angkind]
        s.prsnum = npr
        s.prspart = abi.iptr(prspart)
        s.prslin = abi.iptr(prslin)
        s.prsang = abi.iptr(prsang)
        s.linkind = abi.iptr(linkind)
        s.angkind = abi.iptr(angkind)
        s.compat = self.compat
        nr = len(self.restraints)
        rstpart = np.array([r[0] for r in self.restraints] or [0], dtype=np.int32)
        rstlin = np.ascontiguousarray(np.array([r[1] for r in self.restraints] or [[0.0] * 9], dtype=np.float64).T)
        rstang = np.ascontiguousarray(np.array([r[2] for r in self.restraints] or [[0.0] * 9], dtype=np.float64).T)
        keep += [rstpart, rstlin, rstang]
        s.rstnum = nr
        s.rstpart = abi.iptr(rstpart)
        s.rstlin = abi.rows(rstlin, 9)
        s.rstang = abi.rows(rstang, 9)
        U = self.unsprings

        def csr(key):
            idx = np.zeros(len(U) + 1, dtype=np.int32)
            for i, u in enumerate(U):
                idx[i + 1] = idx[i] + len(u[key])
            lst = np.array([j for u in U for j in u[key]] or [0], dtype=np.int32)
            return lst, idx
        tspr, tidx = csr("tsprings")
        mspr, midx = csr("msprings")
        act, aidx = csr("activate")
        unlim = np.ascontiguousarray(np.array([u["limits"] for u in U] or [[0.0, 0.0]], dtype=np.float64).T)
        unent = np.array([u["entity"] for u in U] or [0], dtype=np.int32)
        unop = np.array([u["op"] for u in U] or [0], dtype=np.int32)
        unabs = np.array([u["abs"] for u in U] or [0], dtype=np.int32)
        nsteps = np.array([u["nsteps"] for u in U] or [1], dtype=np.int32)
        unaction = np.array([u["action"] for u in U] or [0], dtype=np.int32)
        if len(self.unspring_nfreq) < max(1, len(U)):
            self.unspring_nfreq = np.zeros(max(1, len(U)), dtype=np.int32)
        keep += [tspr, tidx, mspr, midx, act, aidx, unlim, unent, unop, unabs, nsteps, unaction]
        s.unsprnum = len(U)
        s.tsprings, s.tspridx = abi.iptr(tspr), abi.iptr(tidx)
        s.msprings, s.mspridx = abi.iptr(mspr), abi.iptr(midx)
        s.activate, s.actidx = abi.iptr(act), abi.iptr(aidx)
        s.unlim = abi.rows(unlim, 2)
        s.unent, s.unop, s.unabs = abi.iptr(unent), abi.iptr(unop), abi.iptr(unabs)
        s.nsteps, s.nfreq, s.unaction = abi.iptr(nsteps), abi.iptr(self.unspring_nfreq), abi.iptr(unaction)
        s.sprmap = abi.iptr(S.sprmap)
        parts = sorted(self.body_forces)
        pbfpart = np.array(parts or [0], dtype=np.int32)
        pbfout = np.ascontiguousarray(np.array([self.body_forces[p] for p in parts] or [[0.0] * 6]).T)
        if getattr(self, "_pbfin", None) is None or self._pbfin.shape[1] != max(1, len(parts)):
            self._pbfin = np.zeros((6, max(1, len(parts))))
        keep += [pbfpart, pbfout]
        s.pbfnum = len(parts)
        s.pbfpart = abi.iptr(pbfpart)
        s.pbfout = abi.rows(pbfout, 6)
        s.pbfin = abi.rows(self._pbfin, 6)
        self._pbf_parts = parts
        from .torsion import torsion_tables
        Q = self.Q
        tt = torsion_tables(self)
        keep.append(tt)
        s.trqsprnum = self.trqsprnum
        s.trqsprpart = abi.rows(Q.tsprpart, 2, abi.I)
        s.trqzdir0 = abi.rows(Q.zdir0, 3)
        s.trqxdir0 = abi.rows(Q.xdir0, 3)
        for o in range(3):
            for c in range(2):
                s.krpy[o][c] = tt[f"krpy{o}"][c].ctypes.data_as(abi.D)
                s.drpy[o][c] = tt[f"drpy{o}"][c].ctypes.data_as(abi.D)
            s.krpyidx[o] = abi.iptr(tt[f"krpyidx{o}"])
            s.drpyidx[o] = abi.iptr(tt[f"drpyidx{o}"])
        s.trqcone = abi.iptr(Q.cone)
        s.trqzdir1 = abi.rows(Q.zdir1, 3)
        s.trqxdir1 = abi.rows(Q.xdir1, 3)
        s.trqrpy = abi.rows(Q.rpy, 3)
        s.trqrpytot = abi.rows(Q.rpytot, 3)
        s.trqrpyspr = abi.rows(Q.rpyspr, 3)
        nscene = getattr(self, "nscene", 0)
        if nscene:
            s.nscene = nscene
            s.pscene = abi.iptr(self.pscene)
            s.tscene = abi.iptr(self.tscene)
            s.oscene = abi.iptr(self.oscene)
            s.sactive = abi.iptr(self.sactive)
        s._keep = keep
        return s

    def pull_body_forces(self):
        """Copy the exported inner forces of the last scene() into body_forces_inner."""
        parts = getattr(self, "_pbf_parts", [])
        for k, p in enumerate(parts):
            self.body_forces_inner[p] = [float(x) for x in self._pbfin[:, k]]

    def pull_obstacles(self):
        """Copy obstacle point/velocity state from the flat views of the last scene()."""
        obspnt, obsang, obslin = self._obs_views
        n = self.obsnum
        self.O.obspnt[:, :n] = obspnt[:3 * n].reshape(n, 3).T
        self.O.obsang[:, :n] = obsang[:3 * n].reshape(n, 3).T
        self.O.obslin[:, :n] = obslin[:3 * n].reshape(n, 3).T

    # ------------------------------------------------------------------ DEM
    def dem(self, duration, step, interval=None, prefix=None, adaptive=0.0, engine=None):
        """DEM (input.cpp:3958-4091, parmec.cpp:2315-2530); adaptive in (0, 1]
        scales the smallest per-particle critical step into the next step.

        Returns the wall time in seconds, as the reference does."""
        from .driver import run_dem
        if duration <= 0:
            raise ValueError("'duration' must be positive")
        if step <= 0:
            raise ValueError("'step' must be positive")
        if not (0.0 <= adaptive <= 1.0):
            raise ValueError("'adaptive' must be in [0, 1]")
        if prefix is not None:
            # the output path keeps its directory and takes the prefix as its name (parmec.cpp:2328-2343)
            from .output import default_path
            base = self.out.path if self.out.path is not None else default_path()
            self.out.path = os.path.join(os.path.dirname(base), str(prefix))
        return run_dem(self, float(duration), float(step), interval, engine, float(adaptive))


def _invert(J):
    """INVERT (macros.h:1033-1050) of a column-major 3x3; zeros when singular."""
    F = [float(x) for x in J]
    det = F[0] * (F[4] * F[8] - F[5] * F[7]) + F[3] * (F[2] * F[7] - F[1] * F[8]) + (F[1] * F[5] - F[2] * F[4]) * F[6]
    if det == 0.0:
        return [0.0] * 9
    det = 1.0 / det
    return [(F[4] * F[8] - F[5] * F[7]) * det, (F[2] * F[7] - F[1] * F[8]) * det, (F[1] * F[5] - F[2] * F[4]) * det,
            (F[5] * F[6] - F[3] * F[8]) * det, (F[0] * F[8] - F[2] * F[6]) * det, (F[2] * F[3] - F[0] * F[5]) * det,
            (F[3] * F[7] - F[4] * F[6]) * det, (F[1] * F[6] - F[0] * F[7]) * det, (F[0] * F[4] - F[1] * F[3]) * det]


def _invert_diag(a):
    """INVERT (macros.h:1033-1050) of diag(a, a, a) for an array of a, as _invert computes it."""
    z = np.zeros_like(a)
    F = [a, z, z, z, a, z, z, z, a]
    det = F[0] * (F[4] * F[8] - F[5] * F[7]) + F[3] * (F[2] * F[7] - F[1] * F[8]) + (F[1] * F[5] - F[2] * F[4]) * F[6]
    det = 1.0 / det
    out = np.stack([(F[4] * F[8] - F[5] * F[7]) * det, (F[2] * F[7] - F[1] * F[8]) * det,
                    (F[1] * F[5] - F[2] * F[4]) * det, (F[5] * F[6] - F[3] * F[8]) * det,
                    (F[0] * F[8] - F[2] * F[6]) * det, (F[2] * F[3] - F[0] * F[5]) * det,
                    (F[3] * F[7] - F[4] * F[6]) * det, (F[1] * F[6] - F[0] * F[7]) * det,
                    (F[0] * F[4] - F[1] * F[3]) * det])
    return out
