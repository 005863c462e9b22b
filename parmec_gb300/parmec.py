"""The `parmec` command namespace of an input deck (input.cpp:4093-4119).

A deck calls these functions as globals, exactly as in the reference:
MATERIAL, SPHERE, MESH, ANALYTICAL, OBSTACLE, GRANULAR, SPRING, PRESCRIBE,
VELOCITY, GRAVITY, DAMPING, TSERIES, HISTORY, CRITICAL, DEM, RESET, OUTPUT,
ARGV.  They act on one process-wide Model, like the reference's globals.
"""
import sys

from .model import Model

_model = Model()
_engine_factory = None   # tests may install a different engine factory


def model():
    """The process-wide Model the commands act on."""
    return _model


def set_engine_factory(factory):
    """Use `factory(model)` to create the compute engine of the next DEM (None: the GPU session)."""
    global _engine_factory
    _engine_factory = factory


def RESET():
    if _model.engine is not None:
        _model.engine.close()
    _model.reset()


def TSERIES(points):
    return _model.tseries(points)


def MATERIAL(density, young, poisson):
    return _model.material(density, young, poisson)


def SPHERE(center, radius, material, color):
    return _model.sphere(center, radius, material, color)


def MESH(nodes, elements, material, colors):
    return _model.mesh(nodes, elements, material, colors)


def ANALYTICAL(inertia=None, mass=0.0, rotation=None, position=None, material=0, particle=-1):
    return _model.analytical(inertia, mass, rotation, position, material, particle)


def OBSTACLE(triangles, color, point=None, linear=None, angular=None):
    return _model.obstacle(triangles, color, point, linear, angular)


def GRANULAR(color1, color2, spring, damper=1.0, friction=None, rolling=0.0, drilling=0.0, kskn=0.5):
    return _model.granular(color1, color2, spring, damper, friction, rolling, drilling, kskn)


def SPRING(part1, point1, part2, geom2, spring, dashpot=None, direction=None, planar=None,
           unload=None, ylim=None, inactive=False, offset=-1, friction=0.0, kskn=0.0):
    return _model.spring(part1, point1, part2, geom2, spring, dashpot, direction, planar,
                         unload, ylim, inactive, offset, friction, kskn)


def PRESCRIBE(parnum, linear=None, angular=None, kind=None):
    return _model.prescribe_motion(parnum, linear, angular, kind)


def TORSION_SPRING(part1, part2, zdir, xdir, kroll=None, kpitch=None, kyaw=None, droll=None, dpitch=None,
                   dyaw=None, cone=None, refpnt=None):
    return _model.torsion_spring(part1, part2, zdir, xdir, kroll, kpitch, kyaw, droll, dpitch, dyaw, cone, refpnt)


def UNSPRING(tsprings, msprings, limits, entity=None, operator=None, abs=False, nsteps=1, nfreq=1, unload=-1,
             activate=None):
    return _model.unspring(tsprings, msprings, limits, entity, operator, abs, nsteps, nfreq, unload, activate)


def EQM(part1, point1, part2=-1, point2=None, direction=None):
    return _model.eqm(part1, point1, part2, point2, direction)


def RESTRAIN(parnum, linear=None, angular=None):
    return _model.restrain(parnum, linear, angular)


def VELOCITY(parnum, linear=None, angular=None):
    return _model.velocity(parnum, linear, angular)


def GRAVITY(gx, gy, gz):
    return _model.set_gravity(gx, gy, gz)


def DAMPING(linear, angular):
    return _model.set_damping(linear, angular)


def HISTORY(entity, source=None, point=None, h5file=None, h5last=False):
    if h5file is not None:
        raise NotImplementedError("HISTORY from HDF5 files is not supported (no HDF5 on this build)")
    return _model.history(entity, source, point)


def CRITICAL(perspring=-1, perparticle=-1):
    return _model.critical(perspring, perparticle)


def OUTPUT(entities=None, subset=None, mode=None, format=None):
    """OUTPUT (input.cpp:3560-3955): entities, particle subset, modes and file formats."""
    from .output import output_command
    return output_command(_model, entities, subset, mode, format)


def ARGV():
    return list(sys.argv[1:])


def DEM(duration, step, interval=None, prefix=None, adaptive=0.0):
    engine = _engine_factory(_model) if _engine_factory is not None else None
    return _model.dem(duration, step, interval, prefix, adaptive, engine=engine)


COMMANDS = ["RESET", "TSERIES", "MATERIAL", "SPHERE", "MESH", "ANALYTICAL", "OBSTACLE", "GRANULAR",
            "SPRING", "TORSION_SPRING", "UNSPRING", "EQM", "PRESCRIBE", "RESTRAIN", "VELOCITY", "GRAVITY", "DAMPING", "HISTORY", "CRITICAL", "OUTPUT",
            "ARGV", "DEM"]


def run_deck(path, argv=None):
    """parmec::input (input.cpp:4133-4196): execute a deck with the commands as globals."""
    if argv is not None:
        sys.argv = [path] + list(argv)
    if path.endswith(".py"):
        _model.out.path = path[:-3]                   # output_path (input.cpp:4141-4155)
    g = {name: globals()[name] for name in COMMANDS}
    g["__name__"] = "__main__"
    g["__file__"] = path
    with open(path) as f:
        code = compile(f.read(), path, "exec")
    exec(code, g)
    return g
