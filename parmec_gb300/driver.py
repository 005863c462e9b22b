"""The host side of dem() (parmec.cpp:2315-2530) above the C ABI.

The reference's loop re-enters Python up to four times per step
(read_gravity_and_damping, prescribe_acceleration, prescribe_velocity,
obstaclev; input.cpp:4199-4503).  With fixed steps every step time is known
before the loop starts, so this driver calls those callbacks (and evaluates
TSERIES) for all steps up front, in the same order as the reference calls
them, and ships the sampled values to the device as per-step tables.  The
device then runs the steps back to back; the host only returns to the loop
where a HISTORY sample is due.
"""
import time as _time

import numpy as np

from . import abi


def _interval(m, interval, step):
    """DEM's interval argument (input.cpp:3975-4075) -> (dt[2], dt_func[2], dt_tms[2])."""
    if interval is None:
        return [step, step], [None, None], [-1, -1]
    if isinstance(interval, tuple):
        if len(interval) != 2:
            raise ValueError("Invalid output interval")
        items = list(interval)
    else:
        items = [interval, interval]
    dt, fn, tm = [0.0, 0.0], [None, None], [-1, -1]
    for k, v in enumerate(items):
        if callable(v):
            fn[k] = v
        elif isinstance(v, int) and not isinstance(v, bool):
            if not (0 <= v < len(m.tms)):
                raise ValueError("Invalid output interval TSERIES number")
            tm[k] = v
        else:
            dt[k] = float(v)
    if dt[0] < 0.0 or dt[1] < 0.0:
        raise ValueError("Invalid, negative, output interval")
    return dt, fn, tm


def _vec3(res, what):
    if not (isinstance(res, tuple) and len(res) == 3):
        raise RuntimeError(f"{what} callback did not return a 3-tuple")
    return [float(res[0]), float(res[1]), float(res[2])]


def obstaclev(m, t):
    """obstaclev (input.cpp:4199-4244): obstacle velocities at time t."""
    ang = np.zeros(3 * max(1, m.obsnum))
    lin = np.zeros(3 * max(1, m.obsnum))
    for i in range(m.obsnum):
        if m.anghis[i] is not None:
            ang[3 * i:3 * i + 3] = _vec3(m.anghis[i](t), "Obstacle angular velocity")
        if m.linhis[i] is not None:
            lin[3 * i:3 * i + 3] = _vec3(m.linhis[i](t), "Obstacle linear velocity")
    return ang, lin


def _prescribed(m, pr, key, t):
    v = pr[key]
    if callable(v):
        return _vec3(v(t), "Prescribed motion")
    return [m.tms[v[0]](t), m.tms[v[1]](t), m.tms[v[2]](t)]


class StepTables:
    """Per-step host inputs, sampled in the reference's call order."""

    def __init__(self, m, times, step, dt, dt_func, dt_tms):
        n = len(times)
        self.stepnum = m.stepnum
        npr = len(m.prescribe)
        self.curtime = np.array(times, dtype=np.float64)
        self.gravity = np.zeros((n, 3))
        self.damping = np.zeros((n, 6))
        self.prs_lin = np.zeros((n, max(1, npr), 3))
        self.prs_ang = np.zeros((n, max(1, npr), 3))
        self.obs_ang = np.zeros((n, max(1, m.obsnum), 3))
        self.obs_lin = np.zeros((n, max(1, m.obsnum), 3))
        self.interval = np.zeros((n, 2))
        grav = list(m.gravity)
        for k, t in enumerate(times):
            # read_gravity_and_damping (input.cpp:4424-4503)
            for c in range(3):
                if m.gravfunc[c] is not None:
                    grav[c] = float(m.gravfunc[c](t))
                elif 0 <= m.gravtms[c] < len(m.tms):
                    grav[c] = m.tms[m.gravtms[c]](t)
            self.gravity[k] = grav
            if m.lindamp is not None:
                self.damping[k, 0:3] = _vec3(m.lindamp(t), "Linear damping")
            elif all(0 <= j < len(m.tms) for j in m.lindamptms):
                self.damping[k, 0:3] = [m.tms[j](t) for j in m.lindamptms]
            if m.angdamp is not None:
                self.damping[k, 3:6] = _vec3(m.angdamp(t), "Angular damping")
            elif all(0 <= j < len(m.tms) for j in m.angdamptms):
                self.damping[k, 3:6] = [m.tms[j](t) for j in m.angdamptms]
            # prescribe_acceleration (input.cpp:4247-4341)
            for i, pr in enumerate(m.prescribe):
                if pr["lin"] is not None and pr["linkind"] == 1:
                    self.prs_lin[k, i] = _prescribed(m, pr, "lin", t)
                if pr["ang"] is not None and pr["angkind"] == 1:
                    self.prs_ang[k, i] = _prescribed(m, pr, "ang", t)
            # prescribe_velocity (input.cpp:4344-4421)
            for i, pr in enumerate(m.prescribe):
                if pr["lin"] is not None and pr["linkind"] == 0:
                    self.prs_lin[k, i] = _prescribed(m, pr, "lin", t)
                if pr["ang"] is not None and pr["angkind"] == 0:
                    self.prs_ang[k, i] = _prescribed(m, pr, "ang", t)
            # current_interval / TMS intervals (parmec.cpp:2463-2479)
            for c in range(2):
                if dt_func[c] is not None:
                    dt[c] = float(dt_func[c](t))
                elif 0 <= dt_tms[c] < len(m.tms):
                    dt[c] = m.tms[dt_tms[c]](t)
            self.interval[k] = dt
            # obstaclev (curtime + step0)
            a, l = obstaclev(m, t + step)
            self.obs_ang[k] = a[:3 * max(1, m.obsnum)].reshape(-1, 3)
            self.obs_lin[k] = l[:3 * max(1, m.obsnum)].reshape(-1, 3)

    def ctab(self, b, e):
        """pg_steptab for rows [b, e) (views; keep self alive while used)."""
        t = abi.PgStepTab()
        t.nsteps = e - b
        sl = slice(b, e)
        self._views = [np.ascontiguousarray(a[sl]) for a in
                       (self.curtime, self.gravity, self.damping, self.prs_lin, self.prs_ang,
                        self.obs_ang, self.obs_lin)]
        t.curtime, t.gravity, t.damping, t.prs_lin, t.prs_ang, t.obs_ang, t.obs_lin = \
            [abi.dptr(v) for v in self._views]
        t.stepnum = self.stepnum
        return t


def step_times(curtime, duration, step):
    """Start times of the steps the reference's loop takes (parmec.cpp:2418):
    for (time = 0; time < duration; time += 0.5*(step0+step1), curtime += ...)."""
    times = []
    t = 0.0
    ct = curtime
    while t < duration:
        times.append(ct)
        inc = 0.5 * (step + step)
        t += inc
        ct += inc
    return times, ct


SPRING_ENTITIES = ("LENGTH", "STROKE", "F", "SF", "FF")


def history_rows(m):
    """(particles, spring positions) that the histories read, sorted and unique."""
    parts, sprs = set(), set()
    for h in m.histories:
        if h["ent"] == "TIME":
            continue
        if h["ent"] in SPRING_ENTITIES and h["point"] is None:
            sprs.update(int(m.S.sprmap[k]) for k in h["list"])
        else:
            parts.update(int(k) for k in h["list"])
    return sorted(parts), sorted(sprs)


def download_for_history(m, eng):
    """What the next history sample reads: a gather of its rows where the
    engine has one, else a full download."""
    if hasattr(eng, "download_rows"):
        p, s = history_rows(m)
        eng.download_rows(p, s)
    else:
        eng.download()


def output_files_now(m, eng, t, downloaded=False):
    """output_files (output.cpp:5127-5140) at time t; downloads the state first
    when a file format this build writes (DUMP, VTK) is selected.  Returns
    whether the host arrays were brought up to date."""
    from .output import OUT_FORMAT_DUMP, OUT_FORMAT_VTK, output_files
    writes = bool(m.out.format & (OUT_FORMAT_DUMP | OUT_FORMAT_VTK))
    if writes and not downloaded:
        eng.download()
    output_files(m, t)
    return writes


def sample_history(m, t):
    """output_history (output.cpp:5143-5533) for list sources."""
    P, S = m.P, m.S
    for h in m.histories:
        ent = h["ent"]
        if ent == "TIME":
            h["out"].append(t)
            continue
        if h["point"] is not None:
            k = h["list"][0]
            x = P.position[0:3, k]
            X = P.position[3:6, k]
            v = P.linear[:, k]
            o = P.angular[3:6, k]
            L = P.rotation[:, k]
            Pp = h["point"]
            Q = [Pp[0] - X[0], Pp[1] - X[1], Pp[2] - X[2]]
            p = [x[0] + (L[0] * Q[0] + L[3] * Q[1] + L[6] * Q[2]),
                 x[1] + (L[1] * Q[0] + L[4] * Q[1] + L[7] * Q[2]),
                 x[2] + (L[2] * Q[0] + L[5] * Q[1] + L[8] * Q[2])]
            a = [p[0] - x[0], p[1] - x[1], p[2] - x[2]]
            vel = [v[0] + a[1] * o[2] - a[2] * o[1], v[1] + a[2] * o[0] - a[0] * o[2],
                   v[2] + a[0] * o[1] - a[1] * o[0]]
            val = {"PX": p[0], "PY": p[1], "PZ": p[2], "PL": float(np.sqrt(np.dot(p, p))),
                   "DX": p[0] - Pp[0], "DY": p[1] - Pp[1], "DZ": p[2] - Pp[2],
                   "DL": float(np.sqrt((p[0] - Pp[0]) ** 2 + (p[1] - Pp[1]) ** 2 + (p[2] - Pp[2]) ** 2)),
                   "VX": vel[0], "VY": vel[1], "VZ": vel[2], "VL": float(np.sqrt(np.dot(vel, vel))),
                   "OX": o[0], "OY": o[1], "OZ": o[2], "OL": float(np.sqrt(np.dot(o, o))),
                   "FX": P.force[0, k], "FY": P.force[1, k], "FZ": P.force[2, k],
                   "FL": float(np.sqrt(np.dot(P.force[:, k], P.force[:, k]))),
                   "TX": P.torque[0, k], "TY": P.torque[1, k], "TZ": P.torque[2, k],
                   "TL": float(np.sqrt(np.dot(P.torque[:, k], P.torque[:, k])))}[ent]
            h["out"].append(float(val))
            continue
        value = 0.0
        for k in h["list"]:
            if ent in ("PX", "PY", "PZ"):
                value += P.position["XYZ".index(ent[1]), k]
            elif ent == "PL":
                value += float(np.sqrt(np.dot(P.position[0:3, k], P.position[0:3, k])))
            elif ent in ("DX", "DY", "DZ"):
                c = "XYZ".index(ent[1])
                value += P.position[c, k] - P.position[3 + c, k]
            elif ent == "DL":
                d = P.position[0:3, k] - P.position[3:6, k]
                value += float(np.sqrt(np.dot(d, d)))
            elif ent in ("VX", "VY", "VZ"):
                value += P.linear["XYZ".index(ent[1]), k]
            elif ent == "VL":
                value += float(np.sqrt(np.dot(P.linear[:, k], P.linear[:, k])))
            elif ent in ("OX", "OY", "OZ"):
                value += P.angular[3 + "XYZ".index(ent[1]), k]
            elif ent == "OL":
                value += float(np.sqrt(np.dot(P.angular[3:6, k], P.angular[3:6, k])))
            elif ent in ("FX", "FY", "FZ"):
                value += P.force["XYZ".index(ent[1]), k]
            elif ent == "FL":
                value += float(np.sqrt(np.dot(P.force[:, k], P.force[:, k])))
            elif ent in ("TX", "TY", "TZ"):
                value += P.torque["XYZ".index(ent[1]), k]
            elif ent == "TL":
                value += float(np.sqrt(np.dot(P.torque[:, k], P.torque[:, k])))
            else:
                l = int(S.sprmap[k])
                if ent == "LENGTH":
                    d = S.sprpnt[6:9, l] - S.sprpnt[0:3, l]
                    value += float(np.sqrt(np.dot(d, d)))
                elif ent == "STROKE":
                    value += S.stroke[0, l]
                elif ent == "F":
                    value += S.sprfrc[0, l]
                elif ent == "SF":
                    value += S.sprfrc[1, l]
                elif ent == "FF":
                    value += S.sprfrc[2, l]
        # a list source reports the mean over its entries (output.cpp:5514-5516)
        h["out"].append(float(value) / float(len(h["list"])))


def default_engine(m):
    from .engine import GpuEngine
    return GpuEngine(m)


def run_dem(m, duration, step, interval, engine, adaptive=0.0):
    """dem() (parmec.cpp:2315-2530); 0 < adaptive <= 1 selects adaptive steps."""
    from .springs import sort_springs
    t_start = _time.perf_counter()
    dt, dt_func, dt_tms = _interval(m, interval, step)
    m.sort_materials()
    if m.springs_changed:
        sort_springs(m)
        m.springs_changed = False
    if m.torsion_changed:
        from .torsion import sort_torsion
        sort_torsion(m)
        m.torsion_changed = False

    eng = engine if engine is not None else m.engine
    if eng is None or eng.model is not m or eng.stale():
        if eng is not None and eng is m.engine:
            eng.close()
        eng = engine if engine is not None else default_engine(m)
        eng.attach(m)
    elif m._dirty:
        eng.upload()
    if engine is None:
        m.engine = eng
    m.last_engine = eng
    m._dirty = False

    if m.curtime == 0.0:
        step0 = step
        output_files_now(m, eng, m.curtime, downloaded=True)
        sample_history(m, m.curtime)
        a, l = obstaclev(m, 0.5 * step0)
        eng.first_half_step(step0, a, l)
    else:
        step0 = m.curstep
    eng.invert_inertia()
    if m.restraints:
        eng.restrain_velocities()                       # parmec.cpp:2413

    if 0.0 < adaptive <= 1.0:
        return _run_adaptive(m, eng, duration, step0, adaptive, dt, dt_func, dt_tms, t_start)

    times, end_time = step_times(m.curtime, duration, step0)
    tabs = StepTables(m, times, step0, list(dt), dt_func, dt_tms)

    # output and history cadence (parmec.cpp:2482-2511): after step k, files
    # when t_k >= curtime_output + interval[0], a history sample when
    # t_k >= curtime_history + interval[1]
    cuts = []
    co, ch = m.curtime_output, m.curtime_history
    for k, t in enumerate(times):
        o = t >= co + tabs.interval[k, 0]
        if o:
            co += tabs.interval[k, 0]
        h = t >= ch + tabs.interval[k, 1]
        if h:
            ch += tabs.interval[k, 1]
        if o or h:
            cuts.append((k, o, h))
    b = 0
    for k, o, h in cuts:
        eng.run(tabs.ctab(b, k + 1), step0)
        got = False
        if o:
            got = output_files_now(m, eng, times[k])
            m.curtime_output += tabs.interval[k, 0]
        if h:
            if not got:
                download_for_history(m, eng)
            sample_history(m, times[k])
            m.curtime_history += tabs.interval[k, 1]
        b = k + 1
    if b < len(times):
        eng.run(tabs.ctab(b, len(times)), step0)
    eng.download()
    m.curtime = end_time
    m.curstep = step0
    m.stepnum += 1
    return _time.perf_counter() - t_start


def _run_adaptive(m, eng, duration, step0, adaptive, dt, dt_func, dt_tms, t_start):
    """The dem() loop with adaptive steps (parmec.cpp:2418-2517): each step's
    callbacks are sampled at its start time, which depends on the previous
    step's step1, so the host runs one step per device call and advances
    time += (step0 + step1)/2 with the step1 the device chose."""
    dtl = list(dt)
    t = 0.0
    ct = m.curtime
    step1 = step0
    while t < duration:
        tabs = StepTables(m, [ct], step0, dtl, dt_func, dt_tms)
        step1 = float(eng.run_adaptive(tabs.ctab(0, 1), step0, adaptive)[0])
        got = False
        if ct >= m.curtime_output + tabs.interval[0, 0]:
            got = output_files_now(m, eng, ct)
            m.curtime_output += tabs.interval[0, 0]
        if ct >= m.curtime_history + tabs.interval[0, 1]:
            if not got:
                download_for_history(m, eng)
            sample_history(m, ct)
            m.curtime_history += tabs.interval[0, 1]
        inc = 0.5 * (step0 + step1)
        t += inc
        ct += inc
        step0 = step1
    eng.download()
    m.curtime = ct
    m.curstep = step1
    m.stepnum += 1
    return _time.perf_counter() - t_start
