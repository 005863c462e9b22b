#!/usr/bin/env python3
"""Throughput of the plain FP64 DEM step on the rotating-drum scene.

Workload: 1,048,576 spheres, radii log-uniform in [0.5, 2] mm, in a cylinder
of 4,096 triangles (R = 0.5 m, L = 0.3 m) rotating at 2 rad/s about x;
GRANULAR spring 1e6 N/m, damping 0.2, friction 0.3; dt = 0.1 of the critical
step.  One bench step = one DEM time step of the whole scene.  The scene
state (~0.6 GB) is larger than L2 (129 MB), so no flush is needed between
steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 (under torchrun) runs independent replicas, one per GPU ("replicas
only": scenes do not exchange data), and reports the aggregate.
--impl reference times the CPU restatement of the reference's ISPC path
(the reference itself cannot be built: no ispc) on all host cores.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

WORKLOAD = ("rotating drum: 1,048,576 spheres, radii log-uniform [0.5,2] mm, 4,096-triangle cylinder "
            "R=0.5 m L=0.3 m at 2 rad/s, GRANULAR kn=1e6 damping 0.2 friction 0.3, dt=0.1 critical")


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def state_bytes(m):
    """Bytes the session uploads / downloads for a scene (the arrays copied)."""
    P, E, T = m.parnum, m.ellnum, m.trinum
    up = P * 8 * (6 + 3 + 9 + 6 + 9 + 9 + 2 + 3 + 3) + P * 4 * 2 + E * (8 * 9 + 4 * 2) + T * (8 * 9 + 8)
    down = P * 8 * (6 + 3 + 9 + 6 + 9 + 1 + 3 + 3) + E * 8 * 3 + T * 8 * 9
    return up, down


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(n_spheres, threads, steps=3):
    """The oracle (restatement of the reference's ISPC path) on a bounded sample:
    the same drum scene, one untimed step, then `steps` timed steps."""
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.scenes import drum
    m, dt, _ = drum(n_spheres)
    eng = OracleEngine(threads=threads)
    m.dem(0.5 * dt, dt, interval=1e9, engine=eng)
    t0 = time.perf_counter()
    m.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    el = time.perf_counter() - t0
    return {"value": m.parnum * steps / el, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} DEM steps of the full {m.parnum}-sphere drum after one untimed step, "
                      f"{el:.1f} s"}


def mixed_form(args, ref64):
    """The mixed-precision form on the same drum: W warm-up and K timed steps,
    then its state against the FP64 form's after the same W + K steps."""
    import torch
    from parmec_gb300 import abi, driver, energy
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import drum
    m, dt, _ = drum(args.spheres)
    eng = GpuEngine(form=abi.PG_FORM_MIXED)
    eng.attach(m)
    m.engine = eng
    m._dirty = False
    m.dem(args.warmup * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    times, end_time = driver.step_times(m.curtime, args.steps * dt - 0.5 * dt, dt)
    tabs = driver.StepTables(m, times, dt, [1e9, 1e9], [None, None], [-1, -1])
    ctab = tabs.ctab(0, len(times))
    stream = torch.cuda.ExternalStream(eng.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    eng.run(ctab, dt)
    ev1.record(stream)
    ev1.synchronize()
    el_ms = ev0.elapsed_time(ev1)
    m.curtime = end_time
    eng.download()
    n = m.parnum
    dx = float(np.max(np.abs(m.P.position[0:3, :n] - ref64["x"])))
    fmax = float(np.max(np.abs(ref64["f"])))
    df = float(np.max(np.abs(m.P.force[:, :n] - ref64["f"]))) / fmax
    E = energy.total(m)
    out = {"form": "mixed: FP32 contact geometry and forces, compensated FP32 pairs for x, v, L, radii and gaps",
           "value": n * args.steps / (el_ms * 1e-3), "unit": "particle-steps/s",
           "ms_per_step": el_ms / args.steps,
           "errors_vs_fp64": {"steps": args.warmup + args.steps, "position_max_abs_m": dx,
                              "force_max_abs_rel_to_max": df,
                              "energy_rel": abs(E - ref64["E"]) / abs(ref64["E"]),
                              "kinetic_energy_rel": abs(energy.kinetic(m) - ref64["K"]) / abs(ref64["K"]),
                              "energy_definition": "kinetic + rotational + gravity potential (parmec_gb300/energy.py)"}}
    eng.close()
    return out


def batched_form(args, scenes):
    """Config 3: 512 shaken boxes (sphere counts log-uniform in [2048, 65536])
    stepped together in one session, mixed form against the plain FP64 form on
    the same GPU.  One step = one time step of every scene."""
    import torch
    from parmec_gb300 import abi, batch, driver
    from parmec_gb300.engine import GpuEngine
    steps = min(args.steps, 100)
    out = {"workload": f"{len(scenes)} shaken boxes, sphere counts log-uniform [2048,65536], "
                       "base excitation f~U[1,20] Hz, a~U[0.1,1] g", "steps": steps}
    legs = ((abi.PG_FORM_MIXED, "mixed", True), (abi.PG_FORM_MIXED, "mixed_per_phase_kernels", False),
            (abi.PG_FORM_FP64, "fp64", False))
    for form, key, fused in legs:
        models = [sc[0] for sc in scenes]
        P, _ = batch.pool(models)
        dt = scenes[0][1]
        # the fused step kernel picks its launch shape during the
        # warm-up steps (real steps; the result does not depend on the shape)
        eng = GpuEngine(form=form, capacity=(32, 32), fused=fused, autotune=fused)
        eng.attach(P)
        for k, sc in enumerate(scenes):
            eng.set_scene(k, True, excitation=sc[2], start=0)
        P.engine = eng
        P._dirty = False
        warm = max(args.warmup, 64) if fused else args.warmup
        P.dem(warm * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        times, end_time = driver.step_times(P.curtime, steps * dt - 0.5 * dt, dt)
        tabs = driver.StepTables(P, times, dt, [1e9, 1e9], [None, None], [-1, -1])
        ctab = tabs.ctab(0, len(times))
        stream = torch.cuda.ExternalStream(eng.stream())
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        eng.run(ctab, dt)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        out[key] = {"value": P.parnum * steps / (ms * 1e-3), "unit": "particle-steps/s",
                    "ms_per_step": ms / steps, "spheres": P.parnum}
        if fused:
            threads, blocks, tuned, graph = eng.fused_config()
            out[key]["kernel"] = {"fused_step": True, "threads": threads, "blocks": blocks,
                                  "autotuned": bool(tuned), "cuda_graph": bool(graph)}
        eng.close()
        del P
    # the faster of the two mixed paths (both give the same bits)
    best = max(("mixed", "mixed_per_phase_kernels"), key=lambda k: out[k]["value"])
    out["mixed_best"] = {"value": out[best]["value"], "unit": "particle-steps/s",
                         "ms_per_step": out[best]["ms_per_step"],
                         "path": "fused step kernel" if best == "mixed" else
                                 "per-phase kernels, one CUDA graph per step"}
    out["mixed_over_fp64"] = out["mixed_best"]["value"] / out["fp64"]["value"]
    return out


def spring_lattice_form(args, n_side):
    """Config 2: the spring-lattice shaking table, n_side^2 MESH cubes (12
    triangles each), 2 n (n-1) neighbour springs and n^2 base springs with
    8-point curves and lookup dashpots, prescribed base acceleration; plain
    FP64 (no contacts: the reference detects none between meshes)."""
    import torch
    from parmec_gb300 import driver
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import spring_lattice
    t0 = time.perf_counter()
    m, dt = spring_lattice(n_side)
    build_s = time.perf_counter() - t0
    eng = GpuEngine()
    m.dem(args.warmup * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    steps = min(args.steps, 200)
    times, end_time = driver.step_times(m.curtime, steps * dt - 0.5 * dt, dt)
    tabs = driver.StepTables(m, times, dt, [1e9, 1e9], [None, None], [-1, -1])
    ctab = tabs.ctab(0, len(times))
    stream = torch.cuda.ExternalStream(eng.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    eng.run(ctab, dt)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    # per kernel group, from a short profiled run of the same session
    eng.profile(True)
    nprof = 10
    times2, _ = driver.step_times(end_time, nprof * dt - 0.5 * dt, dt)
    tabs2 = driver.StepTables(m, times2, dt, [1e9, 1e9], [None, None], [-1, -1])
    eng.run(tabs2.ctab(0, len(times2)), dt)
    groups = eng.profile_read()
    eng.profile(False)
    out = {"workload": f"{n_side}x{n_side} MESH hexahedra (10 mm), {m.sprnum} springs, {m.trinum} triangles, "
                       "base 0.5 g sin(2 pi 5 t) along x, FP64", "steps": steps, "dt": dt,
           "value": m.parnum * steps / (ms * 1e-3), "unit": "particle-steps/s",
           "spring_steps_per_s": m.sprnum * steps / (ms * 1e-3), "ms_per_step": ms / steps,
           "particles": m.parnum, "springs": m.sprnum, "build_s": build_s,
           "kernel_ms": {k: round(v[0] / nprof, 4) for k, v in groups.items()}}
    eng.close()
    return out


def serving_form(args, count):
    """Config 4: a Poisson stream (200 req/s) of excitation-sweep requests
    (sphere counts log-uniform [1024, 262144], 200-5000 steps, sinusoid or
    band-limited noise), served by the continuous-batching pool (mixed and
    FP64 forms, 150 GB HBM budget) and, for comparison, by the plain FP64
    drop-in path one request at a time (a DEM() call per request)."""
    import torch
    from parmec_gb300 import abi
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.serving import Server, request_stream
    reqs = request_stream(count)
    out = {"workload": f"{count} requests, Poisson 200 req/s, spheres log-uniform [1024,262144], "
                       "steps U[200,5000], sinusoid or band-limited noise base excitation", "hbm_budget_gb": 150}
    big = max(q.model.parnum for q in reqs)
    for form, key in ((abi.PG_FORM_MIXED, "mixed_pool"), (abi.PG_FORM_FP64, "fp64_pool")):
        srv = Server(reqs[0].model, reqs[0].dt, form=form, budget_bytes=150e9, max_scenes=256,
                     max_spheres=max(big, sum(q.model.parnum for q in reqs)), max_scene_extent=4.0)
        torch.cuda.synchronize()
        res, st = srv.serve(reqs, realtime=True)
        srv.close()
        out[key] = {"p50_s": st["p50_s"], "p99_s": st["p99_s"], "throughput": st["throughput"],
                    "unit": "particle-steps/s", "wall_s": st["wall_s"], "requests": st["requests"]}
    # the plain FP64 drop-in: each request alone through DEM(), in arrival order
    t0 = time.perf_counter()
    lat, ps = [], 0
    for q in reqs:
        now = time.perf_counter() - t0
        if now < q.arrival:
            time.sleep(q.arrival - now)
        m = q.model
        m.set_gravity(0.0, 0.0, -9.81)
        eng = GpuEngine()
        m.dem(q.steps * q.dt - 0.5 * q.dt, q.dt, interval=1e9, engine=eng)
        eng.close()
        lat.append(time.perf_counter() - t0 - q.arrival)
        ps += m.parnum * q.steps
    wall = time.perf_counter() - t0
    out["fp64_dropin"] = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                          "throughput": ps / wall, "unit": "particle-steps/s", "wall_s": wall,
                          "note": "sinusoid excitation replaced by constant gravity; one DEM() per request"}
    out["mixed_pool_over_fp64_dropin"] = out["mixed_pool"]["throughput"] / out["fp64_dropin"]["throughput"]
    return out


def run_reference(args, rank, world):
    """--impl reference: the CPU restatement on all host cores, rank 0 only."""
    if rank != 0:
        return 0
    from oracle.pyoracle import OracleEngine
    from parmec_gb300.scenes import drum
    threads = os.cpu_count() or 1
    m, dt, info = drum(args.spheres)
    eng = OracleEngine(threads=threads)
    m.dem(0.5 * dt, dt, interval=1e9, engine=eng)
    if args.warmup > 1:
        m.dem((args.warmup - 1) * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    t0 = time.perf_counter()
    m.dem(args.steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    el = time.perf_counter() - t0
    v = m.parnum * args.steps / el
    line = {"impl": "reference", "metric": "particle-steps/s", "value": v, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "spheres": m.parnum},
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} DEM steps of the full drum (the reference's ISPC build "
                                       "cannot be compiled here: no ispc, no HDF5)"},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--spheres", type=int, default=1048576)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=512, help="scenes of the batched leg")
    ap.add_argument("--serving", type=int, default=48, help="requests in the serving stream (0: skip)")
    ap.add_argument("--lattice", type=int, default=256, help="side of the spring lattice (0: skip)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    import __graft_entry__
    if not os.path.exists(os.path.join(HERE, "parmec_gb300", "_build", "libparmec_gb300.so")):
        __graft_entry__.build()
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import drum
    from parmec_gb300 import driver

    m, dt, info = drum(args.spheres)
    eng = GpuEngine()
    eng.attach(m)
    m.engine = eng
    m._dirty = False
    # warm-up: the first DEM call (half step, inverse inertia) and W steps
    try:
        m.dem(args.warmup * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    except RuntimeError:
        print(json.dumps({"warmup_failure_diagnostics": eng.diagnostics()}), file=sys.stderr)
        raise

    # timed region: K steps, device resident, CUDA events on the session stream
    times, end_time = driver.step_times(m.curtime, args.steps * dt - 0.5 * dt, dt)
    tabs = driver.StepTables(m, times, dt, [1e9, 1e9], [None, None], [-1, -1])
    ctab = tabs.ctab(0, len(times))
    stream = torch.cuda.ExternalStream(eng.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = eng.kernel_launches()
    clocks.start()
    ev0.record(stream)
    eng.run(ctab, dt)                       # K steps, one captured CUDA graph per step
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = eng.kernel_launches() - launches0
    m.curtime = end_time
    el_ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([el_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        el_ms = float(t.item())
        dist.barrier()
    # FP64 reference state after W + K steps, for the mixed form's error report
    eng.download()
    ref64 = {"x": m.P.position[0:3, :m.parnum].copy(), "f": m.P.force[:, :m.parnum].copy()}
    from parmec_gb300 import energy as _energy
    ref64["E"] = _energy.total(m)
    ref64["K"] = _energy.kinetic(m)
    # the same K steps again with CUDA events around every kernel group, for the
    # per-kernel durations behind the roofline
    times2, end2 = driver.step_times(m.curtime, args.steps * dt - 0.5 * dt, dt)
    tabs2 = driver.StepTables(m, times2, dt, [1e9, 1e9], [None, None], [-1, -1])
    eng.profile(True)
    eng.run(tabs2.ctab(0, len(times2)), dt)
    torch.cuda.synchronize()
    prof = eng.profile_read()
    eng.profile(False)
    m.curtime = end2
    eng.download()
    contacts = eng.contacts()
    nc = len(contacts["mpart"])
    c_pair = nc / m.parnum

    # end to end through the public DEM command: host arrays -> device, K steps, device -> host;
    # one untimed call of the same path first (first-touch of the host pages and copies)
    m._dirty = True
    m.dem(args.warmup * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    m._dirty = True
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    try:
        m.dem(args.steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
    except RuntimeError:
        print(json.dumps({"e2e_failure_diagnostics": eng.diagnostics()}), file=sys.stderr)
        raise
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    up, down = state_bytes(m)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    total_ps = m.parnum * args.steps * world
    value = total_ps / (el_ms * 1e-3)
    hbm, peak_kind = peaks()
    # roofline of the dominant kernel group (algorithmic bytes: each datum the
    # kernel must read or write, counted once; formulas in the design doc)
    groups = {k: v for k, v in prof.items() if v[1] > 0}
    dom = max(groups, key=lambda k: groups[k][0])
    P = m.parnum
    per_launch = {
        "integrate": P * (696.0 + 53.0 * c_pair),
        "contacts": P * (172.0 + 96.0 * c_pair),
    }
    ms_dom, n_dom = groups[dom]
    bytes_dom = per_launch.get(dom)
    # DRAM bytes per launch: ncu capture of the 262,144-sphere case
    # (profiles/k_integrate_k_contacts_drum_fp64.md) scaled by the units processed
    traffic_per_unit = {"integrate": 458.0, "contacts": 200.0}
    traffic = traffic_per_unit[dom] * P if dom in traffic_per_unit else None
    # FP64 pipe: thread-level FP64 instructions (DADD + DMUL + DFMA) per unit,
    # counted by ncu on the same capture; peak = 2 per clock per SM
    fp64_per_unit = {"integrate": 294.0, "contacts": 161.0}
    fp64 = None
    if dom in fp64_per_unit:
        sm_mhz = clk.get("sm_mhz") or 2070.0
        peak_g = 2.0 * torch.cuda.get_device_properties(0).multi_processor_count * sm_mhz * 1e6 / 1e9
        ach_g = fp64_per_unit[dom] * P / (ms_dom * 1e-3 / args.steps) / 1e9
        fp64 = {"kernel": dom, "ops_per_unit": fp64_per_unit[dom], "achieved": ach_g, "peak": peak_g,
                "unit": "G FP64 inst/s", "frac": ach_g / peak_g,
                "source": "ops per unit from ncu (profiles/k_integrate_k_contacts_drum_fp64.md); "
                          "peak 2 FP64 lanes/clk/SM at the sampled SM clock"}
    if bytes_dom is not None:
        avg_s = ms_dom * 1e-3 / args.steps
        achieved = bytes_dom / avg_s / 1e9
    else:
        achieved = None
    step_bytes = P * (420.0 + 56.0 * c_pair)
    step_gbs = step_bytes / (el_ms * 1e-3 / args.steps) / 1e9
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "plain FP64 (bit-exact with the oracle)",
                   "spheres": m.parnum, "triangles": m.trinum, "parallelism": f"replicas x{world}",
                   "l2": "state ~0.6 GB per replica, larger than L2; no flush",
                   "bed_solid_fraction": round(info["solid_fraction"], 3),
                   "contacts_per_particle": round(c_pair, 3)},
        "e2e": {"value": m.parnum * args.steps * world / e2e_s, "unit": "particle-steps/s",
                "h2d_bytes_per_step": up // args.steps, "d2h_bytes_per_step": down // args.steps,
                "path": "Model.dem() through the pg_session C ABI: per-step host tables (Python callbacks), "
                        "full host->device upload, K steps, device->host download; host SoA arrays "
                        "page-locked by the engine (cudaHostRegister)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None,
                     "traffic": traffic, "traffic_source": "ncu 262,144-sphere capture scaled per unit",
                     "peak_source": peak_kind,
                     "step_algorithmic_gbs": step_gbs, "step_frac": step_gbs / hbm,
                     "note": "FP64-ALU bound on GB300 (2 DFMA/clk/SM): see fp64_pipe and profiles/"},
        "fp64_pipe": fp64,
        "kernel_ms": {k: round(v[0] / args.steps, 4) for k, v in groups.items()},
        "clocks": clk,
    }
    if not args.no_batched:
        from parmec_gb300.scenes import batch_scenes
        line["batched"] = batched_form(args, batch_scenes(args.batch_scenes))
    line["mixed"] = mixed_form(args, ref64)
    if args.lattice > 0:
        line["spring_lattice"] = spring_lattice_form(args, args.lattice)
    if args.serving > 0:
        line["serving"] = serving_form(args, args.serving)
    line["mixed"]["speedup_vs_plain"] = line["mixed"]["value"] / (value / world)
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(args.spheres, os.cpu_count() or 1)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
