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
only": scenes do not exchange data), and reports the aggregate: every
rank's particle-steps over the slowest rank's time.
--impl reference times the reference's own hot path on all host cores: its
ISPC sources translated to C++ at gang size one (oracle/ispc_ref.py; the
ispc compiler is not installed), driven by parmec.cpp's dem() call sequence.
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


def max_over_ranks(x, dist, device):
    """The largest x over the ranks (a job's time is its slowest rank's);
    x itself without a process group."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank, world, seconds):
    """Whole-job throughput: the units every rank processed over the job's time."""
    return units_per_rank * world / seconds


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


def reference_cpu(n_spheres, threads, steps, warmup=1):
    """The reference's own hot path on the host cores: its ISPC sources
    translated to C++ (oracle/ispc_ref.py; tasks spread over `threads`
    OpenMP threads, as its task system spreads them), driven by parmec.cpp's
    dem() call sequence on the same drum.  Falls back to the oracle (the
    restatement) where the translation is not on this host.  Returns
    (particle-steps/s, kind, sample description)."""
    from parmec_gb300.scenes import drum
    m, dt, _ = drum(n_spheres)
    try:
        from oracle import dem_loop, ispc_ref
        lib_path = ispc_ref.build()
    except Exception:
        lib_path = None
    if lib_path:
        lib = dem_loop.library(lib_path)
        host = dem_loop.Host(lib, m, orient=True, ntasks=threads)
        dem_loop.dem(lib, host, warmup * dt - 0.5 * dt, dt)
        t0 = time.perf_counter()
        dem_loop.dem(lib, host, steps * dt - 0.5 * dt, dt)
        el = time.perf_counter() - t0
        host.close()
        kind = "reference"
        what = ("the reference's condet/forces/dynamics/shapes/obstacles/partition ISPC sources translated to C++ "
                f"at gang size one (oracle/ispc_ref.py), g++ -O2, {threads} tasks on OpenMP threads, "
                "driven by parmec.cpp's dem() call sequence")
    else:
        from oracle.pyoracle import OracleEngine
        eng = OracleEngine(threads=threads)
        m.dem(warmup * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        t0 = time.perf_counter()
        m.dem(steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        el = time.perf_counter() - t0
        kind = "port"
        what = f"the oracle restatement on {threads} threads (the reference's sources are not on this host)"
    sample = f"{steps} DEM steps of the full {m.parnum}-sphere drum after {warmup} untimed, {el:.1f} s; {what}"
    return m.parnum * steps / el, kind, sample


def cpu_baseline(n_spheres, threads, steps=60):
    """The reference's CPU hot path on a bounded sample of the same drum
    (60 steps: about 10 s on 16 cores)."""
    v, kind, sample = reference_cpu(n_spheres, threads, steps)
    return {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": kind, "sample": sample}


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
    # per kernel group, on K more steps with CUDA events around each group
    # (after the state above was read)
    times2, end2 = driver.step_times(m.curtime, args.steps * dt - 0.5 * dt, dt)
    tabs2 = driver.StepTables(m, times2, dt, [1e9, 1e9], [None, None], [-1, -1])
    eng.profile(True)
    eng.run(tabs2.ctab(0, len(times2)), dt)
    torch.cuda.synchronize()
    prof = eng.profile_read()
    eng.profile(False)
    kernel_ms = {k: round(v[0] / args.steps, 4) for k, v in prof.items() if v[1] > 0}
    fmax = float(np.max(np.abs(ref64["f"])))
    df = float(np.max(np.abs(m.P.force[:, :n] - ref64["f"]))) / fmax
    E = energy.total(m)
    out = {"form": "mixed: FP32 contact geometry and forces, compensated FP32 pairs for x, v, L, radii and gaps",
           "value": n * args.steps / (el_ms * 1e-3), "unit": "particle-steps/s",
           "ms_per_step": el_ms / args.steps, "kernel_ms": kernel_ms,
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
    from parmec_gb300.serving import range_energy
    legs = ((abi.PG_FORM_MIXED, "mixed", True), (abi.PG_FORM_MIXED, "mixed_per_phase_kernels", False),
            (abi.PG_FORM_FP64, "fp64", False))
    snap = {}
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
        if key in ("mixed_per_phase_kernels", "fp64"):
            # the same W + K steps from the same state in both forms: kept for the error report
            eng.download()
            n = P.parnum
            snap[key] = {"x": P.P.position[0:3, :n].copy(), "f": P.P.force[:, :n].copy(),
                         "E": [range_energy(P, r[0], r[1], sc[2][0:3]) for r, sc in zip(P.scene_ranges, scenes)]}
            # per kernel group, on K more steps with CUDA events around each group
            times2, _ = driver.step_times(end_time, steps * dt - 0.5 * dt, dt)
            tabs2 = driver.StepTables(P, times2, dt, [1e9, 1e9], [None, None], [-1, -1])
            eng.profile(True)
            eng.run(tabs2.ctab(0, len(times2)), dt)
            torch.cuda.synchronize()
            prof = eng.profile_read()
            eng.profile(False)
            out[key]["kernel_ms"] = {g: round(v[0] / steps, 4) for g, v in prof.items() if v[1] > 0}
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
    a, b = snap["mixed_per_phase_kernels"], snap["fp64"]
    erel = np.abs(np.array(a["E"]) - np.array(b["E"])) / np.abs(np.array(b["E"]))
    fmax = float(np.max(np.abs(b["f"])))
    out["errors_vs_fp64"] = {
        "steps": args.warmup + steps, "scenes": len(scenes),
        "energy_rel_max": float(erel.max()), "energy_rel_p50": float(np.percentile(erel, 50)),
        "energy_rel_p99": float(np.percentile(erel, 99)), "scenes_energy_rel_under_1e-6": int(np.sum(erel <= 1e-6)),
        "position_max_abs_m": float(np.max(np.abs(a["x"] - b["x"]))),
        "force_max_abs_rel_to_max": float(np.max(np.abs(a["f"] - b["f"]))) / fmax,
        "energy_definition": "per scene: kinetic + rotational + potential of the scene's base gravity g0, "
                             "mixed form (per-phase kernels; the fused kernel gives the same bits) against FP64"}
    return out


def spring_lattice_form(args, n_side):
    """Config 2: the spring-lattice shaking table, n_side^2 MESH cubes (12
    triangles each), 2 n (n-1) neighbour springs and n^2 base springs with
    8-point curves and lookup dashpots, prescribed base acceleration; plain
    FP64.  Run twice: with springs alone, as the reference computes it (the
    leg's headline), and with mesh-mesh contact on (triangles swept by 1 mm,
    half the gap: every cube touches the plate and its neighbours, so the
    contact work is that of a packed lattice; the reference has no contact
    between meshes)."""
    import torch
    from parmec_gb300 import driver
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.scenes import spring_lattice
    out = {}
    for key, radius in (("with_mesh_contact", 1e-3), ("springs_only", 0.0)):
        t0 = time.perf_counter()
        m, dt = spring_lattice(n_side, contact_radius=radius)
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
        leg = {"steps": steps, "dt": dt, "value": m.parnum * steps / (ms * 1e-3), "unit": "particle-steps/s",
               "spring_steps_per_s": m.sprnum * steps / (ms * 1e-3), "ms_per_step": ms / steps,
               "build_s": build_s, "kernel_ms": {k: round(v[0] / nprof, 4) for k, v in groups.items()}}
        if radius > 0.0:
            pairs, active = eng.mesh_contact_stats()
            leg["mesh_contact"] = {"radius_m": radius, "triangle_pairs_last_step": pairs,
                                   "active_contacts_last_step": active,
                                   "note": "steps with mesh contact run without CUDA graphs (one host wait "
                                           "per step for the pair count)"}
        out[key] = leg
        out.setdefault("particles", m.parnum)
        out.setdefault("springs", m.sprnum)
        out.setdefault("triangles", m.trinum)
        eng.close()
    out["workload"] = (f"{n_side}x{n_side} MESH hexahedra (10 mm), {out['springs']} springs, {out['triangles']} "
                       "triangles, base 0.5 g sin(2 pi 5 t) along x, FP64")
    # the headline is the reference's computation (springs, no contact between meshes)
    head = out["springs_only"]
    out.update({"value": head["value"], "unit": "particle-steps/s", "ms_per_step": head["ms_per_step"],
                "steps": head["steps"]})
    return out

def serving_form(args, count):
    """Config 4: a Poisson stream (200 req/s) of excitation-sweep requests
    (sphere counts log-uniform [1024, 262144], 200-5000 steps, sinusoid or
    band-limited noise), served by the continuous-batching pool (mixed and
    FP64 forms, pool sized by the 150 GB HBM budget alone) and by the plain
    FP64 drop-in path one request at a time (a DEM() call per request, the
    same excitation through a GRAVITY callable)."""
    import torch
    from parmec_gb300 import abi
    from parmec_gb300.engine import GpuEngine
    from parmec_gb300.serving import Server, excitation_gravity, request_stream
    t_gen = time.perf_counter()
    reqs = request_stream(count)
    t_gen = time.perf_counter() - t_gen
    out = {"workload": f"{count} requests, Poisson 200 req/s, spheres log-uniform [1024,262144], "
                       "steps U[200,5000], sinusoid or band-limited noise base excitation", "hbm_budget_gb": 150,
           "requests_built_s": t_gen}
    energies = {}
    for form, key in ((abi.PG_FORM_MIXED, "mixed_pool"), (abi.PG_FORM_FP64, "fp64_pool")):
        srv = Server(reqs[0].model, reqs[0].dt, form=form, budget_bytes=150e9, max_scenes=args.scene_slots,
                     max_scene_extent=4.0)
        torch.cuda.synchronize()
        res, st = srv.serve(reqs, realtime=True)
        srv.close()
        energies[key] = {r.rid: r.energy for r in res if r.error is None}
        out[key] = {"p50_s": st["p50_s"], "p99_s": st["p99_s"], "throughput": st["throughput"],
                    "unit": "particle-steps/s", "wall_s": st["wall_s"], "requests": st["requests"],
                    "rejected": st["rejected"], "admission_wait_s": st["admission_wait_s"], "pool": st["pool"]}
        del srv
    rel = np.array([abs(energies["mixed_pool"][k] - e) / abs(e) for k, e in energies["fp64_pool"].items()
                    if k in energies["mixed_pool"] and e != 0.0])
    out["mixed_vs_fp64_energy_rel"] = {"requests": int(len(rel)), "max": float(rel.max()) if len(rel) else None,
                                       "p50": float(np.percentile(rel, 50)) if len(rel) else None,
                                       "p99": float(np.percentile(rel, 99)) if len(rel) else None,
                                       "under_1e-6": int(np.sum(rel <= 1e-6)),
                                       "definition": "kinetic + rotational + potential of the base gravity g0 "
                                                     "at the request's end, mixed pool against FP64 pool"}
    # the plain FP64 drop-in: each request alone through DEM(), in arrival
    # order, with its excitation as the GRAVITY callable
    t0 = time.perf_counter()
    lat, ps = [], 0
    for q in reqs:
        now = time.perf_counter() - t0
        if now < q.arrival:
            time.sleep(q.arrival - now)
        m = q.model
        g = excitation_gravity(q.excitation)
        m.set_gravity(lambda t, g=g: g(t)[0], lambda t, g=g: g(t)[1], lambda t, g=g: g(t)[2])
        eng = GpuEngine()
        m.dem(q.steps * q.dt - 0.5 * q.dt, q.dt, interval=1e9, engine=eng)
        eng.close()
        lat.append(time.perf_counter() - t0 - q.arrival)
        ps += m.parnum * q.steps
    wall = time.perf_counter() - t0
    out["fp64_dropin"] = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                          "throughput": ps / wall, "unit": "particle-steps/s", "wall_s": wall,
                          "requests": len(lat),
                          "note": "one DEM() per request with the request's excitation as a GRAVITY callable"}
    out["mixed_pool_over_fp64_pool"] = out["mixed_pool"]["throughput"] / out["fp64_pool"]["throughput"]
    out["mixed_pool_over_fp64_dropin"] = out["mixed_pool"]["throughput"] / out["fp64_dropin"]["throughput"]
    return out


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU hot path on all host cores, rank 0
    only, on the same drum, config, metric and unit as the GPU arm; each step
    is a bounded sample of the workload."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from parmec_gb300.scenes import drum
    _, _, info = drum(args.spheres)
    v, kind, sample = reference_cpu(args.spheres, threads, args.steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": "particle-steps/s", "value": v, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * args.spheres / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": arm_config(args, info, world),
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def arm_config(args, info, world):
    """The workload both arms run (identical dicts)."""
    return {"workload": WORKLOAD, "form": "plain FP64", "spheres": args.spheres, "triangles": 4096,
            "parallelism": f"replicas x{world}", "l2": "state ~0.6 GB per replica, larger than L2; no flush",
            "bed_solid_fraction": round(info["solid_fraction"], 3)}


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
    ap.add_argument("--serving", type=int, default=500, help="requests in the serving stream (0: skip)")
    ap.add_argument("--scene-slots", type=int, default=256,
                    help="scene slots of each serving pool (the 150 GB budget bounds its spheres)")
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
    el_ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    if dist:
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
    # five timed DEM calls (each a full upload, K steps and a full download):
    # the median is the line's e2e value
    e2e_runs = []
    for _ in range(5):
        m._dirty = True
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            m.dem(args.steps * dt - 0.5 * dt, dt, interval=1e9, engine=eng)
        except RuntimeError:
            print(json.dumps({"e2e_failure_diagnostics": eng.diagnostics()}), file=sys.stderr)
            raise
        e2e_runs.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.median(e2e_runs)), dist, "cuda")
    up, down = state_bytes(m)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    value = job_value(m.parnum * args.steps, world, el_ms * 1e-3)
    hbm, peak_kind = peaks()
    # roofline of the dominant kernel group: the step's compulsory bytes per
    # particle, B = 420 + 56 c (c = contact pairs per particle, measured on
    # the pair list) times the particles of one launch, over the group's
    # average CUDA-event time per step
    groups = {k: v for k, v in prof.items() if v[1] > 0}
    dom = max(groups, key=lambda k: groups[k][0])
    P = m.parnum
    ms_dom, n_dom = groups[dom]
    avg_s = ms_dom * 1e-3 / args.steps
    step_bytes = P * (420.0 + 56.0 * c_pair)
    achieved = step_bytes / avg_s / 1e9
    # the kernel's own data (each datum it reads or writes, counted once):
    # 652 + 53 c_s + 48 c bytes per particle for the integration (c_s: slave
    # contacts, c: master contacts, whose force and point it sums), 92 + 48 c
    # per sphere for the probe and evaluation passes
    kernel_model = {"integrate": P * (652.0 + 101.0 * c_pair), "contacts": P * (92.0 + 48.0 * c_pair)}
    # DRAM bytes per unit and FP64 instructions per unit of each kernel group,
    # from ncu captures of the 262,144-sphere drum (dram__bytes_read.sum +
    # dram__bytes_write.sum, and DADD + DMUL + DFMA thread instructions, per
    # launch divided by the spheres), scaled to the full drum; the contact
    # group is its probe and evaluation passes, the integration takes the
    # master-side contact sums
    traffic_per_unit = {"integrate": 404.0, "contacts": 251.0}
    fp64_per_unit = {"integrate": 298.0, "contacts": 155.0}
    traffic = traffic_per_unit[dom] * P if dom in traffic_per_unit else None
    fp64 = None
    if dom in fp64_per_unit:
        sm_mhz = clk.get("sm_mhz") or 2070.0
        peak_g = 2.0 * torch.cuda.get_device_properties(0).multi_processor_count * sm_mhz * 1e6 / 1e9
        ach_g = fp64_per_unit[dom] * P / avg_s / 1e9
        fp64 = {"kernel": dom, "ops_per_unit": fp64_per_unit[dom], "achieved": ach_g, "peak": peak_g,
                "unit": "G FP64 inst/s", "frac": ach_g / peak_g,
                "source": "FP64 instructions per unit from one ncu capture; peak 2 FP64 lanes/clk/SM at the "
                          "sampled SM clock"}
    step_gbs = step_bytes / (el_ms * 1e-3 / args.steps) / 1e9
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": arm_config(args, info, world),
        "contacts_per_particle": round(c_pair, 3),
        "e2e": {"value": job_value(m.parnum * args.steps, world, e2e_s), "unit": "particle-steps/s",
                "h2d_bytes_per_step": up // args.steps, "d2h_bytes_per_step": down // args.steps,
                "path": "Model.dem() through the pg_session C ABI: per-step host tables (Python callbacks), "
                        "full host->device upload, K steps, device->host download; host SoA arrays "
                        "page-locked by the engine (cudaHostRegister)",
                "runs_s": [round(x, 4) for x in e2e_runs], "statistic": "median of five DEM calls",
                "segment": f"the five calls continue the same drum from step {2 * args.warmup + 2 * args.steps + 1}, "
                           f"after the timed steps (from step {args.warmup + 1}) and the profiled ones; "
                           "each call includes its upload, its first list rebuild and its download"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "algorithmic_bytes": "420 + 56 c per particle-step (the whole step's compulsory traffic), "
                                          "c = contact pairs per particle",
                     "traffic_source": "ncu DRAM bytes per unit of the 262,144-sphere drum, scaled to the launch",
                     "peak_source": peak_kind,
                     "kernel_model_gbs": kernel_model[dom] / avg_s / 1e9 if dom in kernel_model else None,
                     "step_algorithmic_gbs": step_gbs, "step_frac": step_gbs / hbm,
                     "note": "the FP64 form is bound by the FP64 pipe (2 DFMA/clk/SM on GB300): see fp64_pipe"},
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
