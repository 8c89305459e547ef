"""Benchmark: FLIP substeps/s on one GB300 for the 256^3 dam break with a sphere obstacle.

A step is one full substep (sort, liquid SDF, P2G, extrapolation, body force, pressure
projection with MIC(0)-PCG to a 1e-6 inf-norm relative residual, G2P, RK3 advection with
collisions, removal) of the synthetic seeded scene: 256^3 MAC grid, dx = 1/256, fluid block
x < 0.35, y < 0.5, 8 particles per cell, static sphere (0.6, 0.3, 0.5) r = 0.15, gravity,
PIC ratio 0.05, CFL 5, dt = 1/240.  Synthetic data stands in for the reference's scenes.

  value        substeps/s, mixed-precision PCG, particle state resident in HBM, device
               time of K substeps with CUDA events on the engine's stream (max over ranks)
  e2e          same metric through the C ABI with host buffers: every step uploads the
               particles from pinned host memory, runs the substep, reads them back
  fp64_*       the same with the FP64 PCG at the same 1e-6 residual (zero start, the reference's)
  mixed_zero_start  the mixed solve started from zero like the FP64 one (the headline's mixed solve
               starts from the previous substep's pressure): the precision comparison at equal start
  adjoint      forward + adjoint (differentiable substep, transposed maps) against the forward
  apic         substeps/s with the APIC velocity transfer, and its P2G / G2P kernel times
  viscosity    substeps/s with the viscosity solve (viscosity 1.0), rows and PCG iterations
  save_state_io  GB/s writing the save-state particle files: GPU writer vs the bake script's
               range-read loop through the same library
  parity       the 128^3 dam break (block x < 0.4, y < 0.6), mixed and FP64 PCG to 1e-6: every
               solve against the FP64 PCG on the same system to 1e-12 (pressure and velocity
               relative L2, largest weighted divergence after the projection over ||b||_inf)
  rollout_512  the 512^3 sphere dam break (~215M particles): an 8-substep checkpointed
               differentiable rollout and its adjoint, substeps/s and peak device memory
  roofline     achieved HBM GB/s of the dominant kernel (algorithmic bytes / event time)
  cpu_baseline the CPU restatement of the reference algorithm (oracle) on the host cores,
               one 256^3 substep as the bounded sample

--impl reference times the CPU restatement of the reference engine's substep (the
reference itself cannot be built on the benchmark host: its sources are not shipped
there) on the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "blender-flip-fluids_gb300"))

WORKLOAD = "dam_break_sphere_256"
DT = 1.0 / 240.0
TOL = 1e-6
WARM_START = 2   # start of the mixed solve: 1 the last pressure, 2 linear extrapolation of the last two
METRIC = "substeps/s @256^3 8ppc: mixed vs FP64 PCG at 1e-6 resid; adjoint/forward cost"
KERNELS = {0: "p2g", 1: "liquid_sdf", 2: "spmv_dot_f32", 3: "mic0_apply_f32", 4: "extrapolate", 5: "g2p",
           6: "rk3_advect", 7: "sort", 8: "p2g_apic", 9: "g2p_apic", 10: "viscosity_solve",
           11: "ffp3_output"}
VISCOSITY = 1.0


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-apic", action="store_true")
    ap.add_argument("--no-viscosity", action="store_true")
    ap.add_argument("--no-io", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-rollout", action="store_true", help="skip the 512^3 rollout forward + adjoint leg")
    ap.add_argument("--parity-steps", type=int, default=20,
                    help="substeps of the 128^3 dam break whose solves are checked against an FP64 reference solve")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="run one differentiable substep + adjoint inside a cudaProfilerStart/Stop range (for ncu)")
    ap.add_argument("--profile-substep", action="store_true",
                    help="after the warm-up, run one substep inside a cudaProfilerStart/Stop range (for ncu "
                         "--profile-from-start off) and print its time")
    ap.add_argument("--profile-kernel", choices=sorted(KERNELS.values()),
                    help="after the warm-up, time one kernel (--steps launches) inside a profiler range")
    ap.add_argument("--warm-start", type=int, default=2, choices=[1, 2],
                    help="mixed solve start: 1 the last substep's pressure, 2 the linear extrapolation of the last two")
    ap.add_argument("--profile-viscosity", type=float, default=0.0,
                    help="with --profile-substep: the substeps apply this constant viscosity")
    return ap.parse_args(argv)


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def replica_sync(world, device="cuda"):
    """Barrier and max-over-ranks for `world` independent replicas: every rank runs its own
    scene on its own GPU and nothing crosses ranks on the data path (the reference-exact MIC(0)
    does not shard).  The process group (NCCL on GPUs, gloo in the CPU tests) must already be
    initialised when world > 1."""
    def sync():
        if device == "cuda":
            import torch
            torch.cuda.synchronize()
    if world <= 1:
        return sync, (lambda x: x)
    import torch
    import torch.distributed as dist

    def barrier():
        dist.barrier()
        sync()

    def allmax(x):
        t = torch.tensor([x], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return barrier, allmax


def job_rate(world, steps, ms_max):
    """Whole-job substeps/s of `world` replicas that each ran `steps` substeps, the slowest in ms_max."""
    return world * steps / (ms_max / 1000.0)


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while a region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in self.rows for q in range(4) if r[3 + q] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def scene(name):
    from ffengine_gb300 import scenes
    spec = scenes.WORKLOADS[name]
    pos, vel = scenes.dam_break_particles(spec["n"], spec["xb"], spec["yb"], seed=0)
    return spec, pos, vel


def make_sim(spec, pos, vel, mode, apic=False):
    import ffengine_gb300 as ffe
    n = spec["n"]
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_console_output = False
    sim.enable_surface_reconstruction = False
    if apic:
        sim.set_velocity_transfer_method_APIC()
    else:
        sim.set_velocity_transfer_method_FLIP()
    sim.PICFLIP_ratio = 0.05
    sim.CFL_condition_number = 5
    sim.min_time_steps_per_frame = 1
    sim.max_time_steps_per_frame = 1
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    if spec["sphere"]:   # the sphere as the reference scenes add it: an icosphere MeshObject
        from ffengine_gb300 import scenes
        v, t = scenes.icosphere(*spec["sphere"], 4)
        ob = ffe.MeshObject(n, n, n, 1.0 / n)
        ob.update_mesh_static(ffe.TriangleMesh(v, t))
        sim.add_mesh_obstacle(ob)
    sim.set_pressure_solver_tolerance(TOL)
    sim.set_pressure_solver_mode(mode)
    if mode == 1:
        sim.set_pressure_warm_start(WARM_START)
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    return sim


def timed_substeps(sim, k):
    from ffengine_gb300 import call
    return float(call("FluidSimulation_gb300_run_substeps_timed", [ctypes.c_void_p, ctypes.c_int, ctypes.c_double],
                      ctypes.c_float, sim(), k, DT))


def timed_forward_adjoint(sim, k):
    from ffengine_gb300 import call
    return float(call("FluidSimulation_gb300_run_forward_adjoint_timed",
                      [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double], ctypes.c_float, sim(), k, DT,
                      0.5))


def time_kernel(sim, kid, reps):
    from ffengine_gb300 import call
    b = ctypes.c_double(0)
    ms = call("FluidSimulation_gb300_time_kernel", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
              ctypes.c_float, sim(), kid, reps, ctypes.byref(b))
    return float(ms), b.value


def e2e_run(spec, pos, vel, steps, warmup, barrier):
    """Public API with host buffers: upload (pinned) -> FluidSimulation_update (one substep per
    frame of 1/240 s, with its CFL speed reduction) -> read back, every step."""
    import torch
    import ffengine_gb300 as ffe
    from ffengine_gb300 import FluidSimulationMarkerParticleData_t, call
    sim = make_sim(spec, pos, vel, 1)
    npart = pos.shape[0]
    hp = torch.from_numpy(pos.copy()).pin_memory()
    hv = torch.from_numpy(vel.copy()).pin_memory()
    P = ctypes.c_void_p

    def step():
        nonlocal npart
        d = FluidSimulationMarkerParticleData_t()
        d.size = npart
        d.positions = ctypes.cast(hp.data_ptr(), ctypes.c_char_p)
        d.velocities = ctypes.cast(hv.data_ptr(), ctypes.c_char_p)
        call("FluidSimulation_gb300_set_marker_particle_data", [P, FluidSimulationMarkerParticleData_t], None, sim(), d)
        call("FluidSimulation_update", [P, ctypes.c_double], None, sim(), DT)   # the drop-in's frame call
        nin = npart
        npart = call("FluidSimulation_get_num_marker_particles", [P], ctypes.c_int, sim())
        call("FluidSimulation_get_marker_particle_position_data", [P, P], None, sim(), hp.data_ptr())
        call("FluidSimulation_get_marker_particle_velocity_data", [P, P], None, sim(), hv.data_ptr())
        return nin * 24, npart * 24

    for _ in range(warmup):
        step()
    barrier()
    h2d = d2h = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        a, b = step()
        h2d += a
        d2h += b
    t = time.perf_counter() - t0
    del sim
    return t, h2d / steps, d2h / steps


def rollout_run(workload, k):
    """The 512^3 sphere dam break (~215M particles): a k-substep differentiable rollout with a
    device checkpoint of (x, v) before each substep, then its adjoint (the built-in loss, mean
    vy^2 over the particles above y = 0.25), recomputing every substep from its checkpoint.  One untimed rollout first
    (it sizes every buffer), then the timed one from the same initial state; host-clock times
    around device-synchronised calls.  Peak device memory: free memory before the engine exists
    minus free memory after the adjoint (the engine's buffers only grow)."""
    import torch
    from ffengine_gb300 import FluidSimulationMarkerParticleData_t, call
    spec, pos, vel = scene(workload)
    # the particles the reference's load keeps: inside [0, 1)^3 (float rounding can put a coordinate at 1)
    keep = ((pos >= 0.0) & (pos < 1.0)).all(axis=1)
    pos, vel = np.ascontiguousarray(pos[keep]), np.ascontiguousarray(vel[keep])
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info()
    sim = make_sim(spec, pos[:8], vel[:8], 1)
    P = ctypes.c_void_p

    def reset():
        d = FluidSimulationMarkerParticleData_t()
        d.size = pos.shape[0]
        d.positions = ctypes.cast(pos.ctypes.data, ctypes.c_char_p)
        d.velocities = ctypes.cast(vel.ctypes.data, ctypes.c_char_p)
        call("FluidSimulation_gb300_set_marker_particle_data", [P, FluidSimulationMarkerParticleData_t], None, sim(), d)

    def rollout():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.rollout_forward(k, DT)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        cnt = call("FluidSimulation_gb300_rollout_adjoint", [P, P, P, ctypes.c_double, P, P], ctypes.c_int, sim(),
                   None, None, 0.25, None, None)
        torch.cuda.synchronize()
        return t1 - t0, time.perf_counter() - t1, cnt

    reset()
    rollout()
    reset()
    tf, ta, cnt = rollout()
    free1 = torch.cuda.mem_get_info()[0]
    npart = int(pos.shape[0])
    del sim
    return {"workload": workload, "grid": spec["n"], "particles": npart, "substeps": k,
            "forward_s": tf, "adjoint_s": ta, "forward_substeps_per_s": k / tf,
            "forward_adjoint_substeps_per_s": k / (tf + ta), "adjoint_over_forward": (tf + ta) / tf,
            "loss_particles": int(cnt), "checkpoint_bytes": 24 * npart * k,
            "peak_device_bytes": int(free0 - free1), "device_total_bytes": int(total),
            "timing": "host clock around device-synchronised rollout calls, after one untimed rollout"}


def parity_run(steps, mode):
    """The 128^3 dam break: `steps` substeps whose solves are each checked against the FP64 PCG
    on the same system to 1e-12; the worst and mean errors over the substeps."""
    spec, pos, vel = scene("dam_break_128")
    sim = make_sim(spec, pos, vel, mode)
    sim.set_solve_check(1e-12)
    rows = []
    for _ in range(steps):
        sim.update(DT)
        c = sim.get_solve_check()
        s_ = sim.get_pressure_solver_stats()
        if c["valid"]:
            rows.append((c["p_rel_l2"], c["u_rel_l2"], c["div_rel"], c["div_ref_rel"], s_["rel_residual"],
                         c["ref_rel_residual"]))
    del sim
    a = np.array(rows) if rows else np.zeros((0, 6))
    keys = ("pressure_rel_l2", "velocity_rel_l2", "max_div_over_b", "max_div_over_b_fp64_reference",
            "solver_rel_residual", "reference_rel_residual")
    return {"workload": "dam_break_128", "particles": int(pos.shape[0]), "substeps": len(rows),
            "solver": "mixed" if mode == 1 else "fp64", "tolerance": TOL, "reference_tolerance": 1e-12,
            "max": dict(zip(keys, [float(x) for x in a.max(0)])) if len(rows) else None,
            "mean": dict(zip(keys, [float(x) for x in a.mean(0)])) if len(rows) else None}


def cpu_substep_rate(spec, pos, vel, steps):
    """CPU restatement of the reference substep (oracle) on the host cores."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_api as O
    n = spec["n"]
    dx = 1.0 / n
    objs = []
    if spec["sphere"]:
        from ffengine_gb300 import scenes
        objs = [(*scenes.icosphere(*spec["sphere"], 4), 0, 0.0)]
    solid = O.solid_level_set(n, dx, objs)
    O.lib()
    p, v = pos, vel
    t0 = time.perf_counter()
    for _ in range(steps):
        p, v, st = O.substep(n, dx, DT, 0.05, 5, (0.0, -9.81, 0.0), solid, p, v, tol=TOL)
    t = time.perf_counter() - t0
    return steps / t, t


def threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def run_reference(args):
    rank, _, world = dist_info()
    if rank != 0:
        return
    spec, pos, vel = scene(args.workload)
    steps = max(1, min(args.steps, 2))
    rate, t = cpu_substep_rate(spec, pos, vel, steps)
    sample = ("%d full %s substep(s) of the CPU restatement of the reference engine's substep "
              "(oracle/, OpenMP on all host cores), %.1f s" % (steps, args.workload, t))
    out = {"metric": METRIC, "value": rate, "unit": "substeps/s", "n_gpus": world, "steps": steps, "warmup": 0,
           "ms_per_step": 1000.0 / rate, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+f64", "data": "synthetic seeded dam break (numpy PCG64 seed 0)",
           "config": {"workload": args.workload, "grid": spec["n"], "particles": int(pos.shape[0]),
                      "ppc": 8, "solver": "FP64 MIC(0)-PCG (reference algorithm), 1e-6 inf-norm relative"},
           "impl": "reference",
           "cpu_baseline": {"value": rate, "unit": "substeps/s", "cores": threads(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": rate, "unit": "substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gb300(args):
    rank, local, world = dist_info()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    barrier, allmax = replica_sync(world, "cuda")
    from ffengine_gb300 import build as b
    if not os.path.exists(b.LIB_PATH):
        raise RuntimeError("libffengine_gb300.so is not built: run __graft_entry__.build()")
    spec, pos, vel = scene(args.workload)
    npart = int(pos.shape[0])
    log = lambda *a: print(*a, file=sys.stderr, flush=True) if rank == 0 else None

    # ---- headline: mixed precision, device resident ----
    sim = make_sim(spec, pos, vel, 1)
    for _ in range(args.warmup):
        sim.substep(DT)
    barrier()
    l0 = sim.get_kernel_launch_count()
    with Clocks(local) as clk:
        ms = timed_substeps(sim, args.steps)
    launches = sim.get_kernel_launch_count() - l0
    barrier()
    ms = allmax(ms)
    value = job_rate(world, args.steps, ms)
    stats = sim.get_pressure_solver_stats()
    sim.enable_stage_timing(True)
    sim.substep(DT)
    stages = sim.get_stage_times()
    sim.enable_stage_timing(False)
    log("mixed: %.2f substeps/s (%.1f ms/substep), PCG %s" % (value / world, ms / args.steps, stats))
    log("stage ms: " + json.dumps({k: round(v, 3) for k, v in stages.items()}))
    # per-kernel event timing on the current state
    kt = {}
    for kid in (0, 1, 2, 3, 5, 6, 7, 11):
        t_ms, byt = time_kernel(sim, kid, 5)
        kt[KERNELS[kid]] = (t_ms, byt)
        log("kernel %-15s %8.3f ms  %8.1f GB/s" % (KERNELS[kid], t_ms, byt / (t_ms * 1e-3) / 1e9 if byt else 0))
    it = max(1, int(stats["iterations"]))
    per_substep = {"p2g": kt["p2g"][0], "liquid_sdf": kt["liquid_sdf"][0], "spmv_dot_f32": it * kt["spmv_dot_f32"][0],
                   "mic0_apply_f32": it * kt["mic0_apply_f32"][0], "g2p": kt["g2p"][0], "rk3_advect": kt["rk3_advect"][0],
                   "sort": kt["sort"][0]}
    dom = max(per_substep, key=per_substep.get)
    t_dom, b_dom = kt[dom]
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = b_dom / (t_dom * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        # DRAM bytes of one captured launch unit, scaled to this state by its algorithmic bytes
        cap = json.load(open(tpath)).get(args.workload, {}).get(dom)
        if cap:
            traffic = cap["dram_bytes"] * b_dom / cap["algorithmic_bytes"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": dom, "bytes_per_launch": b_dom, "ms_per_launch": t_dom,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
                "share_of_substep": per_substep[dom] / (ms / args.steps)}
    del sim

    # ---- FP64 PCG at the same residual ----
    sim = make_sim(spec, pos, vel, 0)
    for _ in range(args.warmup):
        sim.substep(DT)
    barrier()
    ms64 = allmax(timed_substeps(sim, args.steps))
    stats64 = sim.get_pressure_solver_stats()
    del sim
    fp64_value = job_rate(world, args.steps, ms64)
    log("fp64: %.2f substeps/s, PCG %s" % (fp64_value / world, stats64))

    # ---- mixed precision from a zero start (the FP64 solver's start): the precision comparison ----
    sim = make_sim(spec, pos, vel, 1)
    sim.set_pressure_warm_start(0)
    for _ in range(args.warmup):
        sim.substep(DT)
    barrier()
    ms0 = allmax(timed_substeps(sim, args.steps))
    stats0 = sim.get_pressure_solver_stats()
    del sim
    zero = {"value": job_rate(world, args.steps, ms0), "unit": "substeps/s", "ms_per_step": ms0 / args.steps,
            "iterations": stats0["iterations"], "rel_residual": stats0["rel_residual"]}
    zero["over_fp64"] = zero["value"] / fp64_value
    log("mixed, zero start: %.2f substeps/s, PCG %s" % (zero["value"] / world, stats0))

    # ---- APIC velocity transfer (affine vectors start at zero), mixed PCG ----
    apic = None
    if not args.no_apic:
        sim = make_sim(spec, pos, vel, 1, apic=True)
        for _ in range(args.warmup):
            sim.substep(DT)
        barrier()
        ms_apic = allmax(timed_substeps(sim, args.steps))
        ap = {}
        for kid in (8, 9):
            t_ms, byt = time_kernel(sim, kid, 5)
            ap[KERNELS[kid]] = {"ms": t_ms, "bytes": byt, "GB_per_s": byt / (t_ms * 1e-3) / 1e9}
        del sim
        apic = {"value": job_rate(world, args.steps, ms_apic), "unit": "substeps/s", "ms_per_step": ms_apic / args.steps,
                "over_flip": (args.steps * 1000.0 / ms_apic) / (args.steps * 1000.0 / ms), "kernels": ap}
        log("apic: %.2f substeps/s (x%.3f of FLIP); %s" % (apic["value"] / world, apic["over_flip"], json.dumps(ap)))

    # ---- viscosity solve before the projection (constant viscosity 1.0), mixed PCG ----
    visc = None
    if not args.no_viscosity:
        sim = make_sim(spec, pos, vel, 1)
        sim.viscosity = VISCOSITY
        sim.substep(DT)
        kv = max(1, min(args.steps, 3))
        barrier()
        ms_visc = allmax(timed_substeps(sim, kv))
        vst = sim.get_viscosity_solver_stats()
        # one more substep with stage timing: the solve's system build, factor and PCG
        sim.enable_stage_timing(True)
        sim.substep(DT)
        sim.enable_stage_timing(False)
        vt = sim.get_viscosity_solver_times()
        del sim
        visc = {"value": job_rate(world, kv, ms_visc), "unit": "substeps/s", "ms_per_step": ms_visc / kv,
                "substeps": kv, "viscosity": VISCOSITY, "solve_ms": vt, "rows": vst["rows"],
                "iterations": vst["iterations"], "residual": vst["error"], "success": vst["success"],
                "preconditioner": "tiled wavefront per velocity component"}
        log("viscosity: %.2f substeps/s (%.1f ms/substep), solve %s, %s" %
            (visc["value"] / world, ms_visc / kv, json.dumps(vt), json.dumps(vst)))

    # ---- save-state particle files (position + velocity): GPU writer vs the bake script's loop of
    # 2^21-particle range reads through the same library (bake.py:2864-2905) ----
    io = None
    if not args.no_io and rank == 0:
        import shutil
        import tempfile
        sim = make_sim(spec, pos, vel, 1)
        sim.substep(DT)
        tmp = tempfile.mkdtemp(prefix="ffgb300_io_")
        try:
            nbytes = 2 * 12 * sim.get_num_marker_particles()
            t0 = time.perf_counter()
            for name in ("position", "velocity"):
                sim.write_marker_particle_file(name, os.path.join(tmp, name + ".gpu"))
            t1 = time.perf_counter()
            n_p, chunk = sim.get_num_marker_particles(), 2 ** 21
            getters = {"position": sim.get_marker_particle_position_data_range,
                       "velocity": sim.get_marker_particle_velocity_data_range}
            for i in range(n_p // chunk + 1):
                s_, e_ = i * chunk, min((i + 1) * chunk, n_p)
                for name, get in getters.items():
                    with open(os.path.join(tmp, name + ".loop"), "ab" if i else "wb") as f:
                        f.write(get(s_, e_))
            t2 = time.perf_counter()
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        del sim
        io = {"bytes": nbytes, "gpu_writer_GB_per_s": nbytes / (t1 - t0) / 1e9,
              "range_read_loop_GB_per_s": nbytes / (t2 - t1) / 1e9, "files": "position + velocity, local temp dir"}
        log("save-state write: GPU writer %.2f GB/s, range-read loop %.2f GB/s" %
            (io["gpu_writer_GB_per_s"], io["range_read_loop_GB_per_s"]))

    # ---- differentiable substep + adjoint (loss: mean v_y^2 over y > 0.5) against the plain forward ----
    adj = None
    if not args.no_adjoint:
        sim = make_sim(spec, pos, vel, 1)
        for _ in range(args.warmup):
            sim.substep(DT)
        ka = max(1, min(args.steps, 5))
        timed_forward_adjoint(sim, 1)
        timed_substeps(sim, 1)
        barrier()
        ms_fwd = allmax(timed_substeps(sim, ka))
        ms_fa = allmax(timed_forward_adjoint(sim, ka))
        del sim
        adj = {"forward_ms": ms_fwd / ka, "forward_adjoint_ms": ms_fa / ka, "ratio": ms_fa / ms_fwd,
               "substeps": ka}
        log("forward+adjoint: %.1f ms vs forward %.1f ms (x%.2f)" % (ms_fa / ka, ms_fwd / ka, ms_fa / ms_fwd))

    # ---- errors of every solve against an FP64 reference solve, 128^3 dam break ----
    parity = None
    if not args.no_parity and rank == 0:
        parity = {"mixed": parity_run(args.parity_steps, 1), "fp64": parity_run(args.parity_steps, 0)}
        log("parity: " + json.dumps(parity))

    # ---- 512^3 sphere dam break: 8-substep checkpointed rollout forward + adjoint, peak memory ----
    rollout = None
    if not args.no_rollout and rank == 0:
        rollout = rollout_run("dam_break_sphere_512", 8)
        log("rollout: " + json.dumps(rollout))

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        t, h2d, d2h = e2e_run(spec, pos, vel, args.steps, args.warmup, barrier)
        t = allmax(t)
        e2e = {"value": job_rate(world, args.steps, t * 1000.0), "unit": "substeps/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
        log("e2e: %.2f substeps/s" % (e2e["value"] / world))

    # ---- CPU baseline (rank 0, one GPU only) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, t = cpu_substep_rate(spec, pos, vel, 1)
        cpu = {"value": rate, "unit": "substeps/s", "cores": threads(), "kind": "port",
               "sample": "1 full %s substep of the CPU restatement of the reference algorithm (oracle/, "
                         "OpenMP), %.1f s" % (args.workload, t)}
        log("cpu baseline: %.4f substeps/s (%.1f s)" % (rate, t))

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "substeps/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32+f64",
               "data": "synthetic seeded dam break (numpy PCG64 seed 0), 8 particles/cell",
               "config": {"workload": args.workload, "grid": spec["n"], "particles": npart, "ppc": 8,
                          "sphere": spec["sphere"], "dt": DT,
                          "solver": "mixed MIC(0)-PCG, FP64 refinement to 1e-6 inf-norm relative residual",
                          "parallelism": "replicas" if world > 1 else "single GPU",
                          "l2": "inputs larger than L2 (particle state %.0f MB)" % (npart * 24 / 1e6)},
               "particle_updates_per_s": value * npart,
               "pcg": {"mixed_iterations": stats["iterations"], "mixed_outer": stats["outer"],
                       "mixed_rel_residual": stats["rel_residual"], "fp64_iterations": stats64["iterations"],
                       "fp64_rel_residual": stats64["rel_residual"],
                       "mixed_start": ("linear extrapolation of the last two substeps' pressures" if WARM_START == 2 else
                                               "previous substep's pressure") + " (warm start); FP64 starts from zero"},
               "fp64_value": fp64_value, "mixed_over_fp64": value / fp64_value, "mixed_zero_start": zero,
               "adjoint_over_forward": adj["ratio"] if adj else None, "adjoint": adj, "apic": apic, "viscosity": visc, "save_state_io": io,
               "stage_ms": stages,
               "kernel_ms": {k: v[0] for k, v in kt.items()},
               "parity": parity, "rollout_512": rollout,
               "roofline": roofline, "clocks": clk.summary(), "gpu_launches": int(launches),
               "e2e": e2e, "cpu_baseline": cpu}
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_profile(args):
    """Small capture targets for ncu: the work inside the profiler range is one substep or one kernel."""
    import torch
    torch.cuda.set_device(0)
    spec, pos, vel = scene(args.workload)
    sim = make_sim(spec, pos, vel, 1, apic=(args.profile_kernel or "").endswith("_apic"))
    if args.profile_viscosity > 0:
        sim.viscosity = args.profile_viscosity
    for _ in range(max(1, args.warmup)):
        sim.substep(DT)
    torch.cuda.synchronize()
    out = {"workload": args.workload, "viscosity": args.profile_viscosity}
    if args.profile_adjoint:
        timed_forward_adjoint(sim, 1)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        ms = timed_forward_adjoint(sim, 1)
        torch.cuda.profiler.stop()
        out.update({"profiled": "differentiable substep + adjoint", "ms": ms})
    elif args.profile_substep:
        torch.cuda.profiler.start()
        ms = timed_substeps(sim, 1)
        torch.cuda.profiler.stop()
        out.update({"profiled": "substep", "ms": ms, "launches_per_substep": None})
        l0 = sim.get_kernel_launch_count()
        timed_substeps(sim, 1)
        out["launches_per_substep"] = sim.get_kernel_launch_count() - l0
    else:
        kid = {v: k for k, v in KERNELS.items()}[args.profile_kernel]
        torch.cuda.profiler.start()
        ms, byt = time_kernel(sim, kid, args.steps)
        torch.cuda.profiler.stop()
        out.update({"profiled": args.profile_kernel, "ms": ms, "bytes": byt,
                    "gbs": byt / (ms * 1e-3) / 1e9 if byt else None})
    print(json.dumps(out), flush=True)


def main():
    global WARM_START
    args = parse()
    WARM_START = args.warm_start
    if args.profile_substep or args.profile_kernel or args.profile_adjoint:
        run_profile(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
