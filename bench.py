"""Benchmark: DG DOF-stages/s of the explicit dGSEM Euler SSP-RK3 stage on GB300.

One "step" = one SSP-RK3 step (3 stages) of the 3D rising-bubble workload
(32^3 hexahedra, N = 4, 4.1 M nodes, 5 conserved variables: 20.48 M DOF) with
its state resident in HBM.  A DOF-stage is one conserved variable at one node
advanced through one RK stage.

  value        device-resident throughput of the headline form (precision
               form when built, else the plain FP64 form), CUDA events on
               the library's stream, K steps bracketed by synchronisation
  e2e          the same metric through the C ABI with host buffers: every
               step copies the state in from pinned host memory, advances it
               and copies it back (set_state -> step -> get_state)
  roofline     dominant kernel: algorithmic bytes / its average launch time
               (per-kernel CUDA events in a profiling pass after the timed
               region) against the measured HBM copy bandwidth
  cpu_baseline the oracle (C restatement of the reference's operators,
               OpenMP over all host cores) on a bounded sample of the same
               workload
  --impl reference  times only that CPU path (the reference's own code does
               not run on the GPU machine: it has no GPU path, and its
               sources are not present there), on the same metric.
  l2_vs_fp64, mass_drift, adjoint_over_forward
               the metric's accuracy and adjoint parts, measured after the
               timed region: relative L2 per conserved variable of the
               precision form against the plain FP64 form after 200 steps
               from the same initial state, the drift of the compensated mass
               sum over those steps in both forms, and the reverse sweep's
               device time over the plain forward's for 200 steps with
               checkpoints every 20 (precision form; the FP64 form's ratio
               beside it over 20 steps)
  --stage-profile  prints per-kernel mean device times of a few steps and the
               step's DOF-stages/s from them (a short fixed launch sequence for
               ncu captures; --workload, --prec, --viscosity) and exits
  --adjoint-profile  prints the adjoint/forward device-time ratio on --workload
               (--adjoint-steps, --adjoint-every, --prec, --viscosity) and exits

Inputs (>= 560 MB of state, stage and primitive arrays) exceed the 129 MB L2,
so no L2 flush is needed between timed steps.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "bubble3d_32_n4"
DT = 0.0075           # largest stable step of this mesh (dt = 0.01 diverges)
METRIC = "DG DOF-stages/s: mixed-precision vs FP64 at stated L2 error; adjoint/forward"
UNIT = "DOF-stages/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def ncu_traffic(kernel):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
    a kernel class from the committed ncu summary of this workload, or None."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(p):
        return None, None
    with open(p) as f:
        d = json.load(f)
    k = d.get("kernels", {}).get(kernel)
    if not k or d.get("workload") != WORKLOAD:
        return None, None
    return float(k["dram_bytes_per_launch"]), d.get("source")


def max_over_ranks(ms, world):
    """The slowest rank's time (replicas: every rank runs the whole workload)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(dofs, steps, ms, world):
    """Whole-job DOF-stages/s of `world` replicas of the workload in `ms`."""
    return world * dofs * 3 * steps / (ms * 1e-3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline(mesh, u, seconds, dt):
    """Oracle on the host cores: SSP-RK3 steps of the full workload, repeated
    until about `seconds` of CPU work has been timed."""
    import oracle

    m = oracle.OracleMesh(mesh)
    m.ssprk3(u, dt, 1)  # warm-up (page-in, thread pool)
    steps, sec, state = 0, 0.0, u
    while sec < seconds:
        t0 = time.perf_counter()
        state = m.ssprk3(state, dt, 1)
        sec += time.perf_counter() - t0
        steps += 1
    dofs = 5 * m.n_int
    return {"value": dofs * 3 * steps / sec, "unit": UNIT, "cores": oracle.lib().nsem_oracle_threads(),
            "kind": "port",
            "sample": f"{steps} SSP-RK3 steps of {WORKLOAD} ({m.n_int} nodes), OpenMP, "
                      f"{sec:.2f} s"}


def config(dofs, world):
    """The workload as both arms name it."""
    return {"workload": WORKLOAD, "elements": 32 ** 3, "order": 4, "dofs": dofs, "dt": DT,
            "scheme": "SSP-RK3", "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (no flush needed)"}


def accuracy(solver, u0, steps):
    """Precision form against the plain FP64 form after `steps` steps from u0:
    relative L2 per conserved variable (and of theta'), and the relative drift
    of the compensated mass sum in both forms."""
    import nebulasem_gb300 as ng

    finals, drift = {}, {}
    for prec, tag in ((ng.FP64, "fp64"), (ng.MIXED, "mixed")):
        solver.set_state(u0)
        m0 = solver.diagnostics()[0]
        solver.step(steps, prec=prec)
        finals[tag] = solver.get_state()
        drift[tag] = (solver.diagnostics()[0] - m0) / m0
    ref, got = finals["fp64"], finals["mixed"]

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    l2 = {v: rel(a, b) for v, a, b in zip(ng.VARS, got, ref)}
    l2["theta_prime"] = rel(got[4] / got[0] - 300.0, ref[4] / ref[0] - 300.0)
    return {"steps": steps, "l2": l2, "mass_drift": drift}


def adjoint_ratio(solver, mesh, u0, steps, every, prec):
    """Device time of the reverse sweep over that of the plain (graph-launched)
    forward run of the same steps, for J = 1/2 sum theta'^2 over the box
    x in [800, 1200], z in [800, 1200] m."""
    import torch

    from nebulasem_gb300 import objective as ob

    n = solver.n_int
    xyz = np.asarray(mesh["cC"]).reshape(-1, 3)[:n]
    mask = ob.box_mask(xyz, (800.0, 1200.0, 800.0, 1200.0))
    stream = torch.cuda.ExternalStream(solver.stream)
    solver.set_state(u0)
    solver.step(steps, prec=prec)            # builds the graph
    solver.set_state(u0)
    solver.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.step(steps, prec=prec, sync=False)
    e1.record(stream)
    solver.sync()
    ms_fwd = e0.elapsed_time(e1)
    solver.set_state(u0)
    ms_ckpt = solver.forward_checkpointed(steps, every, prec=prec)
    _, ms_adj = solver.adjoint(ob.objective_grad(solver.get_state(), mask))
    return {"steps": steps, "ckpt_every": every, "forward_ms": ms_fwd,
            "checkpointed_forward_ms": ms_ckpt, "adjoint_ms": ms_adj,
            "ratio": ms_adj / ms_fwd}


def adjoint_profile(args):
    """Adjoint/forward device-time ratio on a named workload: `--adjoint-steps`
    steps with checkpoints every `--adjoint-every`, in the form `--prec`, with
    `--viscosity` (default none)."""
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import workload

    prec = ng.MIXED if args.prec == "mixed" else ng.FP64
    m, u = workload(args.workload)
    s = ng.Solver(m, dt=args.dt, viscosity=args.viscosity)
    r = adjoint_ratio(s, m, u, args.adjoint_steps, args.adjoint_every, prec)
    r.update({"workload": args.workload, "dt": args.dt, "prec": "mixed" if prec else "fp64",
              "viscosity": args.viscosity or 0.0})
    print(json.dumps(r))
    s.close()


def stage_profile(args):
    """Per-kernel mean device times of a few steps: 3 graph-launched steps,
    then `--profile-steps` launch by launch (a short fixed launch sequence for
    ncu captures: 3 x launches-per-step launches precede the profiled ones).
    --scheme seg instead runs `--profile-steps` graph-launched steps of the
    reference's own segregated update (from the workload's fields, or from a
    golden fixture's mesh and step-0 fields with --fixture) and prints their
    wall time; --scheme conv the same for the scalar convection path."""
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import workload

    if args.scheme == "seg":
        if args.fixture:
            sys.path.insert(0, os.path.join(ROOT, "tests"))
            from conftest import load_golden

            m = load_golden(args.fixture)
            n = int(m["meta"][7])
            rho, U, T = m["fld0_rho"], m["fld0_U"].reshape(n, 3), m["fld0_T"]
        else:
            m, u = workload(args.workload)
            n = int(m["meta"][7])
            rho = u[0]
            U = np.stack([u[1] / rho, u[2] / rho, u[3] / rho], axis=1)
            T = u[4] / rho - 300.0
        s = ng.Solver(m, dt=args.dt, viscosity=args.viscosity)
        s.set_fields(rho, U, T)
        s.step(args.profile_steps, scheme=ng.REF_SEGREGATED)   # builds the graph
        s.set_fields(rho, U, T)
        s.sync()
        t0 = time.perf_counter()
        s.step(args.profile_steps, scheme=ng.REF_SEGREGATED)
        s.sync()
        wall = time.perf_counter() - t0
        print(json.dumps({"scheme": "segregated", "nodes": n, "steps": args.profile_steps,
                          "seconds": wall,
                          "dof_steps_per_s": 5 * n * args.profile_steps / wall}))
        s.close()
        return
    if args.scheme == "conv":
        # the convection app's scalar transport: theta' of the workload in the
        # uniform wind (6, -4, 5) m/s
        m, u = workload(args.workload)
        n = int(m["meta"][7])
        s = ng.Solver(m, dt=args.dt)
        U = np.tile(np.array([6.0, -4.0, 5.0]), (n, 1))
        T = u[4] / u[0] - 300.0
        s.convection_set(U, T)
        s.convection_step(args.profile_steps)
        s.convection_set(U, T)
        s.sync()
        t0 = time.perf_counter()
        s.convection_step(args.profile_steps)
        s.sync()
        wall = time.perf_counter() - t0
        print(json.dumps({"scheme": "convection", "nodes": n, "steps": args.profile_steps,
                          "seconds": wall, "dof_steps_per_s": n * args.profile_steps / wall}))
        s.close()
        return
    prec = ng.MIXED if args.prec != "fp64" else ng.FP64
    if args.fixture:
        # a golden fixture's mesh (e.g. a refined one) and its state u0
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from conftest import VARS, load_golden

        m = load_golden(args.fixture)
        u = [m[f"u0_{v}"] for v in VARS]
    else:
        m, u = workload(args.workload)
    s = ng.Solver(m, dt=args.dt, viscosity=args.viscosity)
    s.set_state(u)
    s.step(3, prec=prec)
    prof = s.profile(args.profile_steps, prec=prec)
    out = {k: v[0] / v[1] for k, v in prof.items()}
    # whole-step throughput of the profiled steps (launch by launch)
    step_ms = sum(v[0] for v in prof.values()) / args.profile_steps
    out["dof_stages_per_s"] = 15 * s.n_int / (step_ms * 1e-3)
    print(json.dumps(out))
    s.close()


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from nebulasem_gb300.mesh import workload

    mesh, u = workload(WORKLOAD)
    steps = max(1, args.steps)
    import oracle

    m = oracle.OracleMesh(mesh)
    for _ in range(min(args.warmup, 1)):
        m.ssprk3(u, DT, 1)
    # one step at a time, bounded to about 90 s of host time in total
    sec, done, state = 0.0, 0, u
    while done < steps and sec < 90.0:
        t0 = time.perf_counter()
        state = m.ssprk3(state, DT, 1)
        sec += time.perf_counter() - t0
        done += 1
    dofs = 5 * m.n_int
    v = dofs * 3 * done / sec
    cores = oracle.lib().nsem_oracle_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (rising thermal bubble initial state, deterministic)",
        "config": config(dofs, world),
        "form": "fp64",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{done} of {steps} SSP-RK3 steps of the full workload "
                                   f"({m.n_int} nodes), {sec:.1f} s"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import workload

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.backend == "nccl" else "gloo")
    import torch

    torch.cuda.set_device(local)
    mesh, u0 = workload(WORKLOAD)
    solver = ng.Solver(mesh, dt=DT, device=local)
    n = solver.n_int
    dofs = 5 * n
    prec_name = args.prec
    fallback = None
    if prec_name == "auto":
        try:
            solver.set_state(u0)
            solver.tendency(prec=ng.MIXED)
            prec_name = "mixed"
        except ng.NsemError as e:
            prec_name = "fp64"
            fallback = f"precision form unavailable on this workload: {e}"
    prec = ng.MIXED if prec_name == "mixed" else ng.FP64
    stream = torch.cuda.ExternalStream(solver.stream)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    def timed(prec_, steps, warmup):
        solver.set_state(u0)
        for _ in range(warmup):
            solver.step(1, prec=prec_, sync=False)
        solver.sync()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            solver.step(1, prec=prec_, sync=False)
        e1.record(stream)
        solver.sync()
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1), world)

    clocks = ClockSampler(local)
    clocks.start()
    ms = timed(prec, args.steps, args.warmup)
    clk = clocks.stop()
    value = whole_job_value(dofs, args.steps, ms, world)

    # the other form, for the mixed/FP64 speed-up
    other = None
    if prec_name == "mixed":
        n64 = max(1, min(args.steps // 2, 100))
        ms64 = timed(ng.FP64, n64, 1)
        other = {"fp64_value": world * dofs * 3 * n64 / (ms64 * 1e-3)}

    # end to end through the C ABI with pinned host buffers
    rho = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    mom = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    rt = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    rho[:] = u0[0]
    mom[:, 0], mom[:, 1], mom[:, 2] = u0[1], u0[2], u0[3]
    rt[:] = u0[4]
    for _ in range(2):
        solver.set_state_raw(rho, mom, rt)
        solver.step(1, prec=prec, sync=False)
        solver.get_state_raw(rho, mom, rt)
    rho[:] = u0[0]
    mom[:, 0], mom[:, 1], mom[:, 2] = u0[1], u0[2], u0[3]
    rt[:] = u0[4]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solver.set_state_raw(rho, mom, rt)
        solver.step(1, prec=prec, sync=False)
        solver.get_state_raw(rho, mom, rt)
    e2e_s = time.perf_counter() - t0
    nbytes = int(rho.nbytes + mom.nbytes + rt.nbytes)
    # the copy legs alone (state staged in and read back, no step)
    reps = 5
    solver.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        solver.set_state_raw(rho, mom, rt)
    solver.sync()
    h2d_s = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        solver.get_state_raw(rho, mom, rt)
    d2h_s = (time.perf_counter() - t0) / reps
    e2e = {"value": world * dofs * 3 * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
           "ms_per_step": 1e3 * e2e_s / args.steps,
           "set_state_ms": 1e3 * h2d_s, "get_state_ms": 1e3 * d2h_s,
           "h2d_gbs": nbytes / h2d_s / 1e9, "d2h_gbs": nbytes / d2h_s / 1e9}

    # per-kernel device times (launch by launch, CUDA events on the same stream)
    solver.set_state(u0)
    prof = solver.profile(max(1, min(args.steps, 5)), prec=prec)
    top = max(prof.items(), key=lambda kv: kv[1][0])
    top_name, (top_ms, top_n) = top
    per_launch_s = top_ms / top_n * 1e-3
    hbm, src = peaks()
    # algorithmic bytes of the dominant kernel's launches: FP64 state traffic of
    # the stage it runs (precision form: one kernel class per stage), or the
    # stage average for the plain form's per-stage kernels
    stage_of = {"mixed_stage1": 1, "mixed_stage2": 2, "mixed_stage3": 3}
    if top_name in stage_of:
        alg_bytes = ng.ALG_BYTES_PER_DOF_STAGE[stage_of[top_name]] * dofs
    else:
        alg_bytes = ng.ALG_BYTES_PER_DOF_STAGE_AVG * dofs
    achieved = alg_bytes / per_launch_s / 1e9
    launches_per_step = sum(c for _, c in prof.values()) / max(1, min(args.steps, 5))
    step_gbs = ng.ALG_BYTES_PER_DOF_STAGE_AVG * value / 1e9
    traffic, traffic_src = ncu_traffic(top_name)
    roof = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
            "traffic_source": traffic_src,
            "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else src,
            "alg_bytes_per_launch": alg_bytes,
            "kernel_ms_per_launch": top_ms / top_n,
            "step_achieved": step_gbs, "step_frac": step_gbs / hbm,
            "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof.items()}}
    if prec_name == "mixed":
        own = ng.mixed_own_bytes_per_node_stage()
        roof["own_layout_bytes_per_dof_stage"] = sum(own.values()) / 15.0

    acc = adj = adj64 = None
    if prec_name == "mixed" and not args.no_extra:
        acc = accuracy(solver, u0, 200)
        adj = adjoint_ratio(solver, mesh, u0, 200, 20, ng.MIXED)
        adj64 = adjoint_ratio(solver, mesh, u0, 20, 5, ng.FP64)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(mesh, u0, args.cpu_seconds, DT)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64" if prec_name == "mixed" else "f64",
            "data": "synthetic (rising thermal bubble initial state, deterministic)",
            "config": config(dofs, world), "form": prec_name,
            "e2e": e2e, "gpu_launches": int(round(launches_per_step * args.steps)),
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
        }
        if other:
            line["fp64_value"] = other["fp64_value"]
            line["mixed_over_fp64"] = value / other["fp64_value"]
        if fallback:
            line["form_fallback"] = fallback
        if acc:
            line["l2_vs_fp64"] = dict(acc["l2"], steps=acc["steps"])
            line["mass_drift"] = dict(acc["mass_drift"], steps=acc["steps"])
        if adj:
            line["adjoint_over_forward"] = adj["ratio"]
            line["adjoint"] = {"mixed": adj, "fp64": adj64}
        print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="auto", choices=["auto", "mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--backend", default="nccl")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the accuracy and adjoint measurements")
    ap.add_argument("--stage-profile", action="store_true")
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--dt", type=float, default=DT)
    ap.add_argument("--profile-steps", type=int, default=5)
    ap.add_argument("--scheme", default="ssprk3", choices=["ssprk3", "seg", "conv"])
    ap.add_argument("--fixture", default=None)
    ap.add_argument("--viscosity", type=float, default=None,
                    help="--stage-profile, --adjoint-profile: artificial viscosity (diffusion YES), default none")
    ap.add_argument("--adjoint-profile", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--adjoint-every", type=int, default=20)
    args = ap.parse_args()
    if args.adjoint_profile:
        adjoint_profile(args)
    elif args.stage_profile:
        stage_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
