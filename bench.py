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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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
        "config": {"workload": WORKLOAD, "elements": 32 ** 3, "order": 4, "dofs": dofs,
                   "dt": DT, "scheme": "SSP-RK3"},
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
    if prec_name == "auto":
        try:
            solver.set_state(u0)
            solver.tendency(prec=ng.MIXED)
            prec_name = "mixed"
        except ng.NsemError:
            prec_name = "fp64"
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
        ms64 = timed(ng.FP64, max(1, args.steps // 2), 1)
        other = {"fp64_value": world * dofs * 3 * max(1, args.steps // 2) / (ms64 * 1e-3)}

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
    e2e = {"value": world * dofs * 3 * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(rho.nbytes + mom.nbytes + rt.nbytes),
           "d2h_bytes_per_step": int(rho.nbytes + mom.nbytes + rt.nbytes)}

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
            "config": {"workload": WORKLOAD, "elements": 32 ** 3, "order": 4, "dofs": dofs,
                       "dt": DT, "scheme": "SSP-RK3", "form": prec_name,
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (no flush needed)"},
            "e2e": e2e, "gpu_launches": int(round(launches_per_step * args.steps)),
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
        }
        if other:
            line["fp64_value"] = other["fp64_value"]
            line["mixed_over_fp64"] = value / other["fp64_value"]
        print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="auto", choices=["auto", "mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--backend", default="nccl")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
