"""Gradient check of the discrete adjoint on the 16^3 N=4 rising bubble.

Workload: 2000^3 m box, 16x16x16 elements, N = 4 (512,000 nodes, 2.56 M DOF),
theta' = 0.5 K cosine bubble of radius 400 m at (1000, 1000, 600) m, plain
FP64 form, 200 SSP-RK3 steps at dt = 0.01 s, RK checkpoints every 20 steps.
Objective J = 1/2 sum of theta'^2 over the nodes of a box at the final time;
control: the initial theta' field.  The adjoint gradient is checked along 8
Gaussian directions (seeds 0..7) against central differences (eps = 1e-6) of
the GPU forward (and at eps = 1e-4) and against the CPU FP64 tangent-linear model (oracle,
dual numbers, with the correctly rounded pow so that its trajectory is the
GPU's bit for bit).

Two boxes are evaluated:
  * x in [800, 1200], z in [1200, 1600] m: the box of the workload as stated;
  * x in [800, 1200], z in [800, 1200] m: the same box 400 m lower, over the
    upper half of the bubble.

Usage (the first part needs a GPU, the second only the CPU):
    python tests/adjoint_c4_report.py gpu --out <dir>/adjoint_c4.npz
    python tests/adjoint_c4_report.py tlm --inp <dir>/adjoint_c4.npz
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

BOXES = {"stated": (800.0, 1200.0, 1200.0, 1600.0), "bubble_top": (800.0, 1200.0, 800.0, 1200.0)}
DT, STEPS, CKPT, NDIR = 0.01, 200, 20, 8
EPS = 1e-6          # the stated central-difference step
EPS_WIDE = 1e-4     # a wider step: its truncation error is O(eps^2), its round-off smaller
WORKLOAD = "bubble3d_16_n4"


def setup():
    from nebulasem_gb300.mesh import workload
    from nebulasem_gb300 import objective as ob
    m, u = workload(WORKLOAD)
    n = int(m["meta"][7])
    xyz = np.asarray(m["cC"]).reshape(-1, 3)[:n]
    p_ref = np.asarray(m["p_ref"])[:n]
    th0 = u[4] / u[0] - 300.0
    u0 = ob.state_from_theta(th0, p_ref)
    masks = {k: ob.box_mask(xyz, b) for k, b in BOXES.items()}
    dirs = [np.random.default_rng(seed).standard_normal(n) for seed in range(NDIR)]
    return m, n, p_ref, th0, u0, masks, dirs


def part_gpu(out):
    import nebulasem_gb300 as ng
    from nebulasem_gb300 import objective as ob
    m, n, p_ref, th0, u0, masks, dirs = setup()
    s = ng.Solver(m, dt=DT)
    res = {}
    # plain forward (graph-launched steps), timed after one warm-up run
    for rep in range(2):
        s.set_state(u0)
        s.sync()
        t = time.perf_counter()
        s.step(STEPS)
        t_plain = (time.perf_counter() - t) * 1e3
    s.set_state(u0)
    ms_fwd = s.forward_checkpointed(STEPS, CKPT)
    uN = s.get_state()
    for name, mask in masks.items():
        lam0, ms_adj = s.adjoint(ob.objective_grad(uN, mask))
        grad = ob.theta_grad(lam0, u0, th0)
        th = uN[4] / uN[0] - 300.0
        res[name] = dict(J=ob.objective(uN, mask), grad=grad, ms_adj=ms_adj,
                         max_theta_box=float(np.abs(th[mask]).max()),
                         dj_adj=np.array([float(np.dot(grad, v)) for v in dirs]),
                         Jp=np.zeros(NDIR), Jm=np.zeros(NDIR),
                         Jp_wide=np.zeros(NDIR), Jm_wide=np.zeros(NDIR))
    for d, v in enumerate(dirs):
        for eps, tag in ((EPS, ""), (EPS_WIDE, "_wide")):
            for sign in (1.0, -1.0):
                s.set_state(ob.state_from_theta(th0 + sign * eps * v, p_ref))
                s.step(STEPS)
                uS = s.get_state()
                for name, mask in masks.items():
                    res[name][("Jp" if sign > 0 else "Jm") + tag][d] = ob.objective(uS, mask)
    s.close()
    flat = dict(ms_fwd_ckpt=ms_fwd, ms_fwd_plain=t_plain, uN=np.stack(uN))
    for name, r in res.items():
        for k, v in r.items():
            flat[f"{name}__{k}"] = v
    np.savez(out, **flat)
    summary = dict(ms_fwd_plain=t_plain, ms_fwd_ckpt=ms_fwd)
    for name, r in res.items():
        dj_fd = (r["Jp"] - r["Jm"]) / (2 * EPS)
        dj_fdw = (r["Jp_wide"] - r["Jm_wide"]) / (2 * EPS_WIDE)
        summary[name] = dict(J=r["J"], max_theta_box=r["max_theta_box"], ms_adj=r["ms_adj"],
                             adj_over_fwd_plain=r["ms_adj"] / t_plain,
                             adj_over_fwd_ckpt=r["ms_adj"] / ms_fwd,
                             fd_rel=[float(abs(a - f) / abs(f)) if f != 0 else None
                                     for a, f in zip(r["dj_adj"], dj_fd)],
                             fd_wide_rel=[float(abs(a - f) / abs(f)) if f != 0 else None
                                          for a, f in zip(r["dj_adj"], dj_fdw)])
    print(json.dumps(summary))


def part_tlm(inp):
    import oracle
    from nebulasem_gb300 import objective as ob
    m, n, p_ref, th0, u0, masks, dirs = setup()
    r = np.load(inp)
    om = oracle.OracleMesh(m)
    oracle.set_pow(1)
    du0 = [[-u0[0] / (th0 + 300.0) * v] + [np.zeros(n) for _ in range(4)] for v in dirs]
    t = time.time()
    uT, duT = om.tlm_ssprk3_multi(u0, du0, DT, STEPS)
    t_tlm = time.time() - t
    same = all(np.array_equal(a, b) for a, b in zip(uT, r["uN"]))
    out = dict(tlm_seconds=t_tlm, threads=oracle.lib().nsem_oracle_threads(),
               cpu_trajectory_equals_gpu=bool(same),
               ms_fwd_plain=float(r["ms_fwd_plain"]), ms_fwd_ckpt=float(r["ms_fwd_ckpt"]))
    for name, mask in masks.items():
        gJ = ob.objective_grad(uT, mask)
        dj_tlm = np.array([sum(float(np.dot(a, b)) for a, b in zip(gJ, duT[d])) for d in range(NDIR)])
        dj_adj = r[f"{name}__dj_adj"]
        dj_fd = (r[f"{name}__Jp"] - r[f"{name}__Jm"]) / (2 * EPS)
        dj_fdw = None
        if f"{name}__Jp_wide" in r:
            dj_fdw = (r[f"{name}__Jp_wide"] - r[f"{name}__Jm_wide"]) / (2 * EPS_WIDE)

        def rel(a, b):
            return [float(abs(x - y) / abs(y)) if y != 0 else None for x, y in zip(a, b)]
        ms_adj = float(r[f"{name}__ms_adj"])
        out[name] = dict(box=BOXES[name], J=float(r[f"{name}__J"]),
                         max_theta_box=float(r[f"{name}__max_theta_box"]),
                         dj_adj=dj_adj.tolist(), dj_tlm=dj_tlm.tolist(), dj_fd=dj_fd.tolist(),
                         rel_adj_vs_tlm=rel(dj_adj, dj_tlm), rel_adj_vs_fd=rel(dj_adj, dj_fd),
                         rel_tlm_vs_fd=rel(dj_tlm, dj_fd),
                         rel_adj_vs_fd_wide=rel(dj_adj, dj_fdw) if dj_fdw is not None else None,
                         ms_adj=ms_adj, adj_over_fwd_plain=ms_adj / out["ms_fwd_plain"],
                         adj_over_fwd_ckpt=ms_adj / out["ms_fwd_ckpt"])
    print(json.dumps(out, indent=1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("part", choices=("gpu", "tlm"))
    ap.add_argument("--out", default="adjoint_c4.npz")
    ap.add_argument("--inp", default="adjoint_c4.npz")
    a = ap.parse_args()
    if a.part == "gpu":
        part_gpu(a.out)
    else:
        part_tlm(a.inp)


if __name__ == "__main__":
    main()
