"""Per-kernel device times of a few SSP-RK3 steps on a named workload.

    python -m nebulasem_gb300.stage_profile --workload bubble3d_32_n4 --prec mixed

Builds the workload, runs --steps graph-launched steps, then --profile-steps
steps launch by launch with CUDA events around every kernel (nsem_profile) and
prints one JSON object {kernel class: mean ms per launch}.  A small, fixed
launch sequence for profilers: (--steps x launches per step) launches precede
the profiled ones.
"""
import argparse
import json

from . import FP64, MIXED, Solver
from .mesh import workload


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="bubble3d_32_n4")
    ap.add_argument("--prec", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--dt", type=float, default=0.0075)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--profile-steps", type=int, default=5)
    a = ap.parse_args()
    prec = MIXED if a.prec == "mixed" else FP64
    m, u = workload(a.workload)
    s = Solver(m, dt=a.dt)
    s.set_state(u)
    s.step(a.steps, prec=prec)
    prof = s.profile(a.profile_steps, prec=prec)
    print(json.dumps({k: v[0] / v[1] for k, v in prof.items()}))
    s.close()


if __name__ == "__main__":
    main()
