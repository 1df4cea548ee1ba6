"""Accuracy of the precision form against the plain FP64 form on a bubble workload.

Runs the same initial state through `steps` SSP-RK3 steps in both forms on the
GPU and prints one JSON object: relative L2 error per conserved variable of the
precision form against the FP64 form, the drift of the compensated mass and
energy sums over the run for both forms, the wall time of each run (the second of two), and a
SHA-256 digest of the FP64 final state.  The FP64 form is bit-for-bit the
oracle with the correctly rounded pow; `--with-oracle` also runs that oracle on
the host cores from the same inputs and compares the two final states bit for
bit; `--oracle` runs the oracle alone and prints its digest.

    python tests/precision_report.py --workload bubble3d_16_n7 --dt 0.005 --steps 400
    python tests/precision_report.py --workload bubble3d_16_n7 --dt 0.005 --steps 400 --oracle
"""
import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")


def digest(u):
    h = hashlib.sha256()
    for a in u:
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return h.hexdigest()


def input_digest(m, u0):
    """Digest of the initial state and the hydrostatic background (both made
    with numpy transcendental functions, whose last bits may differ between
    host architectures)."""
    return digest(list(u0) + [np.asarray(m["p_ref"]), np.asarray(m["rho_ref"])])


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def run_gpu(name, dt, steps, adjoint_ckpt=0, with_oracle=False, viscosity=0.0):
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import workload
    m, u0 = workload(name)
    n = int(m["meta"][7])
    s = ng.Solver(m, dt=dt, viscosity=viscosity, Pr=0.9)
    out = dict(workload=name, dt=dt, steps=steps, nodes=n, dof=5 * n, input_sha256=input_digest(m, u0))
    if viscosity:
        out["viscosity"] = viscosity
    finals = {}
    for prec, tag in ((ng.FP64, "fp64"), (ng.MIXED, "mixed")):
        # the second of two identical runs is timed (the first builds the graph)
        for rep in range(2):
            s.set_state(u0)
            d0 = s.diagnostics()
            s.sync()
            t = time.perf_counter()
            try:
                s.step(steps, prec=prec)
                s.sync()
                ok = True
            except ng.NsemError as e:
                ok = False
                out[f"{tag}_error"] = str(e)
            wall = time.perf_counter() - t
            if not ok:
                break
        if not ok:
            out[f"{tag}_finite"] = False
            continue
        u = s.get_state()
        d1 = s.diagnostics()
        finite = all(np.isfinite(a).all() for a in u)
        out[f"{tag}_finite"] = bool(finite)
        out[f"{tag}_seconds"] = wall
        out[f"{tag}_dof_stages_per_s"] = 5 * n * 3 * steps / wall
        out[f"{tag}_mass_drift_rel"] = float((d1[0] - d0[0]) / d0[0])
        out[f"{tag}_energy_drift_rel"] = float((d1[1] - d0[1]) / d0[1])
        finals[tag] = u
    if adjoint_ckpt and "fp64" in finals and out.get("fp64_finite"):
        # FP64 discrete adjoint of J = 1/2 sum theta'^2 over x in [800, 1200],
        # z in [1200, 1600] m: checkpointed forward, then the reverse sweep
        from nebulasem_gb300 import objective as ob
        xyz = np.asarray(m["cC"]).reshape(-1, 3)[:n]
        mask = ob.box_mask(xyz)
        s.set_state(u0)
        ms_fwd = s.forward_checkpointed(steps, adjoint_ckpt)
        _, ms_adj = s.adjoint(ob.objective_grad(s.get_state(), mask))
        out.update(adjoint_ckpt=adjoint_ckpt, fwd_ckpt_ms=ms_fwd, adjoint_ms=ms_adj,
                   adjoint_over_fp64_forward=ms_adj / (1e3 * out["fp64_seconds"]),
                   adjoint_over_ckpt_forward=ms_adj / ms_fwd)
        if "mixed_seconds" in out:
            out["adjoint_over_mixed_forward"] = ms_adj / (1e3 * out["mixed_seconds"])
    s.close()
    if "fp64" in finals:
        out["fp64_sha256"] = digest(finals["fp64"])
        if with_oracle:
            # the oracle on the same host, same inputs
            import oracle
            om = oracle.OracleMesh(m)
            oracle.set_pow(1)
            t = time.time()
            uo = om.ssprk3(u0, dt, steps)
            out["oracle_seconds"] = time.time() - t
            out["oracle_threads"] = oracle.lib().nsem_oracle_threads()
            out["oracle_sha256"] = digest(uo)
            out["fp64_equals_oracle_bitwise"] = out["oracle_sha256"] == out["fp64_sha256"]
            out["fp64_vs_oracle_max_rel_l2"] = max(rel_l2(a, b) for a, b in zip(finals["fp64"], uo))
    if "fp64" in finals and "mixed" in finals:
        ref, got = finals["fp64"], finals["mixed"]
        scale = max(np.linalg.norm(x) for x in ref[1:4])
        err = {}
        for a, b, v in zip(got, ref, VARS):
            if np.linalg.norm(b) < 1e-10 * scale:
                err[v] = dict(abs_l2=float(np.linalg.norm(a - b)), note="zero in FP64 up to round-off")
            else:
                err[v] = rel_l2(a, b)
        out["mixed_rel_l2_vs_fp64"] = err
        out["mixed_momentum_vector_rel_l2"] = rel_l2(np.stack(got[1:4]), np.stack(ref[1:4]))
        th_ref = ref[4] / ref[0] - 300.0
        th_got = got[4] / got[0] - 300.0
        out["mixed_theta_prime_rel_l2"] = rel_l2(th_got, th_ref)
    return out


def run_segregated(name, dt, steps, with_oracle=False, fixture=None):
    """The reference's own update (segregated forward Euler) on the GPU from the
    workload's fields (or a golden fixture's mesh and step-0 fields, e.g. an
    adaptively refined mesh); throughput and, with the oracle, bitwise
    comparison."""
    import nebulasem_gb300 as ng
    if fixture:
        from conftest import load_golden
        m = load_golden(fixture)
        n = int(m["meta"][7])
        rho, U, T = m["fld0_rho"], m["fld0_U"].reshape(n, 3), m["fld0_T"]
        name = fixture
    else:
        from nebulasem_gb300.mesh import workload
        m, u0 = workload(name)
        n = int(m["meta"][7])
        rho = u0[0]
        U = np.stack([u0[1] / rho, u0[2] / rho, u0[3] / rho], axis=1)
        T = u0[4] / rho - 300.0
    s = ng.Solver(m, dt=dt)
    out = dict(workload=name, scheme="REF_SEGREGATED", dt=dt, steps=steps, nodes=n, dof=5 * n)
    for rep in range(2):
        s.set_fields(rho, U, T)
        s.sync()
        t = time.perf_counter()
        s.step(steps, scheme=ng.REF_SEGREGATED)
        s.sync()
        wall = time.perf_counter() - t
    r, u, th = s.get_fields()
    s.close()
    out["seconds"] = wall
    out["dof_steps_per_s"] = 5 * n * steps / wall   # one stage per step
    out["finite"] = bool(np.isfinite(r).all() and np.isfinite(u).all() and np.isfinite(th).all())
    out["sha256"] = digest([r, u.reshape(-1), th])
    if with_oracle:
        import oracle
        om = oracle.OracleMesh(m)
        oracle.set_pow(1)
        t = time.time()
        ro, uo, to = om.segregated(rho, U, T, dt, steps)
        out["oracle_seconds"] = time.time() - t
        out["oracle_threads"] = oracle.lib().nsem_oracle_threads()
        out["oracle_sha256"] = digest([ro, uo.reshape(-1), to])
        out["equals_oracle_bitwise"] = out["oracle_sha256"] == out["sha256"]
    return out


def run_convection(name, dt, steps, with_oracle=False):
    """The reference's scalar convection of the workload's theta' in a uniform
    wind (6, -4, 5) m/s on the GPU; throughput and, with the oracle, bitwise
    comparison."""
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import workload
    m, u0 = workload(name)
    n = int(m["meta"][7])
    T = u0[4] / u0[0] - 300.0
    U = np.tile(np.array([6.0, -4.0, 5.0]), (n, 1))
    s = ng.Solver(m, dt=dt)
    out = dict(workload=name, scheme="convection", dt=dt, steps=steps, nodes=n, dof=n)
    for rep in range(2):
        s.convection_set(U, T)
        s.sync()
        t = time.perf_counter()
        s.convection_step(steps)
        s.sync()
        wall = time.perf_counter() - t
    got = s.convection_get()
    s.close()
    out["seconds"] = wall
    out["dof_steps_per_s"] = n * steps / wall
    out["sha256"] = digest([got])
    if with_oracle:
        import oracle
        om = oracle.OracleMesh(m)
        t = time.time()
        want = om.convection(U, T, dt, steps)
        out["oracle_seconds"] = time.time() - t
        out["oracle_threads"] = oracle.lib().nsem_oracle_threads()
        out["equals_oracle_bitwise"] = bool(np.array_equal(got, want))
    return out


def run_oracle(name, dt, steps):
    import oracle
    from nebulasem_gb300.mesh import workload
    m, u0 = workload(name)
    om = oracle.OracleMesh(m)
    oracle.set_pow(1)
    t = time.time()
    u = om.ssprk3(u0, dt, steps)
    return dict(workload=name, dt=dt, steps=steps, input_sha256=input_digest(m, u0),
                oracle_seconds=time.time() - t,
                threads=oracle.lib().nsem_oracle_threads(),
                finite=bool(all(np.isfinite(a).all() for a in u)),
                oracle_sha256=digest(u))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="")
    ap.add_argument("--fixture", default=None,
                    help="segregated scheme on a golden fixture's mesh (e.g. amr_g3_4n3)")
    ap.add_argument("--dt", type=float, required=True)
    ap.add_argument("--steps", type=int, required=True)
    ap.add_argument("--oracle", action="store_true")
    ap.add_argument("--scheme", default="ssprk3", choices=["ssprk3", "seg", "conv"],
                    help="seg: the reference's own segregated update (FP64)")
    ap.add_argument("--with-oracle", action="store_true",
                    help="also run the oracle on this host and compare bit for bit")
    ap.add_argument("--viscosity", type=float, default=0.0,
                    help="artificial viscosity nu (diffusion YES, Pr 0.9) for both forms")
    ap.add_argument("--adjoint-ckpt", type=int, default=0,
                    help="also time the FP64 adjoint with checkpoints every k steps")
    a = ap.parse_args()
    if a.scheme == "seg":
        r = run_segregated(a.workload, a.dt, a.steps, a.with_oracle, a.fixture)
    elif a.scheme == "conv":
        r = run_convection(a.workload, a.dt, a.steps, a.with_oracle)
    elif a.oracle:
        r = run_oracle(a.workload, a.dt, a.steps)
    else:
        r = run_gpu(a.workload, a.dt, a.steps, a.adjoint_ckpt, a.with_oracle, a.viscosity)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
