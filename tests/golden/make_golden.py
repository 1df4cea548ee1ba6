"""Generate the golden fixtures from the reference library itself.

Builds the reference NebulaSEM sources (read-only checkout given by --ref)
with oracle/Makefile.ref into oracle/_ref, writes rising-bubble case
directories (oracle/make_case.py), runs the reference mesh app and the oracle
harness (oracle/ref_harness.cpp, which calls the reference's own divf /
rusanov / applyExplicitBCs), and stores per case one compressed .npz:

  geometry  meta, cC, cV, Jinv, FO, FN, fN, fI, allFaces, faceIdx0/1,
            xgl/wgl/psi/dpsi per direction, bcU, p_ref, rho_ref, gh
  states    u0_* (initial, at rest), L0_* (its tendency), up_* (smooth
            velocity perturbation), Lp_*, p0prime/ppprime (p - p_ref),
            traj_<step>_* (coupled SSP-RK3 states after <step> steps)

Segregated-scheme fixtures (seg_<case>.npz): the unmodified reference `euler`
binary (its own time loop, euler.cpp:179-287, BDF1) runs the case for N steps
and writes its fields; stored are the geometry, the step-0 fields as the solver
holds them (rho, U, T = theta', from the harness) and the binary's step-N
fields read back from its binary field files.

Scalar convection fixtures (conv_<case>.npz): the unmodified reference
`convection` app on a uniform wind; geometry, step-0 fields and its step-N T.

Run in the build container (the reference is not present on GPU machines):
  python tests/golden/make_golden.py --ref <reference source tree>
"""
import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import load_dump  # noqa: E402
from oracle.make_case import CASES, write_case  # noqa: E402

VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")

# fixture -> (dt, start state, [dump steps], total steps[, case, viscosity])
PLAN = {
    "c1_2d": (0.0175, "rest", [50, 500], 500),
    "g3_2": (0.01, "pert", [20], 20),
    "g3_4n3": (0.01, "pert", [10, 30], 30),
    "g3_2n7": (0.005, "pert", [10], 10),
    # coupled SSP-RK3 with the artificial viscosity of diffusion YES
    "g3_2_visc": (0.01, "pert", [10], 10, "g3_2", 1.5),
    "c1_2d_visc": (0.005, "rest", [40], 40, "c1_2d", 1.5),
}

# fixture -> (case, dt, steps, artificial viscosity, time scheme) for the
# segregated scheme, at steps the scheme keeps stable; viscosity 1.5 as the
# reference's srtb example; AB1 as its srtb-3d example (same arithmetic as BDF1)
SEG_PLAN = {
    "c1_2d": ("c1_2d", 0.005, 100, 0.0, "BDF1"),
    "g3_2": ("g3_2", 0.005, 30, 0.0, "BDF1"),
    "c1_2d_visc": ("c1_2d", 0.005, 30, 1.5, "BDF1"),
    "g3_2_visc": ("g3_2", 0.005, 10, 1.5, "BDF1"),
    "g3_2_visc_ab1": ("g3_2", 0.005, 10, 1.5, "AB1"),
    # the reference's srtb example as shipped: its viscosity and gravity, the
    # Fluid:: defaults for P0, cp, cv (examples/atmo/srtb/controls)
    "srtb": ("c1_2d", 0.005, 100, 1.5, "BDF1", "srtb"),
    # curved blocks: the srtb-curved example's arcs, and a cosine hill
    "srtb_curved": ("c1_2d", 0.005, 100, 1.5, "BDF1", "srtb", "arc_y"),
    "hill": ("c1_2d", 0.005, 100, 1.5, "BDF1", "srtb", "hill"),
    # wall grading with odd counts (one more division, the factor inversion)
    "graded": ("c1_2d", 0.005, 50, 1.5, "BDF1", "srtb", None, ((9, 1, 9), (0.5, 1.0, 2.0))),
}

# fixture -> (case, dt, steps, artificial viscosity, refinement threshold) for
# the segregated scheme on a mesh refined once by the reference's prepare
# -refine (2:1 non-conforming faces): 2D with viscosity, 3D with 2x2 mortars
AMR_PLAN = {
    "c1_2d_visc": ("c1_2d", 0.005, 20, 1.5, 0.3),
    "g3_4n3": ("g3_4n3", 0.005, 10, 0.0, 0.2),
    # the block under the cosine hill, refined (curved and non-conforming)
    "hill_2d_visc": ("c1_2d", 0.005, 20, 1.5, 0.3, "hill"),
}

# fixture -> (case, dt, steps, wind[, refinement threshold]) for the
# reference's scalar convection app; with a threshold the mesh is refined once
# by prepare -refine first (2:1 non-conforming faces)
CONV_PLAN = {
    "c1_2d": ("c1_2d", 0.5, 40, (5.0, 0.0, 3.0)),
    "g3_2": ("g3_2", 1.0, 30, (6.0, -4.0, 5.0)),
    "amr_c1_2d": ("c1_2d", 0.5, 40, (5.0, 0.0, 3.0), 0.3),
    "amr_g3_4n3": ("g3_4n3", 1.0, 30, (6.0, -4.0, 5.0), 0.2),
}

# the advection-leveque example made small: n x n elements, order, dt, steps
LEVEQUE_PLAN = {
    "leveque_ab2": (8, 4, 0.0005, 40),
}

KEEP_F64 = ["cC", "cV", "Jinv", "fN", "fI", "p_ref", "rho_ref", "gh",
            "xgl0", "xgl1", "xgl2", "wgl0", "wgl1", "wgl2",
            "psi0", "psi1", "psi2", "dpsi0", "dpsi1", "dpsi2"]
KEEP_U32 = ["meta", "FO", "FN", "allFaces", "faceIdx0", "faceIdx1", "bcU"]


def run(cmd, cwd, threads=8):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    subprocess.run(cmd, cwd=cwd, check=True, env=env, stdout=subprocess.DEVNULL)


def make_case(name, ref_bin, tmp):
    dt, start, dumps, nsteps = PLAN[name][:4]
    base = PLAN[name][4] if len(PLAN[name]) > 4 else name
    visc = PLAN[name][5] if len(PLAN[name]) > 5 else 0.0
    case = os.path.join(tmp, name)
    write_case(case, dt=dt, steps=nsteps, viscosity=visc, **CASES[base])
    run([os.path.join(ref_bin, "mesh"), "grid", "-o", "grid_0.bin"], case)
    os.makedirs(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler_oracle"), "./controls", "setup", "out"], case)
    d = load_dump(os.path.join(case, "out"))
    os.makedirs(os.path.join(case, "rk"))
    every = dumps[0] if len(dumps) == 1 else int(np.gcd.reduce(dumps))
    args = [os.path.join(ref_bin, "euler_oracle"), "./controls", "rk3", "rk",
            str(nsteps), str(every)]
    if start == "pert":
        args.append("pert")
    run(args, case)
    r = load_dump(os.path.join(case, "rk"))
    n_int = int(d["meta"][7])
    out = {k: d[k] for k in KEEP_F64 + KEEP_U32}
    for tag in ("u0", "L0", "up", "Lp"):
        for v in VARS:
            out[f"{tag}_{v}"] = d[f"{tag}_{v}"]
    out["p0prime"] = d["p0prime"][:n_int]
    out["ppprime"] = d["ppprime"][:n_int]
    for s in dumps:
        for v in VARS:
            out[f"traj_{s}_{v}"] = r[f"s{s:05d}_{v}"]
    out["dt"] = np.float64(dt)
    out["viscosity"] = np.float64(visc)
    out["Pr"] = np.float64(0.9)
    out["start"] = np.array(start)
    out["steps"] = np.array(dumps, dtype=np.int64)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {n_int} interior nodes -> {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


def make_seg_case(name, ref_bin, tmp):
    from nebulasem_gb300.fields import read_field
    from oracle.make_case import SRTB_FLUID
    base, dt, nsteps, visc, scheme = SEG_PLAN[name][:5]
    fluid = dict(SRTB_FLUID) if len(SEG_PLAN[name]) > 5 else {}
    fluid.pop("viscosity", None)
    curved = SEG_PLAN[name][6] if len(SEG_PLAN[name]) > 6 else None
    grading = SEG_PLAN[name][7] if len(SEG_PLAN[name]) > 7 else None
    case = os.path.join(tmp, "seg_" + name)
    write_case(case, dt=dt, steps=nsteps, viscosity=visc, time_scheme=scheme, **fluid,
               **CASES[base], curved=curved, grading=grading)
    run([os.path.join(ref_bin, "mesh"), "grid", "-o", "grid_0.bin"], case)
    os.makedirs(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler_oracle"), "./controls", "setup", "out"], case)
    d = load_dump(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler"), "./controls"], case)
    n_int = int(d["meta"][7])
    out = {k: d[k] for k in KEEP_F64 + KEEP_U32}
    out["fld0_rho"] = d["fld_rho"][:n_int]
    out["fld0_U"] = d["fld_U"][:3 * n_int]
    out["fld0_T"] = d["fld_T"][:n_int]
    for f in ("rho", "U", "T"):
        v = read_field(os.path.join(case, f"{f}1.bin")).values
        assert v.shape[0] == n_int
        out[f"fldN_{f}"] = v.reshape(-1)
    out["dt"] = np.float64(dt)
    out["nsteps"] = np.int64(nsteps)
    out["viscosity"] = np.float64(visc)
    out["Pr"] = np.float64(0.9)
    if curved:
        out["curved"] = np.array(curved)
    if grading:
        out["grading"] = np.array(grading, dtype=np.float64)
    if fluid:
        # constants in the names the oracle and the Python host read
        out["P0"] = np.float64(fluid["P0"])
        out["cp"] = np.float64(fluid["cp"])
        out["cv"] = np.float64(fluid["cv"])
        out["R"] = np.float64(fluid["cp"] - fluid["cv"])
        out["gamma"] = np.float64(fluid["cp"] / fluid["cv"])
        out["gravity"] = np.array([0.0, 0.0, fluid["gz"]])
    path = os.path.join(HERE, f"seg_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"seg_{name}: {n_int} interior nodes, {nsteps} steps -> {path} "
          f"({os.path.getsize(path) / 1e6:.2f} MB)")


def make_amr_case(name, ref_bin, tmp):
    """Segregated-scheme fixture on an adaptively refined mesh: the mesh app's
    grid refined once by the reference's prepare -refine, the harness's dump
    of that mesh (with its non-conforming faces and 2:1 tables) and initial
    state, and the unmodified euler binary's fields after the steps."""
    from nebulasem_gb300.fields import read_field
    base, dt, nsteps, visc, fmax = AMR_PLAN[name][:5]
    curved = AMR_PLAN[name][5] if len(AMR_PLAN[name]) > 5 else None
    case = os.path.join(tmp, "amr_" + name)
    write_case(case, dt=dt, steps=nsteps, viscosity=visc, refine=fmax, curved=curved,
               **CASES[base])
    run([os.path.join(ref_bin, "mesh"), "grid", "-o", "grid_0.bin"], case)
    run([os.path.join(ref_bin, "prepare"), "./controls", "-refine"], case)
    os.makedirs(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler_oracle"), "./controls", "setup", "out"], case)
    d = load_dump(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler"), "./controls"], case)
    n_int = int(d["meta"][7])
    out = {k: d[k] for k in KEEP_F64 + KEEP_U32}
    # the coupled form on the same mesh: the harness's tendency at its start
    # state and its SSP-RK3 trajectory over the reference's own operators
    rk_steps = 5
    os.makedirs(os.path.join(case, "rk"))
    run([os.path.join(ref_bin, "euler_oracle"), "./controls", "rk3", "rk", str(rk_steps),
         str(rk_steps)], case)
    r = load_dump(os.path.join(case, "rk"))
    for v in VARS:
        out[f"u0_{v}"] = d[f"u0_{v}"]
        out[f"L0_{v}"] = d[f"L0_{v}"]
        out[f"rk_{v}"] = r[f"s{rk_steps:05d}_{v}"]
    out["rk_steps"] = np.int64(rk_steps)
    out["mortar"] = d["mortar"]
    assert len(out["mortar"]) > 0, "no cell was refined"
    for dd in range(3):
        for h in range(2):
            out[f"psiRef{dd}{h}"] = d[f"psiRef{dd}{h}"]
            out[f"psiCor{dd}{h}"] = d[f"psiCor{dd}{h}"]
    out["fld0_rho"] = d["fld_rho"][:n_int]
    out["fld0_U"] = d["fld_U"][:3 * n_int]
    out["fld0_T"] = d["fld_T"][:n_int]
    for f in ("rho", "U", "T"):
        v = read_field(os.path.join(case, f"{f}1.bin")).values
        assert v.shape[0] == n_int
        out[f"fldN_{f}"] = v.reshape(-1)
    out["dt"] = np.float64(dt)
    out["nsteps"] = np.int64(nsteps)
    out["viscosity"] = np.float64(visc)
    out["Pr"] = np.float64(0.9)
    path = os.path.join(HERE, f"amr_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"amr_{name}: {n_int} interior nodes, {len(out['mortar']) // 4} mortar faces, "
          f"{nsteps} steps -> {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


def make_conv_case(name, ref_bin, tmp):
    """Scalar convection fixture: the unmodified reference `convection` app
    (convection.cpp, problem_init NONE, BDF1) on a uniform wind; geometry and
    the step-0 fields from the harness (run on a copy of the controls naming
    the euler solver, which the harness binary requires)."""
    from nebulasem_gb300.fields import read_field
    base, dt, nsteps, wind = CONV_PLAN[name][:4]
    fmax = CONV_PLAN[name][4] if len(CONV_PLAN[name]) > 4 else None
    case = os.path.join(tmp, "conv_" + name)
    write_case(case, dt=dt, steps=nsteps, solver="convection", wind=wind, refine=fmax,
               **CASES[base])
    with open(os.path.join(case, "controls")) as f:
        ctl = f.read()
    with open(os.path.join(case, "controls_setup"), "w") as f:
        f.write(ctl.replace("solver                       convection",
                            "solver                       euler"))
    run([os.path.join(ref_bin, "mesh"), "grid", "-o", "grid_0.bin"], case)
    if fmax:
        run([os.path.join(ref_bin, "prepare"), "./controls_setup", "-refine"], case)
    os.makedirs(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler_oracle"), "./controls_setup", "setup", "out"], case)
    d = load_dump(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "convection"), "./controls"], case)
    n_int = int(d["meta"][7])
    out = {k: d[k] for k in KEEP_F64 + KEEP_U32}
    if fmax:
        assert len(d["mortar"]) > 0, "no cell was refined"
        out["mortar"] = d["mortar"]
        for dd in range(3):
            for h in range(2):
                out[f"psiRef{dd}{h}"] = d[f"psiRef{dd}{h}"]
                out[f"psiCor{dd}{h}"] = d[f"psiCor{dd}{h}"]
    out["fld0_U"] = d["fld_U"][:3 * n_int]
    out["fld0_T"] = d["fld_T"][:n_int]
    v = read_field(os.path.join(case, "T1.bin")).values
    assert v.shape[0] == n_int
    out["fldN_T"] = v.reshape(-1)
    out["dt"] = np.float64(dt)
    out["nsteps"] = np.int64(nsteps)
    path = os.path.join(HERE, f"conv_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"conv_{name}: {n_int} interior nodes, {nsteps} steps -> {path} "
          f"({os.path.getsize(path) / 1e6:.2f} MB)")


def make_leveque_case(name, ref_bin, tmp):
    """The unmodified `convection` app with problem_init LEVEQUE and AB2: the
    wind's spatial part on every node and its time factors (C library sin,
    cos, pow, as the app evaluates them), step-0 and step-N scalar."""
    from nebulasem_gb300.fields import read_field
    from oracle.make_case import leveque_wind, write_leveque_case

    n, order, dt, nsteps = LEVEQUE_PLAN[name]
    case = os.path.join(tmp, "conv_" + name)
    write_leveque_case(case, n=n, order=order, dt=dt, steps=nsteps)
    run([os.path.join(ref_bin, "mesh"), "grid", "-o", "grid_0.bin"], case)
    os.makedirs(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "euler_oracle"), "./controls_setup", "setup", "out"], case)
    d = load_dump(os.path.join(case, "out"))
    run([os.path.join(ref_bin, "convection"), "./controls"], case)
    n_int = int(d["meta"][7])
    out = {k: d[k] for k in KEEP_F64 + KEEP_U32}
    A, scale = leveque_wind(d["cC"], nsteps, dt)
    out["wind_all"] = np.asarray(A, dtype=np.float64).reshape(-1)
    out["wind_scale"] = np.asarray(scale, dtype=np.float64)
    out["fld0_T"] = d["fld_T"][:n_int]
    v = read_field(os.path.join(case, "T1.bin")).values
    assert v.shape[0] == n_int
    out["fldN_T"] = v.reshape(-1)
    out["dt"] = np.float64(dt)
    out["nsteps"] = np.int64(nsteps)
    out["time_scheme"] = np.int64(2)
    np.savez_compressed(os.path.join(HERE, f"conv_{name}.npz"), **out)
    print("wrote", f"conv_{name}.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference NebulaSEM source tree")
    ap.add_argument("--cases", nargs="*", default=sorted(PLAN))
    ap.add_argument("--seg-cases", nargs="*", default=sorted(SEG_PLAN))
    ap.add_argument("--conv-cases", nargs="*", default=sorted(CONV_PLAN))
    ap.add_argument("--amr-cases", nargs="*", default=sorted(AMR_PLAN))
    ap.add_argument("--leveque-cases", nargs="*", default=sorted(LEVEQUE_PLAN))
    ap.add_argument("-j", type=int, default=8)
    a = ap.parse_args()
    subprocess.run(["make", "-f", "oracle/Makefile.ref", f"REF={a.ref}", f"-j{a.j}"],
                   cwd=ROOT, check=True)
    ref_bin = os.path.join(ROOT, "oracle", "_ref")
    tmp = tempfile.mkdtemp(prefix="nsem_golden_")
    try:
        for name in a.cases:
            make_case(name, ref_bin, tmp)
        for name in a.seg_cases:
            make_seg_case(name, ref_bin, tmp)
        for name in a.conv_cases:
            make_conv_case(name, ref_bin, tmp)
        for name in a.leveque_cases:
            make_leveque_case(name, ref_bin, tmp)
        for name in a.amr_cases:
            make_amr_case(name, ref_bin, tmp)
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
