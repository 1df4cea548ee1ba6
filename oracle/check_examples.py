"""Run the reference's own atmospheric examples through the host driver's
case set-up and compare with the unmodified reference binaries
(TEST INFRASTRUCTURE; needs the reference sources and oracle/_ref).

For each example directory under <ref>/examples/atmo: copy it, shorten the
run to 20 steps written once, run the reference mesh app and `euler` on it,
let nsem_euler write its case arrays (--dump, no GPU), run the oracle's
segregated scheme (C library pow, as the reference) on those arrays, and
compare the node coordinates and the final rho, U, T with the reference's
output files node by node (nodes matched by coordinates; the reference's
geometry from the harness).  Examples the driver does not model (AMR,
multi-block meshes, spherical problems, other time schemes) are reported with
its message.

    python oracle/check_examples.py --ref <reference source tree> srtb srtb-inclined srtb-curved ctbs dc lrtb
"""
import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nebulasem_gb300.fields import read_field  # noqa: E402


def ctl_values(path, key):
    for line in open(path):
        w = line.split("#")[0].split()
        if len(w) >= 2 and w[0] == key:
            return w[1:]
    return None


def node_order(cC, n):
    c = np.asarray(cC).reshape(-1, 3)[:n]
    return np.lexsort((np.round(c[:, 2], 6), np.round(c[:, 1], 6), np.round(c[:, 0], 6)))


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def check(ref, name, tmp, steps, no_amr):
    from nebulasem_gb300 import build
    exe = build.build_driver()
    refbin = os.path.join(HERE, "_ref")
    d = os.path.join(tmp, name)
    shutil.copytree(os.path.join(ref, "examples", "atmo", name), d)
    for root, _, files in os.walk(d):
        for f in files:
            os.chmod(os.path.join(root, f), 0o644)
    ctl = os.path.join(d, "controls")
    lines = []
    for line in open(ctl).read().splitlines():
        w = line.split()
        if w and w[0] == "end_step":
            line = f"    end_step {steps}"
        elif w and w[0] == "write_interval":
            line = f"    write_interval {steps}"
        elif w and (w[0] == "print_time" or (no_amr and w[0] == "amr_step")):
            continue
        lines.append(line)
    with open(ctl, "w") as f:
        f.write("\n".join(lines) + "\n")
    grid = [f for f in os.listdir(d) if f != "controls" and not f.endswith(".txt")][0]
    r = subprocess.run([exe, "./controls", "--blocks", grid, "--dump", "dump"], cwd=d,
                       capture_output=True, text=True)
    if r.returncode:
        return dict(example=name, refused=r.stderr.strip())
    env = dict(os.environ, OMP_NUM_THREADS="8")
    subprocess.run([os.path.join(refbin, "mesh"), grid, "-o", "grid_0.bin"], cwd=d,
                   capture_output=True, check=True)
    subprocess.run([os.path.join(refbin, "euler"), "./controls"], cwd=d, capture_output=True,
                   env=env, check=True)
    os.makedirs(os.path.join(d, "out"))
    subprocess.run([os.path.join(refbin, "euler_oracle"), "./controls", "setup", "out"], cwd=d,
                   capture_output=True, env=env, check=True)
    a = oracle.load_dump(os.path.join(d, "dump"))
    g = oracle.load_dump(os.path.join(d, "out"))
    num = lambda k, dflt: float((ctl_values(ctl, k) or [dflt])[0])
    cp, cv = num("cp", 1004.67), num("cv", 715.5)
    a.update(P0=num("P0", 101325), R=cp - cv, gamma=cp / cv, T0=num("T0", 300), Pr=num("Pr", 0.9))
    gv = ctl_values(ctl, "gravity")
    a["gravity"] = np.array([float(x) for x in gv]) if gv else np.array([0, 0, -9.860616])
    diffusion = (ctl_values(ctl, "diffusion") or ["YES"])[0].upper() == "YES"
    a["viscosity"] = num("viscosity", 1.568e-5) if diffusion else 0.0
    dt = num("dt", 0.1)
    oracle.set_pow(0)
    rho, U, T = oracle.OracleMesh(a).segregated(a["fld_rho"], a["fld_U"], a["fld_T"], dt, steps)
    n = int(a["meta"][7])
    kd, kg = node_order(a["cC"], n), node_order(g["cC"], n)
    ext = ".bin" if os.path.exists(os.path.join(d, "rho1.bin")) else ".txt"
    out = {f: read_field(os.path.join(d, f + "1" + ext)).values for f in ("rho", "U", "T")}
    return dict(example=name, nodes=n, viscosity=a["viscosity"], dt=dt, steps=steps,
                reference_files=ext,
                coord_max_diff=float(np.abs(a["cC"].reshape(-1, 3)[kd]
                                            - g["cC"].reshape(-1, 3)[:n][kg]).max()),
                rho=rel_l2(rho[kd], out["rho"][kg, 0]), T=rel_l2(np.asarray(T)[kd], out["T"][kg, 0]),
                U=rel_l2(np.asarray(U).reshape(-1, 3)[kd], out["U"][kg]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference NebulaSEM source tree")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--no-amr", action="store_true", help="drop amr_step from the controls")
    ap.add_argument("examples", nargs="+")
    a = ap.parse_args()
    subprocess.run(["make", "-f", "oracle/Makefile.ref", f"REF={a.ref}", "-j8"], cwd=ROOT,
                   check=True, capture_output=True)
    tmp = tempfile.mkdtemp(prefix="nsem_examples_")
    try:
        for name in a.examples:
            print(check(a.ref, name, tmp, a.steps, a.no_amr))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
