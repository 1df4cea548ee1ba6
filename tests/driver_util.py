"""Helpers for the host-driver tests: write a case directory in the
reference's input formats, run nsem_euler in it, read what it wrote."""
import os
import subprocess

import numpy as np

from conftest import ROOT

from oracle import load_dump
from oracle.make_case import CASES, write_case


def driver_exe():
    from nebulasem_gb300 import build
    build.build()
    return build.DRIVER_EXE


def make_case(tmp, case, **kw):
    d = os.path.join(str(tmp), case)
    write_case(d, **{**CASES[case], **kw})
    return d


def rotate_case_z(case_dir, deg):
    """Rotate a 2D case's key points about the z axis through the origin by deg
    degrees (a parallelepiped block as the reference's srtb-inclined example);
    the bubble centre in T0.txt rotates with it."""
    import math
    c, s_ = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    path = os.path.join(case_dir, "grid")
    lines = open(path).read().split("\n")
    n = int(lines[0])
    for q in range(2, 2 + n):
        x, y, z = (float(v) for v in lines[q].split())
        lines[q] = f"{c * x - s_ * y!r} {s_ * x + c * y!r} {z!r}"
    open(path, "w").write("\n".join(lines))
    t = os.path.join(case_dir, "T0.txt")
    txt = open(t).read()
    import re
    m = re.search(r"cosine (\S+) (\S+)\s+(\S+) (\S+) (\S+)\s+(\S+) (\S+) (\S+)", txt)
    v, a, cx, cy, cz, rx, ry, rz = (float(g) for g in m.groups())
    # the initialiser's radii scale the global axes: a bubble that is round in
    # x and y (ry = rx) keeps its shape under a rotation about z (every node of
    # the unrotated 2D case lies in the bubble centre's y plane, so ry does not
    # matter there)
    ncx, ncy = c * cx - s_ * cy, s_ * cx + c * cy
    new = f"cosine {v!r} {a!r}    {ncx!r} {ncy!r} {cz!r}   {rx!r} {rx!r} {rz!r}"
    open(t, "w").write(txt[:m.start()] + new + txt[m.end():])


def run_driver(case_dir, *args, check=True):
    r = subprocess.run([driver_exe(), "./controls", *args], cwd=case_dir, capture_output=True,
                       text=True, timeout=600)
    if check and r.returncode != 0:
        raise AssertionError(f"nsem_euler failed ({r.returncode}):\n{r.stdout}\n{r.stderr}")
    return r


def dump_case(case_dir):
    out = os.path.join(case_dir, "dump")
    run_driver(case_dir, "--dump", out)
    return load_dump(out)


def node_order(cC, n):
    """Permutation sorting the first n nodes by (x, y, z) rounded to 1e-6 m."""
    c = np.asarray(cC).reshape(-1, 3)[:n]
    return np.lexsort((np.round(c[:, 2], 6), np.round(c[:, 1], 6), np.round(c[:, 0], 6)))


__all__ = ["ROOT", "driver_exe", "make_case", "run_driver", "dump_case", "node_order",
           "rotate_case_z"]
