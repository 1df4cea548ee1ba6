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


__all__ = ["ROOT", "driver_exe", "make_case", "run_driver", "dump_case", "node_order"]
