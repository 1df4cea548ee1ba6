"""The oracle (C restatement) reproduces the reference library bit for bit.

The fixtures were produced by the reference's own operators
(tests/golden/make_golden.py); any drift in the restatement shows up as a
non-zero count of differing doubles.
"""
import numpy as np
import pytest

import oracle
from conftest import golden_state, load_golden

CASES = ["c1_2d", "g3_2", "g3_4n3", "g3_2n7"]


@pytest.mark.parametrize("case", CASES)
def test_tendency_bitwise(case):
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    n = m.n_int
    for tag, ltag, ptag in (("u0", "L0", "p0prime"), ("up", "Lp", "ppprime")):
        L, p = m.tendency(golden_state(g, tag), return_p=True)
        assert np.array_equal(p[:n], g[ptag]), f"{case} {tag}: p' differs"
        for a, b, v in zip(L, golden_state(g, ltag), oracle.VARS):
            assert np.array_equal(a, b), f"{case} {tag} {v}: {(a != b).sum()} values differ"


@pytest.mark.parametrize("case", CASES)
def test_ssprk3_trajectory_bitwise(case):
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    dt = float(g["dt"])
    u = golden_state(g, "u0" if str(g["start"]) == "rest" else "up")
    done = 0
    for s in g["steps"]:
        u = m.ssprk3(u, dt, int(s) - done)
        done = int(s)
        for a, b, v in zip(u, golden_state(g, f"traj_{s}"), oracle.VARS):
            assert np.array_equal(a, b), f"{case} step {s} {v}: {(a != b).sum()} differ"
