"""The oracle's coupled operator chain with the artificial viscosity of
diffusion YES (mu = rho nu, strong-form DG gradients) reproduces the reference
library's own divf / rusanov / gradf chain bit for bit (fixtures made by the
reference-linked harness, tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle
from conftest import VARS, golden_state, load_golden


@pytest.mark.parametrize("case", ["g3_2_visc", "c1_2d_visc"])
def test_viscous_tendency_and_trajectory_bitwise(case):
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    assert m.struct.nu == 1.5
    for tag in ("u0", "up"):
        L = m.tendency(golden_state(g, tag))
        want = golden_state(g, "L0" if tag == "u0" else "Lp")
        for a, b, v in zip(L, want, VARS):
            assert np.array_equal(a, b), (case, tag, v)
    start = golden_state(g, "up" if str(g["start"]) == "pert" else "u0")
    step = int(g["steps"][-1])
    u = m.ssprk3(start, float(g["dt"]), step)
    for a, v in zip(u, VARS):
        assert np.array_equal(a, g[f"traj_{step}_{v}"]), (case, v)
    # the viscosity changes the result
    g0 = dict(g)
    g0["viscosity"] = 0.0
    L0 = oracle.OracleMesh(g0).tendency(golden_state(g, "up"))
    assert not np.array_equal(L0[1], golden_state(g, "Lp")[1])
