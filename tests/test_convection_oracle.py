"""The oracle's restatement of the reference's scalar DG convection
(apps/convection/convection.cpp, problem_init NONE, BDF1) reproduces the
unmodified reference `convection` app bit for bit (fixtures
tests/golden/conv_*.npz, made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle
from conftest import load_golden


@pytest.mark.parametrize("case", ["conv_c1_2d", "conv_g3_2", "conv_amr_c1_2d", "conv_amr_g3_4n3"])
def test_convection_oracle_matches_reference_binary(case):
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    n = m.n_int
    t = m.convection(g["fld0_U"].reshape(n, 3), g["fld0_T"], float(g["dt"]), int(g["nsteps"]))
    assert np.array_equal(t, g["fldN_T"])
    assert np.abs(t - g["fld0_T"]).max() > 1e-3


def test_convection_oracle_leveque_ab2_matches_reference_binary():
    """problem_init LEVEQUE (analytic wind, ghosts included, scaled by
    cos(pi t / T) every step) with time_scheme AB2 (first step AB1): the
    unmodified app's step-N scalar bit for bit; AB1 alone differs."""
    g = load_golden("conv_leveque_ab2")
    m = oracle.OracleMesh(g)
    A = g["wind_all"].reshape(-1, 3)[:m.n_all]
    dt, steps = float(g["dt"]), int(g["nsteps"])
    t = m.convection_wind(A, g["wind_scale"], 2, g["fld0_T"], dt, steps)
    assert np.array_equal(t, g["fldN_T"])
    t1 = m.convection_wind(A, g["wind_scale"], 1, g["fld0_T"], dt, steps)
    assert np.abs(t1 - g["fldN_T"]).max() > 1e-4
