"""The oracle's restatement of the reference's scalar DG convection
(apps/convection/convection.cpp, problem_init NONE, BDF1) reproduces the
unmodified reference `convection` app bit for bit (fixtures
tests/golden/conv_*.npz, made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle
from conftest import load_golden


@pytest.mark.parametrize("case", ["conv_c1_2d", "conv_g3_2", "conv_amr_c1_2d"])
def test_convection_oracle_matches_reference_binary(case):
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    n = m.n_int
    t = m.convection(g["fld0_U"].reshape(n, 3), g["fld0_T"], float(g["dt"]), int(g["nsteps"]))
    assert np.array_equal(t, g["fldN_T"])
    assert np.abs(t - g["fld0_T"]).max() > 1e-3
