"""The oracle's restatement of the reference's own time update (segregated
forward Euler, euler.cpp:179-287 with BDF1; with and without the artificial
viscosity of diffusion YES) reproduces the unmodified reference
`euler` binary bit for bit (fixtures tests/golden/seg_*.npz, made by
tests/golden/make_golden.py from the binary's field files)."""
import numpy as np
import pytest

import oracle
from conftest import load_golden


@pytest.mark.parametrize("case", ["seg_c1_2d", "seg_g3_2", "seg_c1_2d_visc", "seg_g3_2_visc",
                                  "seg_g3_2_visc_ab1", "seg_srtb"])
def test_segregated_oracle_matches_reference_binary(case):
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    n = m.n_int
    oracle.set_pow(0)   # the reference's C library pow
    r, u, t = m.segregated(g["fld0_rho"], g["fld0_U"].reshape(n, 3), g["fld0_T"],
                           float(g["dt"]), int(g["nsteps"]))
    assert np.array_equal(r, g["fldN_rho"])
    assert np.array_equal(u.reshape(-1), g["fldN_U"])
    assert np.array_equal(t, g["fldN_T"])
    # and the run moved the state
    assert not np.array_equal(r, g["fld0_rho"])
