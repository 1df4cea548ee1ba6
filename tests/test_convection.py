"""Scalar DG convection on the GPU (nsem_convection_*) against the oracle's
restatement, which is pinned bit for bit to the reference's `convection` app
(tests/test_convection_oracle.py): no pow enters, so the GPU result equals the
reference's bit for bit."""
import numpy as np
import pytest

import oracle
from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["conv_c1_2d", "conv_g3_2", "conv_amr_c1_2d", "conv_amr_g3_4n3"])
def test_convection_gpu_bitwise_vs_reference(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    n = int(g["meta"][7])
    dt, steps = float(g["dt"]), int(g["nsteps"])
    U = g["fld0_U"].reshape(n, 3)
    s = ng.Solver(g, dt=dt)
    s.convection_set(U, g["fld0_T"])
    s.convection_step(steps // 3)
    s.convection_step(steps - steps // 3)
    t = s.convection_get()
    assert np.array_equal(t, g["fldN_T"])
    m = oracle.OracleMesh(g)
    assert np.array_equal(t, m.convection(U, g["fld0_T"], dt, steps))
    s.close()


def test_convection_gpu_leveque_ab2_bitwise_vs_reference():
    """The analytic LEVEQUE wind and AB2 on the GPU, in two calls (the AB2
    history carries over): the unmodified app's scalar bit for bit."""
    import nebulasem_gb300 as ng
    g = load_golden("conv_leveque_ab2")
    n = int(g["meta"][7])
    n_all = int(g["meta"][8])
    dt, steps = float(g["dt"]), int(g["nsteps"])
    A = g["wind_all"].reshape(-1, 3)[:n_all]
    sc = g["wind_scale"]
    s = ng.Solver(g, dt=dt)
    s.convection_set(np.zeros((n, 3)), g["fld0_T"])
    s.convection_wind(A, 2)
    k = steps // 3
    s.convection_step_scaled(k, sc[:k])
    s.convection_step_scaled(steps - k, sc[k:])
    t = s.convection_get()
    assert np.array_equal(t, g["fldN_T"])
    s.close()
