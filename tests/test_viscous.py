"""Coupled SSP-RK3 FP64 form with the artificial viscosity of diffusion YES on
the GPU, bit for bit against the oracle (correctly rounded pow), which matches
the reference library's own chain bit for bit (tests/test_viscous_oracle.py)."""
import numpy as np
import pytest

import oracle
from conftest import VARS, golden_state, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["g3_2_visc", "c1_2d_visc"])
def test_viscous_fp64_bitwise_vs_oracle(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    dt = float(g["dt"])
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    s = ng.Solver(g, dt=dt)
    up = golden_state(g, "up")
    s.set_state(up)
    L = s.tendency()
    for a, b, v in zip(L, m.tendency(up), VARS):
        assert np.array_equal(a, b), (case, "tendency", v)
    start = golden_state(g, "up" if str(g["start"]) == "pert" else "u0")
    steps = int(g["steps"][-1])
    s.set_state(start)
    s.step(steps // 2)
    s.step(steps - steps // 2)
    got = s.get_state()
    want = m.ssprk3(start, dt, steps)
    oracle.set_pow(0)
    for a, b, v in zip(got, want, VARS):
        assert np.array_equal(a, b), (case, "trajectory", v)
    s.close()


@pytest.mark.parametrize("case", ["g3_2_visc", "c1_2d_visc"])
def test_viscous_precision_form_vs_fp64(case):
    """The precision form with the artificial viscosity (FP32 gradients of
    the stage state, viscous volume and face fluxes) against the FP64 form:
    tendency and trajectory within the form's 1e-5 relative L2."""
    import nebulasem_gb300 as ng
    from conftest import rel_l2
    g = load_golden(case)
    dt = float(g["dt"])
    s = ng.Solver(g, dt=dt)
    up = golden_state(g, "up")
    s.set_state(up)
    L64 = s.tendency(prec=ng.FP64)
    L32 = s.tendency(prec=ng.MIXED)
    scale = max(np.linalg.norm(x) for x in L64)
    for a, b, v in zip(L32, L64, VARS):
        if np.linalg.norm(b) < 1e-8 * scale:
            continue
        assert rel_l2(a, b) <= 1e-5, (case, v, rel_l2(a, b))
    # the viscous terms are present: dropping them moves the momentum
    # tendency far more than the precision form's own error
    s_inv = ng.Solver(g, dt=dt, viscosity=0.0)
    s_inv.set_state(up)
    L_inv = s_inv.tendency(prec=ng.MIXED)
    s_inv.close()
    mom = [c for c in (1, 2, 3) if np.linalg.norm(L64[c]) >= 1e-8 * scale]
    d_inv = max(rel_l2(L_inv[c], L64[c]) for c in mom)
    d_mix = max(rel_l2(L32[c], L64[c]) for c in mom)
    assert d_inv > 1e-5 and d_inv > 10 * d_mix, (d_inv, d_mix)
    start = golden_state(g, "up" if str(g["start"]) == "pert" else "u0")
    steps = int(g["steps"][-1])
    s.set_state(start)
    s.step(steps, prec=ng.FP64)
    ref = s.get_state()
    s.set_state(start)
    s.step(steps, prec=ng.MIXED)
    got = s.get_state()
    # rho and rho theta per variable; momentum as one vector field (from rest
    # the horizontal components are still ~1e-4 of the vertical one here)
    for c in (0, 4):
        assert rel_l2(got[c], ref[c]) <= 1e-5, (case, VARS[c], rel_l2(got[c], ref[c]))
    mom = rel_l2(np.stack(got[1:4]), np.stack(ref[1:4]))
    assert mom <= 1e-5, (case, "momentum", mom)
    s.close()


def test_viscous_precision_form_3d_bubble():
    """16^3 N=4 bubble with viscosity 1.5, 40 steps: precision vs FP64."""
    import nebulasem_gb300 as ng
    from conftest import rel_l2
    from nebulasem_gb300.mesh import workload
    m, u = workload("bubble3d_16_n4")
    s = ng.Solver(m, dt=0.005, viscosity=1.5, Pr=0.9)
    s.set_state(u)
    s.step(40, prec=ng.FP64)
    ref = s.get_state()
    s.set_state(u)
    s.step(40, prec=ng.MIXED)
    got = s.get_state()
    for c in (0, 4):
        assert rel_l2(got[c], ref[c]) <= 1e-5, (VARS[c], rel_l2(got[c], ref[c]))
    mom = rel_l2(np.stack(got[1:4]), np.stack(ref[1:4]))
    assert mom <= 1e-5, ("momentum", mom)
    s.close()
