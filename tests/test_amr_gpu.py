"""The reference's segregated scheme on adaptively refined meshes (2:1
non-conforming faces) on the GPU through the C ABI, against the oracle's
mortar restatement (itself bit-identical to the unmodified euler binary,
tests/test_amr_oracle.py).  With the correctly rounded pow in the oracle the
GPU result is bit for bit (the precision form on these meshes:
tests/test_mixed_mortar.py)."""
import numpy as np
import pytest

import oracle
from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["amr_c1_2d_visc", "amr_g3_4n3", "amr_hill_2d_visc"])
def test_amr_segregated_gpu_bitwise_vs_oracle(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    n = int(g["meta"][7])
    dt, steps = float(g["dt"]), int(g["nsteps"])
    rho0, U0, T0 = g["fld0_rho"], g["fld0_U"].reshape(n, 3), g["fld0_T"]
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    try:
        r_o, u_o, t_o = m.segregated(rho0, U0, T0, dt, steps)
    finally:
        oracle.set_pow(0)
    s = ng.Solver(g, dt=dt)
    s.set_fields(rho0, U0, T0)
    s.step(steps // 2, scheme=ng.REF_SEGREGATED)
    s.step(steps - steps // 2, scheme=ng.REF_SEGREGATED)
    r, u, t = s.get_fields()
    assert np.array_equal(r, r_o)
    assert np.array_equal(u, np.asarray(u_o).reshape(n, 3))
    assert np.array_equal(t, t_o)
    # against the binary: the C library pow's last bits only (measured up to
    # 1.4e-14 in rho, on the curved refined mesh)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    assert rel(r, g["fldN_rho"]) <= 3e-14
    assert rel(t, g["fldN_T"]) <= 1e-10
    s.close()


VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")


@pytest.mark.parametrize("case", ["amr_c1_2d_visc", "amr_g3_4n3", "amr_hill_2d_visc"])
def test_amr_coupled_fp64_gpu_bitwise_vs_oracle(case):
    """The plain FP64 form (tendency and SSP-RK3) on the refined meshes: bit
    for bit the oracle with the correctly rounded pow; the oracle itself is
    bit for bit the reference's operators (tests/test_amr_oracle.py)."""
    import nebulasem_gb300 as ng
    g = load_golden(case)
    dt, steps = float(g["dt"]), int(g["rk_steps"])
    u0 = [g[f"u0_{v}"] for v in VARS]
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    try:
        L_o = m.tendency(u0)
        u_o = m.ssprk3(u0, dt, steps)
    finally:
        oracle.set_pow(0)
    s = ng.Solver(g, dt=dt)
    s.set_state(u0)
    L = s.tendency()
    for a, b, v in zip(L, L_o, VARS):
        assert np.array_equal(a, b), v
    s.step(steps)
    for a, b, v in zip(s.get_state(), u_o, VARS):
        assert np.array_equal(a, b), v
    s.close()
