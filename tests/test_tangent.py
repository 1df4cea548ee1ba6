"""Tangent-linear form on the GPU (nsem_jvp, nsem_tlm) against the CPU dual-number
tangent-linear oracle, and its duality with the adjoint (nsem_vjp, nsem_adjoint)."""
import numpy as np
import pytest

import oracle
from conftest import golden_state, load_golden

pytestmark = pytest.mark.gpu


def dot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


def rel(a, b):
    return float(np.sqrt(sum(np.sum((x - y) ** 2) for x, y in zip(a, b))) /
                 np.sqrt(sum(np.sum(y ** 2) for y in b)))


def perturbation(rng, u):
    # relative: keeps the SYMMETRY ghost on the branch of the value (see
    # tests/test_oracle_tlm.py)
    return [a * rng.standard_normal(a.shape[0]) * 1e-2 for a in u]


@pytest.mark.parametrize("case", ["g3_2", "g3_4n3", "c1_2d", "g3_2n7"])
def test_jvp_vs_cpu_tangent_and_vjp(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    u = golden_state(g, "up")
    s = ng.Solver(g, dt=float(g["dt"]))
    s.set_state(u)
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    rng = np.random.default_rng(5)
    for trial in range(2):
        dv = perturbation(rng, u)
        _, Ld_cpu = m.jvp(u, dv)
        Ld = s.jvp(dv)
        assert rel(Ld, Ld_cpu) <= 1e-11, (case, trial, rel(Ld, Ld_cpu))
        # duality with the vector-Jacobian product on the GPU
        w = [rng.standard_normal(m.n_int) for _ in range(5)]
        lhs, rhs = dot(w, Ld), dot(s.vjp(w), dv)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= 1e-11 * scale, (case, trial, lhs, rhs)
    oracle.set_pow(0)
    s.close()


def test_tlm_trajectory_vs_cpu_and_adjoint_duality():
    import nebulasem_gb300 as ng
    g = load_golden("g3_2")
    u = golden_state(g, "up")
    dt, steps = float(g["dt"]), 12
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    rng = np.random.default_rng(9)
    du0 = perturbation(rng, u)
    uT_cpu, duT_cpu = m.tlm_ssprk3(u, du0, dt, steps)
    oracle.set_pow(0)

    s = ng.Solver(g, dt=dt)
    s.set_state(u)
    duT, ms = s.tlm(steps, du0)
    uT = s.get_state()
    assert all(np.array_equal(a, b) for a, b in zip(uT, uT_cpu))   # same trajectory
    assert rel(duT, duT_cpu) <= 1e-10, rel(duT, duT_cpu)
    assert ms > 0

    # <lam_N, du_N> = <lam_0, du_0> for the adjoint of the same steps
    lamN = [rng.standard_normal(m.n_int) for _ in range(5)]
    s.set_state(u)
    s.forward_checkpointed(steps, 5)
    lam0, _ = s.adjoint(lamN)
    lhs, rhs = dot(lamN, duT), dot(lam0, du0)
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (lhs, rhs)
    s.close()


@pytest.mark.parametrize("case", ["g3_2_visc", "c1_2d_visc"])
def test_viscous_jvp_tlm_and_adjoint(case):
    """With the artificial viscosity: the tangent of the viscous fluxes
    (d(mu grad U) with the gradients' own tangent, the SYMMETRY ghost
    linearised) against the dual-number oracle, one tendency and a 10-step
    trajectory; the adjoint (the gradients' transpose) by duality with it."""
    import nebulasem_gb300 as ng
    g = load_golden(case)
    u = golden_state(g, "up")
    dt = float(g["dt"])
    s = ng.Solver(g, dt=dt)
    s.set_state(u)
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    rng = np.random.default_rng(13)
    dv = perturbation(rng, u)
    _, Ld_cpu = m.jvp(u, dv)
    Ld = s.jvp(dv)
    assert rel(Ld, Ld_cpu) <= 1e-11, (case, rel(Ld, Ld_cpu))
    uT_cpu, duT_cpu = m.tlm_ssprk3(u, dv, dt, 10)
    oracle.set_pow(0)
    s.set_state(u)
    duT, _ = s.tlm(10, dv)
    assert all(np.array_equal(a, b) for a, b in zip(s.get_state(), uT_cpu))
    assert rel(duT, duT_cpu) <= 1e-10, (case, rel(duT, duT_cpu))
    # the adjoint of the viscous terms: duality with the tangent, one tendency
    # (<w, J dv> = <J^T w, dv>) and the 10-step trajectory (<lam_N, du_N> =
    # <lam_0, du_0>)
    s.set_state(u)
    for trial in range(2):
        w = [rng.standard_normal(m.n_int) for _ in range(5)]
        Ld = s.jvp(dv)
        lhs, rhs = dot(w, Ld), dot(s.vjp(w), dv)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= 1e-11 * scale, (case, trial, lhs, rhs)
    lamN = [rng.standard_normal(m.n_int) for _ in range(5)]
    s.set_state(u)
    s.forward_checkpointed(10, 5)
    lam0, _ = s.adjoint(lamN)
    lhs, rhs = dot(lamN, duT), dot(lam0, dv)
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (case, lhs, rhs)
    s.close()
