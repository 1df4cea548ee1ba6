"""Discrete adjoint of the plain form against the CPU tangent-linear model and
finite differences.

  * dot-product test: <w, J_L(u) du> from the CPU dual-number TLM equals
    <J_L(u)^T w, du> from the GPU vector-Jacobian product;
  * gradient of J = 1/2 sum_box theta'^2 at the final time with respect to the
    initial theta' field, from the checkpointed reverse SSP-RK3 sweep, matches
    the CPU TLM directional derivative and central differences (eps = 1e-6)
    along seeded Gaussian directions.
"""
import numpy as np
import pytest

import oracle
from conftest import golden_state, load_golden

pytestmark = pytest.mark.gpu


def dot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


@pytest.mark.parametrize("case", ["g3_2", "g3_4n3", "c1_2d", "g3_2n7"])
def test_vjp_dot_product(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    u = golden_state(g, "up")
    s = ng.Solver(g, dt=float(g["dt"]))
    s.set_state(u)
    m = oracle.OracleMesh(g)
    rng = np.random.default_rng(11)
    n = m.n_int
    for trial in range(2):
        du = [rng.standard_normal(n) * sc for sc in (1e-3, 1e-1, 1e-1, 1e-1, 1e-1)]
        if case == "c1_2d":
            du[2][:] = 0.0
        w = [rng.standard_normal(n) for _ in range(5)]
        _, Ld = m.jvp(u, du)
        lhs = dot(w, Ld)
        gv = s.vjp(w)
        rhs = dot(gv, du)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= 1e-10 * scale, (case, trial, lhs, rhs, scale)
    s.close()


def test_adjoint_gradient_vs_tlm_and_fd():
    import nebulasem_gb300 as ng
    from nebulasem_gb300 import objective as ob
    g = load_golden("g3_2")
    n = int(g["meta"][7])
    xyz = g["cC"].reshape(-1, 3)[:n]
    p_ref = g["p_ref"][:n]
    u_ref = golden_state(g, "u0")
    th0 = u_ref[4] / u_ref[0] - 300.0
    u0 = ob.state_from_theta(th0, p_ref)
    mask = ob.box_mask(xyz, (800.0, 1200.0, 400.0, 1000.0))
    dt, steps, every = 0.01, 20, 5

    s = ng.Solver(g, dt=dt)
    s.set_state(u0)
    s.forward_checkpointed(steps, every)
    uN = s.get_state()
    J0 = ob.objective(uN, mask)
    assert J0 > 0
    lam0, _ = s.adjoint(ob.objective_grad(uN, mask))
    grad = ob.theta_grad(lam0, u0, th0)
    # the reverse sweep leaves the final state in place
    again = s.get_state()
    assert all(np.array_equal(a, b) for a, b in zip(again, uN))

    m = oracle.OracleMesh(g)
    rng = np.random.default_rng(2024)
    eps = 1e-6
    for d in range(3):
        v = rng.standard_normal(n)
        dj_adj = float(np.dot(grad, v))
        du0 = [-u0[0] / (th0 + 300.0) * v] + [np.zeros(n) for _ in range(4)]
        uT, duT = m.tlm_ssprk3(u0, du0, dt, steps)
        dj_tlm = dot(ob.objective_grad(uT, mask), duT)
        Jp = Jm = None
        for sign in (1.0, -1.0):
            s.set_state(ob.state_from_theta(th0 + sign * eps * v, p_ref))
            s.step(steps)
            val = ob.objective(s.get_state(), mask)
            if sign > 0:
                Jp = val
            else:
                Jm = val
        dj_fd = (Jp - Jm) / (2 * eps)
        assert abs(dj_adj - dj_tlm) <= 1e-8 * abs(dj_tlm), (d, dj_adj, dj_tlm)
        assert abs(dj_adj - dj_fd) <= 1e-6 * abs(dj_fd), (d, dj_adj, dj_fd)
    s.close()
