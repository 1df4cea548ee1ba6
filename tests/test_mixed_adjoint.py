"""Discrete adjoint of the precision form (FP32 bulk, FP64 adjoint state).

  * transpose test: <w, J(u) du> from the CPU FP64 tangent-linear oracle
    against <J32(u)^T w, du> from the precision form's vector-Jacobian
    product (FP32 at the FP32 shadow of u): agreement to 1e-5 of
    sum |w . J du|, inviscid and with the artificial viscosity (the viscous
    fluxes' transposes and the gradients' transpose);
  * gradient of J = 1/2 sum_box theta'^2 at the final time with respect to the
    initial state, precision-form forward and reverse sweep against the plain
    FP64 adjoint (itself checked against the tangent-linear model and finite
    differences): relative L2 <= 1e-5 of dJ/dtheta'_0, on golden fixtures
    (inviscid and viscous) and on the 48^3, N = 4 bubble (100 steps of dt
    0.005 s, checkpoints every 10 steps); the rising-bubble box x in
    [800, 1200], z in [800, 1200] m;
  * inclined and curved elements: the transpose test on the curved 2D
    fixtures (hill, srtb-curved) and the gradient on the 16^3 bubble box
    tilted by 30 degrees, inviscid and viscous.
"""
import numpy as np
import pytest

import oracle
from conftest import golden_state, load_golden, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def dot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


@pytest.mark.parametrize("case", ["g3_2", "g3_4n3", "c1_2d", "g3_2n7", "g3_2_visc", "c1_2d_visc"])
def test_mixed_vjp_transpose(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    u = golden_state(g, "up")
    s = ng.Solver(g, dt=float(g["dt"]))
    s.set_state(u)
    m = oracle.OracleMesh(g)
    rng = np.random.default_rng(5)
    n = m.n_int
    for trial in range(2):
        du = [rng.standard_normal(n) * sc for sc in (1e-3, 1e-1, 1e-1, 1e-1, 1e-1)]
        if case.startswith("c1_2d"):
            du[2][:] = 0.0
        w = [rng.standard_normal(n) for _ in range(5)]
        _, Ld = m.jvp(u, du)
        lhs = dot(w, Ld)
        gv = s.vjp(w, prec=ng.MIXED)
        rhs = dot(gv, du)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= TOL * scale, (case, trial, lhs, rhs, scale)
    s.close()


def _gradients(mesh, u_init, dt, steps, every, box):
    import nebulasem_gb300 as ng
    from nebulasem_gb300 import objective as ob
    n = int(mesh["meta"][7])
    xyz = np.asarray(mesh["cC"]).reshape(-1, 3)[:n]
    p_ref = np.asarray(mesh["p_ref"])[:n]
    th0 = u_init[4] / u_init[0] - 300.0
    u0 = ob.state_from_theta(th0, p_ref)
    mask = ob.box_mask(xyz, box)
    s = ng.Solver(mesh, dt=dt)
    out = {}
    for prec, tag in ((ng.FP64, "fp64"), (ng.MIXED, "mixed")):
        s.set_state(u0)
        ms_f = s.forward_checkpointed(steps, every, prec=prec)
        uN = s.get_state()
        lam0, ms_a = s.adjoint(ob.objective_grad(uN, mask))
        out[tag] = ob.theta_grad(lam0, u0, th0)
        out[tag + "_J"] = ob.objective(uN, mask)
        out[tag + "_ms"] = (ms_f, ms_a)
        # the reverse sweep leaves the final state in place
        again = s.get_state()
        assert all(np.allclose(a, b, rtol=1e-14, atol=0) for a, b in zip(again, uN)), tag
    s.close()
    return out


@pytest.mark.parametrize("case", ["g3_2", "g3_2_visc"])
def test_mixed_adjoint_gradient_fixture(case):
    g = load_golden(case)
    out = _gradients(g, golden_state(g, "u0"), 0.01, 20, 5, (800.0, 1200.0, 400.0, 1000.0))
    assert out["fp64_J"] > 0
    assert rel_l2(out["mixed"], out["fp64"]) <= TOL, (case, rel_l2(out["mixed"], out["fp64"]))


def test_mixed_adjoint_gradient_48cubed():
    from nebulasem_gb300.mesh import workload
    m, u = workload("bubble3d_48_n4")
    out = _gradients(m, u, 0.005, 100, 10, (800.0, 1200.0, 800.0, 1200.0))
    assert out["fp64_J"] > 1.0
    err = rel_l2(out["mixed"], out["fp64"])
    assert err <= TOL, err


GENERAL = [("seg_hill", 0.0), ("seg_hill", 1.5), ("seg_srtb_curved", 0.0), ("seg_srtb_curved", 1.5)]


@pytest.mark.parametrize("case,nu", GENERAL)
def test_mixed_vjp_transpose_general_geometry(case, nu):
    """Curved elements (the cosine hill, the srtb-curved arcs: per-node metric
    and face normals), inviscid and viscous, at a state 5 steps into the run."""
    import nebulasem_gb300 as ng
    g = dict(load_golden(case))
    g["viscosity"] = nu
    s = ng.Solver(g, dt=float(g["dt"]))
    s.set_fields(g["fld0_rho"], g["fld0_U"], g["fld0_T"])
    s.step(5)
    u = s.get_state()
    m = oracle.OracleMesh(g)
    rng = np.random.default_rng(7)
    n = m.n_int
    for trial in range(2):
        du = [rng.standard_normal(n) * sc for sc in (1e-3, 1e-1, 1e-1, 1e-1, 1e-1)]
        du[2][:] = 0.0
        w = [rng.standard_normal(n) for _ in range(5)]
        _, Ld = m.jvp(u, du)
        lhs = dot(w, Ld)
        s.set_state(u)
        gv = s.vjp(w, prec=ng.MIXED)
        rhs = dot(gv, du)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= TOL * scale, (case, nu, trial, lhs, rhs, scale)
    s.close()


@pytest.mark.parametrize("nu", [0.0, 1.5])
def test_mixed_adjoint_gradient_tilted_16cubed(nu):
    """The 16^3, N = 4 bubble in the box tilted by 30 degrees (every element
    inclined), 20 steps, checkpoints every 5: the precision form's gradient
    against the FP64 adjoint's."""
    from nebulasem_gb300.mesh import workload
    m, u = workload("bubble3d_16_n4_tilt30")
    m = dict(m)
    m["viscosity"] = nu
    out = _gradients(m, u, 0.005 if nu else 0.01, 20, 5, (800.0, 1200.0, 800.0, 1200.0))
    assert out["fp64_J"] > 0
    err = rel_l2(out["mixed"], out["fp64"])
    assert err <= TOL, (nu, err)
