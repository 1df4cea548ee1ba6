"""Tangent-linear and adjoint forms of the plain FP64 form on adaptively
refined meshes (2:1 non-conforming faces; the reference refines with its
`prepare -refine`), inviscid and with the artificial viscosity of diffusion YES.

On a mortar face the coarse side enters the flux through quantities
interpolated from the coarse face's nodes and lifts the projected fluxes; the
tangent interpolates the quantities' tangents and projects the flux tangents,
the adjoint gathers the projections' transposes and scatters the
interpolation's transpose back onto the coarse nodes.  With the viscosity the
quantities carry - mu grad U, - (mu / Pr) grad theta, and the gradients have
mortar face terms of their own (the coarse side interpolated into cds, the
projection back onto the coarse side), whose tangents are the same linear maps
of the tangents and whose transposes gather and scatter back.  Checked on the
refined fixtures (2D, 64 mortar faces, straight and curved; 3D N = 3 with
2 x 2 mortars), each inviscid and with viscosity 1.5 (the srtb examples'
value), at a state with a developed velocity field:

  * tangent against central differences of the GPU tendency: <= 1e-6 relative
    (with the viscosity along directions relative to the state, see direction());
  * duality of the single-tendency products: <w, J dv> = <J^T w, dv> to 1e-10
    of sum |w . J dv|;
  * duality over 10 SSP-RK3 steps (tangent-linear run against the
    checkpointed reverse sweep): <lam_N, dv_N> = <lam_0, dv_0> to 1e-10.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")
CASES = [(c, nu) for c in ("amr_g3_4n3", "amr_c1_2d_visc", "amr_hill_2d_visc") for nu in (0.0, 1.5)]


def dot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


def solver_at_developed_state(case, nu):
    """Solver on the fixture's refined mesh with viscosity nu, advanced 5 steps
    from the fixture's initial state so that the velocity field is not zero."""
    import nebulasem_gb300 as ng
    g = load_golden(case)
    s = ng.Solver(g, dt=float(g["dt"]), viscosity=nu)
    s.set_state([g[f"u0_{v}"] for v in VARS])
    s.step(5)
    u = s.get_state()
    return s, u, g


def direction(u, seed, two_d, nu=0.0):
    """A random direction.  With the viscosity it is relative to the state
    (each variable scaled by its own value): the SYMMETRY ghost velocity of the
    gradients is the tangential velocity rescaled to |U|, whose derivative grows
    as 1 / |U_t|^2 where the tangential wall velocity is small, so an additive
    perturbation leaves the range in which a central difference is linear
    there (on conforming meshes too: the dual-number oracle and the GPU
    tangent agree to 1e-16 and both differ from such differences by 1e-4)."""
    rng = np.random.default_rng(seed)
    n = len(u[0])
    if nu:
        du = [a * rng.standard_normal(n) * 1e-2 for a in u]
    else:
        du = [rng.standard_normal(n) * sc for sc in (1e-3, 1e-1, 1e-1, 1e-1, 1e-1)]
    if two_d:
        du[2][:] = 0.0
    return du


@pytest.mark.parametrize("case,nu", CASES)
def test_amr_jvp_vs_central_differences(case, nu):
    s, u, g = solver_at_developed_state(case, nu)
    two_d = int(g["meta"][1]) == 1
    assert np.abs(u[1]).max() > 0
    du = direction(u, 3, two_d, nu)
    eps = 1e-5
    s.set_state(u)
    Ld = s.jvp(du)
    Ls = []
    for sg in (1.0, -1.0):
        s.set_state([a + sg * eps * b for a, b in zip(u, du)])
        Ls.append(s.tendency())
    for v, (a, lp, lm) in enumerate(zip(Ld, *Ls)):
        fd = (lp - lm) / (2 * eps)
        nf = np.linalg.norm(fd)
        if nf == 0:
            assert np.linalg.norm(a) == 0
            continue
        assert np.linalg.norm(a - fd) <= 1e-6 * nf, (case, nu, VARS[v], np.linalg.norm(a - fd) / nf)
    s.close()


@pytest.mark.parametrize("case,nu", CASES)
def test_amr_vjp_duality(case, nu):
    s, u, g = solver_at_developed_state(case, nu)
    two_d = int(g["meta"][1]) == 1
    rng = np.random.default_rng(7)
    n = len(u[0])
    for trial in range(2):
        du = direction(u, 11 + trial, two_d, nu)
        w = [rng.standard_normal(n) for _ in range(5)]
        s.set_state(u)
        Ld = s.jvp(du)
        gv = s.vjp(w)
        lhs, rhs = dot(w, Ld), dot(gv, du)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= 1e-10 * scale, (case, nu, trial, lhs, rhs, scale)
    s.close()


@pytest.mark.parametrize("case,nu", CASES)
def test_amr_tlm_adjoint_duality(case, nu):
    s, u, g = solver_at_developed_state(case, nu)
    two_d = int(g["meta"][1]) == 1
    n = len(u[0])
    du0 = direction(u, 5, two_d, nu)
    lamN = [np.random.default_rng(9 + v).standard_normal(n) for v in range(5)]
    if two_d:
        lamN[2][:] = 0.0
    steps = 10
    s.set_state(u)
    duN, _ = s.tlm(steps, du0)
    s.set_state(u)
    s.forward_checkpointed(steps, 4)
    lam0, _ = s.adjoint(lamN)
    lhs, rhs = dot(lamN, duN), dot(lam0, du0)
    scale = sum(np.abs(x * y).sum() for x, y in zip(lamN, duN))
    assert abs(lhs - rhs) <= 1e-10 * scale, (case, nu, lhs, rhs, scale)
    s.close()

