"""Precision form on adaptively refined meshes (2:1 mortar faces; the
reference refines with its `prepare -refine`), with and without the
artificial viscosity of diffusion YES.

Per stage, mortar kernels interpolate the coarse side's face quantities onto
each mortar slot with psiRef (the fine side reads its own node), form the
Rusanov flux vectors there, project them back onto the coarse face's nodes
with psiCor, and hand both sides' outward values to the stage kernel -- the
plain form's mortar treatment (field.h:2019-2248) in FP32 on the perturbation
state; viscous runs give the gradients' face values the same treatment (the
coarse side's U and theta interpolated into the face averages, which are
projected back onto the coarse nodes) and carry -mu grad U, -(mu/Pr) grad theta
in the interpolated flux tensors.  Checked against the plain FP64 form (itself bit for bit the oracle and
the reference's operators on these meshes, tests/test_amr_gpu.py) on the
refined fixtures (2D N = 4, 64 mortar faces; 3D N = 3, 48 faces of 2 x 2
mortars):

  * tendency at a perturbed developed state: relative L2 per variable <= 1e-5;
  * 40 SSP-RK3 steps from the fixture's state: relative L2 per conserved
    variable and in theta' <= 1e-5, mass drift <= 1e-12 relative;
  * each mesh inviscid and with viscosity 1.5 (the 2D fixture's value);
  * the precision form's adjoint, inviscid and viscous: the transposed stage
    with the transposes of the mortar kernels (and of the gradients' mortar
    face values), <w, J du> from the plain FP64 tangent (tests/test_amr_tangent.py
    checks it against central differences and its own adjoint) against
    <J32^T w, du> to 1e-5 of sum |w . J du|; the gradient of
    1/2 sum_box theta'^2 after 20 steps (checkpoints every 5) from the
    precision-form forward and reverse sweep against the FP64 adjoint's,
    relative L2 <= 1e-5.
"""
import json

import numpy as np
import pytest

from conftest import VARS, load_golden, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
CASES = ["amr_g3_4n3", "amr_c1_2d_visc", "amr_hill_2d_visc"]
VISC = [0.0, 1.5]


def solver(case, visc=0.0):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    s = ng.Solver(g, dt=float(g["dt"]), viscosity=visc)
    u0 = [g[f"u0_{v}"] for v in VARS]
    return s, u0, g


@pytest.mark.parametrize("visc", VISC)
@pytest.mark.parametrize("case", CASES)
def test_mortar_tendency_vs_fp64(case, visc):
    import nebulasem_gb300 as ng
    s, u0, g = solver(case, visc)
    s.set_state(u0)
    s.step(5, prec=ng.FP64)
    u = s.get_state()
    rng = np.random.default_rng(3)
    n = len(u[0])
    for v, sc in enumerate((1e-3, 1e-1, 1e-1, 1e-1, 1e-1)):
        u[v] = u[v] + sc * rng.standard_normal(n)
    s.set_state(u)
    L64 = s.tendency(prec=ng.FP64)
    L32 = s.tendency(prec=ng.MIXED)
    top = max(np.linalg.norm(x) for x in L64)
    for a, b, v in zip(L32, L64, VARS):
        if np.linalg.norm(b) < 1e-8 * top:
            continue
        assert rel_l2(a, b) <= TOL, f"{case} nu={visc} {v}: {rel_l2(a, b):.3e}"
    s.close()


@pytest.mark.parametrize("visc", VISC)
@pytest.mark.parametrize("case", CASES)
def test_mortar_trajectory_vs_fp64(case, visc):
    import nebulasem_gb300 as ng
    s, u0, g = solver(case, visc)
    steps = 40
    out = {}
    for prec, name in ((ng.FP64, "fp64"), (ng.MIXED, "mixed")):
        s.set_state(u0)
        d0 = s.diagnostics()
        s.step(steps, prec=prec)
        out[name] = s.get_state()
        d1 = s.diagnostics()
        out[name + "_drift"] = (d1[0] - d0[0]) / d0[0]
    s.close()
    ref, got = out["fp64"], out["mixed"]
    l2 = {v: rel_l2(a, b) for a, b, v in zip(got, ref, VARS)}
    l2["theta'"] = rel_l2(got[4] / got[0] - 300.0, ref[4] / ref[0] - 300.0)
    # the measured figures (shown with pytest -s)
    print(json.dumps({"case": case, "viscosity": visc, "steps": steps, "l2_vs_fp64": l2,
                      "mass_drift": {t: out[t + "_drift"] for t in ("mixed", "fp64")}}))
    scale = max(np.linalg.norm(x) for x in ref[1:4])
    assert scale > 0
    for a, b, v in zip(got, ref, VARS):
        assert np.isfinite(a).all(), v
        if np.linalg.norm(b) < 1e-10 * scale:
            assert np.linalg.norm(a - b) <= 1e-10 * scale, v
            continue
        assert l2[v] <= TOL, f"{case} nu={visc} {v}: {l2[v]:.3e}"
    assert l2["theta'"] <= TOL
    for t in ("mixed", "fp64"):
        assert abs(out[t + "_drift"]) <= 1e-12, (t, out[t + "_drift"])


def dot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


@pytest.mark.parametrize("visc", VISC)
@pytest.mark.parametrize("case", CASES)
def test_mortar_vjp_transpose(case, visc):
    import nebulasem_gb300 as ng
    s, u0, g = solver(case, visc)
    s.set_state(u0)
    s.step(5, prec=ng.FP64)
    u = s.get_state()
    two_d = int(g["meta"][1]) == 1
    rng = np.random.default_rng(9)
    n = len(u[0])
    for trial in range(2):
        du = [rng.standard_normal(n) * sc for sc in (1e-3, 1e-1, 1e-1, 1e-1, 1e-1)]
        if two_d:
            du[2][:] = 0.0
        w = [rng.standard_normal(n) for _ in range(5)]
        s.set_state(u)
        Ld = s.jvp(du)
        gv = s.vjp(w, prec=ng.MIXED)
        lhs, rhs = dot(w, Ld), dot(gv, du)
        scale = sum(np.abs(x * y).sum() for x, y in zip(w, Ld))
        assert abs(lhs - rhs) <= TOL * scale, (case, visc, trial, lhs, rhs, scale)
    s.close()


@pytest.mark.parametrize("visc", VISC)
@pytest.mark.parametrize("case", CASES)
def test_mortar_adjoint_gradient(case, visc):
    import nebulasem_gb300 as ng
    from nebulasem_gb300 import objective as ob
    s, u_fix, g = solver(case, visc)
    n = len(u_fix[0])
    xyz = np.asarray(g["cC"]).reshape(-1, 3)[:n]
    p_ref = np.asarray(g["p_ref"])[:n]
    th0 = u_fix[4] / u_fix[0] - 300.0
    u0 = ob.state_from_theta(th0, p_ref)
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    mid, half = (lo + hi) / 2, (hi - lo) / 4
    box = (mid[0] - half[0], mid[0] + half[0], mid[2] - half[2], mid[2] + half[2])
    mask = ob.box_mask(xyz, box)
    assert mask.any()
    out = {}
    for prec, tag in ((ng.FP64, "fp64"), (ng.MIXED, "mixed")):
        s.set_state(u0)
        s.forward_checkpointed(20, 5, prec=prec)
        uN = s.get_state()
        lam0, _ = s.adjoint(ob.objective_grad(uN, mask))
        out[tag] = lam0
        out[tag + "_th"] = ob.theta_grad(lam0, u0, th0)
        out[tag + "_J"] = ob.objective(uN, mask)
    s.close()
    assert out["fp64_J"] > 0
    err_th = rel_l2(out["mixed_th"], out["fp64_th"])
    err_all = rel_l2(np.concatenate(out["mixed"]), np.concatenate(out["fp64"]))
    print(case, visc, "dJ/dtheta'", err_th, "dJ/du", err_all)
    assert err_th <= TOL, (case, visc, err_th)
    assert err_all <= TOL, (case, visc, err_all)
