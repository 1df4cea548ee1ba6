"""Precision form on inclined and curved elements, with and without the
artificial viscosity of diffusion YES.

The general-geometry stage kernels carry the full metric Jinv cV per node and
the weighted normal per face node (viscous runs: a gradient kernel with the
full metric, and the viscous fluxes along the metric columns and the face
normals); they are checked against the plain FP64 form on

  * the srtb-curved example's arcs, the cosine hill and the wall-graded block
    (2D, N = 4, golden fixtures of the euler binary's meshes);
  * blocks rotated by 30 degrees about z through the host driver: the 2D
    c1_2d case (N = 4), a 3D 4 x 3 x 2 block at N = 3 and a 3D 2 x 2 x 2 block
    at N = 7;
  * the 16^3, N = 4 bubble box tilted by 30 degrees about y, so that gravity
    is inclined to every element (100 steps).

Gates (the precision form's stated tolerances): tendency relative L2 per
variable <= 1e-5 at a perturbed developed state; state after 50 SSP-RK3 steps
<= 1e-5 per conserved variable and in theta'; mass drift <= 1e-12 relative;
the hydrostatic rest state on the hill stays exactly at rest.  Each mesh
inviscid and with viscosity 1.5 (the srtb examples' value).  The precision
form's adjoint on such elements: tests/test_mixed_adjoint.py.
"""
import json

import numpy as np
import pytest

from conftest import VARS, load_golden, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
FIXTURES = ["seg_srtb_curved", "seg_hill", "seg_graded"]
ROTATED = {"c1_2d": 0.005, "g3_4n3": 0.01, "g3_2n7": 0.01}


VISC = [0.0, 1.5]


def fixture_mesh(name):
    g = load_golden(name)
    return g, (g["fld0_rho"], g["fld0_U"], g["fld0_T"]), float(g["dt"])


def rotated_mesh(tmp_path, case):
    from driver_util import dump_case, make_case, rotate_case_z
    dt = ROTATED[case]
    d = make_case(tmp_path, case, dt=dt, steps=1, viscosity=0.0)
    rotate_case_z(d, 30.0)
    a = dump_case(d)
    return a, (a["fld_rho"], a["fld_U"], a["fld_T"]), dt


def solver(mesh, fields, dt, visc=0.0):
    import nebulasem_gb300 as ng
    s = ng.Solver(mesh, dt=dt, viscosity=visc)
    s.set_fields(*fields)
    return s, s.get_state()


def metric_is_general(mesh):
    J = np.asarray(mesh["Jinv"]).reshape(-1, 9)
    return np.abs(J[:, 3:]).max() > 1e-6 * np.abs(J[:, :3]).max()


def check_tendency(s, u0, tag, two_d=False):
    """At the state 10 steps on, perturbed node by node (a developed bubble
    flow is nearly divergence-free: its mass tendency is a residual of much
    larger terms and no test of relative accuracy; the perturbed state has
    O(1) divergence, as the golden fixtures' perturbed states)."""
    import nebulasem_gb300 as ng
    s.set_state(u0)
    s.step(10, prec=ng.FP64)
    u = s.get_state()
    rng = np.random.default_rng(3)
    n = len(u[0])
    for v, sc in enumerate((1e-3, 1e-1, 1e-1, 1e-1, 1e-1)):
        if not (two_d and v == 2):
            u[v] = u[v] + sc * rng.standard_normal(n)
    s.set_state(u)
    L64 = s.tendency(prec=ng.FP64)
    L32 = s.tendency(prec=ng.MIXED)
    top = max(np.linalg.norm(x) for x in L64)
    for a, b, v in zip(L32, L64, VARS):
        if np.linalg.norm(b) < 1e-8 * top:
            continue
        assert rel_l2(a, b) <= TOL, f"{tag} {v}: {rel_l2(a, b):.3e}"


def check_trajectory(s, u0, tag, steps=50):
    import nebulasem_gb300 as ng
    out = {}
    for prec, name in ((ng.FP64, "fp64"), (ng.MIXED, "mixed")):
        s.set_state(u0)
        d0 = s.diagnostics()
        s.step(steps, prec=prec)
        out[name] = s.get_state()
        d1 = s.diagnostics()
        drift = (d1[0] - d0[0]) / d0[0]
        assert abs(drift) <= 1e-12, f"{tag} {name} mass drift {drift:.3e}"
    ref, got = out["fp64"], out["mixed"]
    scale = max(np.linalg.norm(x) for x in ref[1:4])
    assert scale > 0
    # the measured figures (shown with pytest -s)
    l2 = {v: rel_l2(a, b) for a, b, v in zip(got, ref, VARS)}
    l2["theta'"] = rel_l2(got[4] / got[0] - 300.0, ref[4] / ref[0] - 300.0)
    print(json.dumps({"case": tag, "steps": steps, "l2_vs_fp64": l2}))
    for a, b, v in zip(got, ref, VARS):
        assert np.isfinite(a).all(), (tag, v)
        if np.linalg.norm(b) < 1e-10 * scale:
            assert np.linalg.norm(a - b) <= 1e-10 * scale, (tag, v)
            continue
        assert rel_l2(a, b) <= TOL, f"{tag} {v}: {rel_l2(a, b):.3e}"
    err = rel_l2(got[4] / got[0] - 300.0, ref[4] / ref[0] - 300.0)
    assert err <= TOL, f"{tag} theta': {err:.3e}"


@pytest.mark.parametrize("visc", VISC)
@pytest.mark.parametrize("name", FIXTURES)
def test_general_geometry_fixture(name, visc):
    mesh, fields, dt = fixture_mesh(name)
    if name != "seg_graded":
        assert metric_is_general(mesh)
    s, u0 = solver(mesh, fields, dt, visc)
    tag = f"{name} nu={visc}"
    check_tendency(s, u0, tag, two_d=True)
    check_trajectory(s, u0, tag)
    s.close()


@pytest.mark.parametrize("visc", VISC)
@pytest.mark.parametrize("case", sorted(ROTATED))
def test_general_geometry_rotated(tmp_path, case, visc):
    mesh, fields, dt = rotated_mesh(tmp_path, case)
    assert metric_is_general(mesh)
    s, u0 = solver(mesh, fields, dt, visc)
    tag = f"{case} rotated nu={visc}"
    check_tendency(s, u0, tag, two_d=int(mesh["meta"][1]) == 1)
    check_trajectory(s, u0, tag)
    s.close()


@pytest.mark.parametrize("visc", VISC)
def test_general_geometry_tilted_bubble_16cubed(visc):
    """The 16^3, N = 4 bubble in the box tilted by 30 degrees about y (every
    element inclined to gravity), 100 steps of dt 0.01 s (40 of dt 0.005 s
    with viscosity)."""
    from nebulasem_gb300.mesh import workload
    import nebulasem_gb300 as ng
    m, u0 = workload("bubble3d_16_n4_tilt30")
    assert metric_is_general(m)
    dt, steps = (0.01, 100) if visc == 0.0 else (0.005, 40)
    s = ng.Solver(m, dt=dt, viscosity=visc)
    check_trajectory(s, u0, f"bubble3d_16_n4_tilt30 nu={visc}", steps=steps)
    s.close()


def test_general_geometry_rest_state_is_exact():
    """Hydrostatic rest over the hill: the perturbation form keeps it exactly."""
    import nebulasem_gb300 as ng
    g = load_golden("seg_hill")
    n = int(g["meta"][7])
    s = ng.Solver(g, dt=float(g["dt"]), viscosity=0.0)
    s.set_fields(np.asarray(g["rho_ref"])[:n], np.zeros((n, 3)), np.zeros(n))
    u = s.get_state()
    L = s.tendency(prec=ng.MIXED)
    for a in L:
        assert np.abs(a).max() == 0.0
    s.step(10, prec=ng.MIXED)
    got = s.get_state()
    for a, b in zip(got, u):
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max())
    s.close()

