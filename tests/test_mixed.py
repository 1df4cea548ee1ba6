"""Precision form (FP32 bulk, FP64 background/RK/sums) against the plain form.

Gates (the precision form's stated tolerances): tendency relative L2 per
variable <= 1e-5 against the FP64 form; state after SSP-RK3 steps <= 1e-5;
a resting hydrostatic atmosphere stays exactly at rest; mass is conserved to
round-off.
"""
import numpy as np
import pytest

from conftest import VARS, golden_state, load_golden, rel_l2

pytestmark = pytest.mark.gpu

CASES = ["c1_2d", "g3_2", "g3_4n3", "g3_2n7"]


def make(g, dt=None):
    import nebulasem_gb300 as ng
    return ng.Solver(g, dt=float(g["dt"]) if dt is None else dt)


@pytest.mark.parametrize("case", CASES)
def test_mixed_tendency_vs_fp64(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    s = make(g)
    u = golden_state(g, "up")
    s.set_state(u)
    L64 = s.tendency(prec=ng.FP64)
    L32 = s.tendency(prec=ng.MIXED)
    for a, b, v in zip(L32, L64, VARS):
        if np.linalg.norm(b) < 1e-8 * max(np.linalg.norm(x) for x in L64):
            continue
        assert rel_l2(a, b) <= 1e-5, f"{case} {v}: {rel_l2(a, b):.3e}"
    s.close()


@pytest.mark.parametrize("case", CASES)
def test_mixed_trajectory_vs_fp64(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    u0 = golden_state(g, "u0" if str(g["start"]) == "rest" else "up")
    steps = int(g["steps"][-1])
    s = make(g)
    s.set_state(u0)
    s.step(steps, prec=ng.FP64)
    ref = s.get_state()
    s.set_state(u0)
    s.step(steps, prec=ng.MIXED)
    got = s.get_state()
    scale = max(np.linalg.norm(x) for x in ref[1:4])
    for a, b, v in zip(got, ref, VARS):
        if np.linalg.norm(b) < 1e-10 * scale:
            # a variable that is identically zero up to FP64 round-off (v in 2D)
            assert np.linalg.norm(a - b) <= 1e-10 * scale, v
            continue
        assert rel_l2(a, b) <= 1e-5, f"{case} {v}: {rel_l2(a, b):.3e}"
    s.close()


def test_mixed_rest_state_is_exact():
    """No bubble: the perturbation form keeps the hydrostatic rest state exactly."""
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import box_mesh, bubble_state
    m = box_mesh((3, 3, 3), 4, (2000.0,) * 3)
    u, p_ref, rho_ref, gh = bubble_state(m, 0.0, (1000.0,) * 3, (400.0,) * 3)
    m["p_ref"], m["rho_ref"] = p_ref, rho_ref
    s = ng.Solver(m, dt=0.0075)
    s.set_state(u)
    L = s.tendency(prec=ng.MIXED)
    for a in L:
        assert np.abs(a).max() == 0.0
    s.step(10, prec=ng.MIXED)
    got = s.get_state()
    for a, b in zip(got, u):
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max())
    s.close()


def test_mixed_mass_conservation_and_state_switching():
    """Mass drift of the precision form over 40 steps and switching between
    forms mid-run (the state moves between representations on demand)."""
    import nebulasem_gb300 as ng
    from nebulasem_gb300.mesh import workload
    m, u = workload("bubble3d_8_n4")
    s = ng.Solver(m, dt=0.0075)
    s.set_state(u)
    m0 = s.diagnostics()
    s.step(20, prec=ng.MIXED)
    s.step(1, prec=ng.FP64)
    s.step(19, prec=ng.MIXED)
    m1 = s.diagnostics()
    assert abs(m1[0] - m0[0]) / m0[0] < 1e-10, (m0, m1)
    assert abs(m1[2] - m0[2]) == 0.0
    s.close()


def test_mixed_order7_line_sum_paths(monkeypatch):
    """Order 7: line sums on the FP32 pipes (the default) and on the tensor
    cores (NSEM_MIXED_LINES=tensor: three TF32 products per term) both stay
    within 1e-5 of the FP64 form and agree with each other to FP32 rounding."""
    import nebulasem_gb300 as ng
    g = load_golden("g3_2n7")
    u = golden_state(g, "up")
    got = {}
    for lines in ("fp32", "tensor"):
        monkeypatch.setenv("NSEM_MIXED_LINES", lines)
        s = make(g)
        s.set_state(u)
        L64 = s.tendency(prec=ng.FP64)
        got[lines] = s.tendency(prec=ng.MIXED)
        s.step(5, prec=ng.MIXED)
        got[lines + "_traj"] = s.get_state()
        s.close()
        for a, b, v in zip(got[lines], L64, VARS):
            if np.linalg.norm(b) < 1e-8 * max(np.linalg.norm(x) for x in L64):
                continue
            assert rel_l2(a, b) <= 1e-5, (lines, v, rel_l2(a, b))
    for a, b, v in zip(got["tensor"], got["fp32"], VARS):
        assert rel_l2(a, b) <= 1e-6, (v, rel_l2(a, b))
    for a, b, v in zip(got["tensor_traj"], got["fp32_traj"], VARS):
        assert rel_l2(a, b) <= 1e-6, (v, rel_l2(a, b))
