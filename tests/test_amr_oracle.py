"""The oracle's segregated scheme on adaptively refined meshes (2:1
non-conforming faces) against the unmodified reference `euler` binary.

Fixtures (tests/golden/make_golden.py, AMR_PLAN): the mesh app's grid refined
once by the reference's `prepare -refine`, the harness's dump of that mesh with
its non-conforming faces (the coarse side, the coarse face and the halves the
mortar covers) and the 2:1 tables psiRef / psiCor, and the binary's fields
after the steps.  With the C library pow, as the binary, the oracle's mortar
restatement (scatter_non_conforming / gather_non_conforming,
src/field/field.h:2019-2248) reproduces them bit for bit; dropping it changes
theta' by 10-80 %."""
import numpy as np
import pytest

import oracle
from conftest import load_golden


@pytest.mark.parametrize("case", ["amr_c1_2d_visc", "amr_g3_4n3", "amr_hill_2d_visc"])
def test_amr_oracle_bitwise_vs_euler_binary(case):
    g = load_golden(case)
    n = int(g["meta"][7])
    dt, steps = float(g["dt"]), int(g["nsteps"])
    rho0, U0, T0 = g["fld0_rho"], g["fld0_U"].reshape(n, 3), g["fld0_T"]
    assert len(g["mortar"]) // 4 > 0
    m = oracle.OracleMesh(g)
    oracle.set_pow(0)
    rho, U, T = m.segregated(rho0, U0, T0, dt, steps)
    assert np.array_equal(rho, g["fldN_rho"])
    assert np.array_equal(np.asarray(U).reshape(-1), g["fldN_U"])
    assert np.array_equal(T, g["fldN_T"])
    # the same mesh treated as conforming is far off
    h = {k: v for k, v in g.items() if k != "mortar"}
    r2, U2, T2 = oracle.OracleMesh(h).segregated(rho0, U0, T0, dt, steps)
    assert np.linalg.norm(T2 - g["fldN_T"]) > 0.05 * np.linalg.norm(g["fldN_T"])


def test_amr_mesh_shape():
    """The 2D fixture: 40 of the 100 cells split in four (220 cells), 64 mortar
    faces, all with the coarse cell as the owner; halves in the refined plane
    only (the collapsed y direction keeps half 0)."""
    g = load_golden("amr_c1_2d_visc")
    meta = g["meta"]
    assert int(meta[5]) == 220 and int(meta[7]) == 5500
    mort = g["mortar"].reshape(-1, 4)
    assert mort.shape[0] == 64
    assert set(mort[:, 1]) == {2}
    fid, halves = mort[:, 2], mort[:, 3]
    assert np.all(halves[fid <= 1] <= 1)          # x, y faces: y half 0
    assert np.all((halves[fid >= 4] & 1) == 0)    # y, z faces: y half 0


VARS = ("rho", "rhou", "rhov", "rhow", "rhotheta")


@pytest.mark.parametrize("case", ["amr_c1_2d_visc", "amr_g3_4n3", "amr_hill_2d_visc"])
def test_amr_coupled_oracle_bitwise_vs_reference_operators(case):
    """The coupled form on the refined mesh: the oracle's tendency equals the
    reference's own operators (the harness) at the start state, and 5 SSP-RK3
    steps equal the harness's trajectory, bit for bit."""
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    oracle.set_pow(0)
    u0 = [g[f"u0_{v}"] for v in VARS]
    L = m.tendency(u0)
    for a, v in zip(L, VARS):
        assert np.array_equal(a, g[f"L0_{v}"]), v
    u = m.ssprk3(u0, float(g["dt"]), int(g["rk_steps"]))
    for a, v in zip(u, VARS):
        assert np.array_equal(a, g[f"rk_{v}"]), v
