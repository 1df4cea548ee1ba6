"""Edge cases of the mesh: a single element (every face a SYMMETRY wall, no
neighbour at all), a single 2D element, and a one-element-thick 3D slab.

  * plain FP64 form: tendency and 10 SSP-RK3 steps bit for bit the oracle
    (correctly rounded pow);
  * precision form: 10 steps within 1e-5 relative L2 of the FP64 form (the
    velocity components that are zero to round-off in both are compared
    absolutely), mass conserved to 1e-12.
"""
import numpy as np
import pytest

import oracle
from conftest import VARS, rel_l2

pytestmark = pytest.mark.gpu

# (elements, order, lengths, dim)
MESHES = {
    "one_3d_n4": ((1, 1, 1), 4, (2000.0, 2000.0, 2000.0), 3),
    "one_2d_n4": ((1, 1, 1), 4, (1000.0, 100.0, 1000.0), 2),
    "slab_3d_n3": ((4, 1, 3), 3, (2000.0, 500.0, 1500.0), 3),
    "one_3d_n7": ((1, 1, 1), 7, (2000.0, 2000.0, 2000.0), 3),
}


def mesh_and_state(name):
    from nebulasem_gb300.mesh import box_mesh, bubble_state
    n, order, length, dim = MESHES[name]
    m = box_mesh(n, order, length, dim=dim)
    centre = (length[0] / 2, length[1] / 2, length[2] * 0.35)
    radius = (length[0] / 3, 1e4 if dim == 2 else length[1] / 3, length[2] / 3)
    u, p_ref, rho_ref, _ = bubble_state(m, 0.5, centre, radius)
    m["p_ref"], m["rho_ref"] = p_ref, rho_ref
    return m, u


@pytest.mark.parametrize("name", sorted(MESHES))
def test_edge_mesh_fp64_bitwise_and_precision(name):
    import nebulasem_gb300 as ng
    m, u0 = mesh_and_state(name)
    dt, steps = 0.01, 10
    om = oracle.OracleMesh(m)
    oracle.set_pow(1)
    try:
        L_o = om.tendency(u0)
        u_o = om.ssprk3(u0, dt, steps)
    finally:
        oracle.set_pow(0)
    s = ng.Solver(m, dt=dt)
    s.set_state(u0)
    for a, b, v in zip(s.tendency(), L_o, VARS):
        assert np.array_equal(a, b), (name, "tendency", v)
    s.step(steps)
    u64 = s.get_state()
    for a, b, v in zip(u64, u_o, VARS):
        assert np.array_equal(a, b), (name, "state", v)
    s.set_state(u0)
    d0 = s.diagnostics()
    s.step(steps, prec=ng.MIXED)
    u32 = s.get_state()
    d1 = s.diagnostics()
    assert abs((d1[0] - d0[0]) / d0[0]) <= 1e-12
    scale = max(np.linalg.norm(x) for x in u64[1:4])
    assert scale > 0
    for a, b, v in zip(u32, u64, VARS):
        if np.linalg.norm(b) < 1e-10 * scale:
            assert np.linalg.norm(a - b) <= 1e-10 * scale, (name, v)
            continue
        assert rel_l2(a, b) <= 1e-5, (name, v, rel_l2(a, b))
    s.close()
