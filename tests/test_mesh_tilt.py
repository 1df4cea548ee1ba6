"""The tilted box workloads (inclined elements) against the untilted box.

Rotating the box, its gravity and its momentum by the same rotation R leaves
the discrete Euler operator invariant: on the tilted mesh (coordinates
R (x - c) + c, metric R diag(2/h), normals R fN) with gravity R g, the same
background arrays and the momentum rotated, the oracle's tendencies of rho and
rho theta equal the untilted ones and the momentum tendency is R times the
untilted one, to round-off (measured: 1.5e-9 relative L2 for rho and rho
theta, 9e-11 for the momentum).  This pins the tilted mesh arrays that the
precision form's general-geometry kernels are measured on.
"""
import numpy as np

import oracle
from conftest import rel_l2


def test_tilted_box_is_rotation_invariant():
    from nebulasem_gb300.mesh import box_mesh, bubble_state, rotation_y
    n, order, length = (3, 2, 3), 4, (2000.0, 1500.0, 2000.0)
    m = box_mesh(n, order, length)
    u, p_ref, rho_ref, _ = bubble_state(m, 0.5, (1000.0, 750.0, 600.0), (400.0,) * 3)
    m["p_ref"], m["rho_ref"] = p_ref, rho_ref
    om = oracle.OracleMesh(m)
    u = om.ssprk3(u, 0.01, 5)            # a state with a developed velocity field
    L = om.tendency(u)
    R = rotation_y(30.0)
    mt = box_mesh(n, order, length, tilt=30.0)
    mt["p_ref"], mt["rho_ref"] = p_ref, rho_ref
    mt["gravity"] = R @ np.array([0.0, 0.0, -9.81])
    ot = oracle.OracleMesh(mt)
    mom = np.stack(u[1:4], axis=1) @ R.T
    Lt = ot.tendency([u[0], mom[:, 0], mom[:, 1], mom[:, 2], u[4]])
    assert np.abs(np.stack(u[1:4])).max() > 0
    assert rel_l2(Lt[0], L[0]) < 1e-8
    assert rel_l2(Lt[4], L[4]) < 1e-8
    Lm = np.stack(L[1:4], axis=1) @ R.T
    Lmt = np.stack(Lt[1:4], axis=1)
    assert rel_l2(Lmt, Lm) < 1e-9
    # the tilted metric is full: off-diagonal entries of the order of the diagonal
    J = np.asarray(mt["Jinv"]).reshape(-1, 9)[: int(mt["meta"][7])]
    assert np.abs(J[:, 3:]).max() > 0.3 * np.abs(J[:, :3]).max()
