"""Gradient check of the discrete adjoint on the 16^3, N = 4 rising bubble.

Workload: 2000^3 m box, 16^3 elements, N = 4 (512,000 nodes, 2.56 M DOF),
theta' = 0.5 K cosine bubble, plain FP64 form, 200 SSP-RK3 steps of
dt = 0.01 s, RK checkpoints every 20 steps.  Objective
J = 1/2 sum theta'^2 over the nodes of a box at the final time; control: the
initial theta' field; 8 Gaussian directions (seeds 0..7).

The box x in [800, 1200], z in [1200, 1600] m lies above the bubble, which
rises by less than a metre in the 2 s simulated: theta' there stays at
round-off (J ~ 1e-21) and no finite difference of it means anything.  The
check therefore uses the box 400 m lower, z in [800, 1200] m, over the upper
half of the bubble (J ~ 4.7).

Gates, per direction v:
  * the adjoint's directional derivative <dJ/dtheta'_0, v> against the GPU
    tangent-linear model of the same trajectory: <= 1e-10 relative;
  * against central differences of the GPU forward at eps = 1e-6: the
    difference is at most 1e-6 of |dJ/dtheta'_0| |v| (the directional
    derivative's natural scale; relative to the derivative itself, round-off
    of about 1e-12 in J divided by 2 eps dominates for directions whose
    derivative is small);
  * against central differences at eps = 1e-4: <= 1e-6 relative to the
    derivative itself.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WORKLOAD = "bubble3d_16_n4"
DT, STEPS, CKPT, NDIR = 0.01, 200, 20, 8
BOX = (800.0, 1200.0, 800.0, 1200.0)


def test_adjoint_gradient_16cubed_200_steps():
    import nebulasem_gb300 as ng
    from nebulasem_gb300 import objective as ob
    from nebulasem_gb300.mesh import workload

    m, u = workload(WORKLOAD)
    n = int(m["meta"][7])
    xyz = np.asarray(m["cC"]).reshape(-1, 3)[:n]
    p_ref = np.asarray(m["p_ref"])[:n]
    th0 = u[4] / u[0] - 300.0
    u0 = ob.state_from_theta(th0, p_ref)
    mask = ob.box_mask(xyz, BOX)

    s = ng.Solver(m, dt=DT)
    s.set_state(u0)
    s.forward_checkpointed(STEPS, CKPT)
    uN = s.get_state()
    J = ob.objective(uN, mask)
    assert J > 1.0
    lam0, _ = s.adjoint(ob.objective_grad(uN, mask))
    grad = ob.theta_grad(lam0, u0, th0)
    gnorm = float(np.linalg.norm(grad))
    rows = []
    for seed in range(NDIR):
        v = np.random.default_rng(seed).standard_normal(n)
        dj_adj = float(np.dot(grad, v))
        # tangent-linear model of the same FP64 trajectory
        s.set_state(u0)
        du0 = [-u0[0] / (th0 + 300.0) * v] + [np.zeros(n) for _ in range(4)]
        duN, _ = s.tlm(STEPS, du0)
        uT = s.get_state()
        dj_tlm = float(sum(np.dot(a, b) for a, b in zip(ob.objective_grad(uT, mask), duN)))
        fd = {}
        for eps in (1e-6, 1e-4):
            Js = []
            for sign in (1.0, -1.0):
                s.set_state(ob.state_from_theta(th0 + sign * eps * v, p_ref))
                s.step(STEPS)
                Js.append(ob.objective(s.get_state(), mask))
            fd[eps] = (Js[0] - Js[1]) / (2 * eps)
        rows.append((seed, dj_adj, dj_tlm, fd[1e-6], fd[1e-4]))
    s.close()
    scale = gnorm * np.sqrt(n)   # |grad| |v| for a standard normal v
    # the measured figures (shown with pytest -s)
    print(json.dumps({"J": J, "rows": [
        {"seed": sd, "adj": a, "adj_vs_tlm": abs(a - t) / abs(t), "adj_vs_fd6": abs(a - f6) / abs(f6),
         "adj_vs_fd4": abs(a - f4) / abs(f4)} for sd, a, t, f6, f4 in rows]}))
    for seed, adj, tlm, fd6, fd4 in rows:
        assert abs(adj - tlm) <= 1e-10 * abs(tlm), (seed, adj, tlm)
        assert abs(adj - fd6) <= 1e-6 * scale, (seed, adj, fd6, scale)
        assert abs(adj - fd4) <= 1e-6 * abs(fd4), (seed, adj, fd4)
