"""The CPU tangent-linear oracle (oracle/nsem_tlm.cpp) against the plain
oracle, without and with artificial viscosity: its value part reproduces the
oracle bit for bit, several directions in one pass equal one pass per
direction, and its directional derivatives match central differences
(eps = 1e-6) of the oracle's SSP-RK3 along 8 seeded Gaussian directions."""
import numpy as np
import pytest

import oracle
from conftest import golden_state, load_golden


@pytest.fixture(scope="module", params=["g3_2", "g3_2_visc"])
def case(request):
    """inviscid, and with the artificial viscosity of diffusion YES"""
    g = load_golden(request.param)
    return oracle.OracleMesh(g), golden_state(g, "up")


def perturbation(rng, u):
    """Relative perturbation of every conserved variable.  A component that is
    zero stays zero: the SYMMETRY ghost velocity is discontinuous where the
    tangential velocity crosses |r| = 1e-7 (tensor.h:486-494 rescales it to
    |U|), so an additive perturbation of a wall node whose velocity is purely
    normal would put a jump inside the difference stencil."""
    return [a * rng.standard_normal(a.shape[0]) * 1e-2 for a in u]


def test_jvp_value_is_the_oracle(case):
    m, u = case
    du = perturbation(np.random.default_rng(1), u)
    for which in (0, 1):
        oracle.set_pow(which)
        L, _ = m.jvp(u, du)
        assert all(np.array_equal(a, b) for a, b in zip(L, m.tendency(u)))
    oracle.set_pow(0)


def test_multi_direction_pass_equals_single(case):
    m, u = case
    rng = np.random.default_rng(2)
    dus = [perturbation(rng, u) for _ in range(3)]
    uA, dA = m.tlm_ssprk3_multi(u, dus, 0.01, 3)
    assert all(np.array_equal(a, b) for a, b in zip(uA, m.ssprk3(u, 0.01, 3)))
    for d in range(3):
        _, dB = m.tlm_ssprk3(u, dus[d], 0.01, 3)
        assert all(np.array_equal(a, b) for a, b in zip(dA[d], dB))


def test_tlm_matches_central_differences(case):
    m, u = case
    dt, steps, eps = 0.01, 10, 1e-6
    dirs = [perturbation(np.random.default_rng(seed), u) for seed in range(8)]
    w = [np.random.default_rng(100).standard_normal(m.n_int) for _ in range(5)]
    _, duT = m.tlm_ssprk3_multi(u, dirs, dt, steps)
    for d, du in enumerate(dirs):
        up = m.ssprk3([a + eps * b for a, b in zip(u, du)], dt, steps)
        um = m.ssprk3([a - eps * b for a, b in zip(u, du)], dt, steps)
        fd = sum(float(np.dot(x, (p - q) / (2 * eps))) for x, p, q in zip(w, up, um))
        tl = sum(float(np.dot(x, y)) for x, y in zip(w, duT[d]))
        assert abs(fd - tl) <= 1e-6 * abs(tl), (d, fd, tl)
