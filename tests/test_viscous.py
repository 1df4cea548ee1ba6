"""Coupled SSP-RK3 FP64 form with the artificial viscosity of diffusion YES on
the GPU, bit for bit against the oracle (correctly rounded pow), which matches
the reference library's own chain bit for bit (tests/test_viscous_oracle.py)."""
import numpy as np
import pytest

import oracle
from conftest import VARS, golden_state, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["g3_2_visc", "c1_2d_visc"])
def test_viscous_fp64_bitwise_vs_oracle(case):
    import nebulasem_gb300 as ng
    g = load_golden(case)
    dt = float(g["dt"])
    m = oracle.OracleMesh(g)
    oracle.set_pow(1)
    s = ng.Solver(g, dt=dt)
    up = golden_state(g, "up")
    s.set_state(up)
    L = s.tendency()
    for a, b, v in zip(L, m.tendency(up), VARS):
        assert np.array_equal(a, b), (case, "tendency", v)
    start = golden_state(g, "up" if str(g["start"]) == "pert" else "u0")
    steps = int(g["steps"][-1])
    s.set_state(start)
    s.step(steps // 2)
    s.step(steps - steps // 2)
    got = s.get_state()
    want = m.ssprk3(start, dt, steps)
    oracle.set_pow(0)
    for a, b, v in zip(got, want, VARS):
        assert np.array_equal(a, b), (case, "trajectory", v)
    # forms without viscous terms refuse instead of silently dropping them
    with pytest.raises(ng.NsemError) as e:
        s.step(1, prec=ng.MIXED)
    assert e.value.status == 5
    with pytest.raises(ng.NsemError) as e:
        s.vjp([np.zeros(m.n_int)] * 5)
    assert e.value.status == 5
    s.close()
