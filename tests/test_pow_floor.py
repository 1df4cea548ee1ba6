"""The double-double pow is correctly rounded, and the parity floor it
implies against the reference (C library pow) is what the FP64 gate uses."""
import numpy as np
import pytest

import oracle
from conftest import golden_state, load_golden, rel_l2


def test_pow_dd_matches_correct_rounding():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(7)
    xs = np.concatenate([rng.uniform(0.8, 1.05, 3000), np.exp(rng.uniform(-30, 30, 1000))])
    for y in (1004.5 / 717.5, 287.0 / 1004.5, 717.5 / 1004.5):
        for x in xs:
            want = float(mpmath.mpf(float(x)) ** mpmath.mpf(y))
            assert oracle.pow_dd(float(x), y) == want, (x, y)


def test_pow_dd_special_values():
    assert oracle.pow_dd(1.0, 1.4) == 1.0
    assert oracle.pow_dd(2.0, 0.0) == 1.0
    assert oracle.pow_dd(0.0, 1.4) == 0.0
    assert np.isnan(oracle.pow_dd(-1.0, 1.4))


@pytest.mark.parametrize("case", ["c1_2d", "g3_4n3"])
def test_floor_only_in_momentum(case):
    """With a correctly rounded pow the oracle stays within 1e-12 of the
    reference in rho and rho*theta; momentum differences are the pow floor."""
    g = load_golden(case)
    m = oracle.OracleMesh(g)
    u0 = golden_state(g, "u0" if str(g["start"]) == "rest" else "up")
    st = int(g["steps"][-1])
    oracle.set_pow(1)
    try:
        u = m.ssprk3(u0, float(g["dt"]), st)
    finally:
        oracle.set_pow(0)
    ref = golden_state(g, f"traj_{st}")
    assert rel_l2(u[0], ref[0]) <= 1e-12
    assert rel_l2(u[4], ref[4]) <= 1e-12
    for c in (1, 3):
        assert rel_l2(u[c], ref[c]) <= 1e-9
