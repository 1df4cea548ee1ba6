"""The fast phase of the correctly rounded pow: its error bound holds with
the stated margin, and whenever its rounding test passes it returns the same
double as the accurate double-double phase."""
import math

import numpy as np
import pytest

import oracle

GAMMA = 1004.5 / 717.5       # cp / cv: the equation of state's exponent
KAPPA = 287.0 / 1004.5       # R / cp: Exner function


@pytest.mark.parametrize("xlo,xhi,y", [(0.5, 1.5, GAMMA), (0.5, 1.5, KAPPA), (0.9, 1.1, 1 / GAMMA),
                                       (1e-5, 1e5, 3.7), (1e-300, 1e300, GAMMA)])
def test_fast_phase_agrees_with_accurate_phase(xlo, xhi, y):
    fb, mm = oracle.pow_fast_sweep(4_000_000, 2024, xlo, xhi, y)
    assert mm == 0
    if xhi / xlo < 1e20:
        # near-midpoint cases only: the accurate phase runs for a few calls in 2^14
        assert fb < 4_000_000 * 2.0 ** -11


def test_fast_phase_error_bound_has_margin():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 160
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.uniform(0.5, 1.5, 1500), np.exp(rng.uniform(-200, 200, 500)),
                         1.0 + rng.uniform(-1e-6, 1e-6, 200)])
    worst = 0.0
    for y in (GAMMA, KAPPA, -2.5):
        for x in xs:
            r = oracle.pow_fast_core(float(x), y)
            if r is None:
                continue
            hi, lo, err, k = r
            exact = mpmath.mpf(float(x)) ** mpmath.mpf(y)
            got = (mpmath.mpf(hi) + mpmath.mpf(lo)) * mpmath.mpf(2) ** k
            e = abs(got - exact) / (mpmath.mpf(err) * mpmath.mpf(2) ** k)
            worst = max(worst, float(e))
    assert worst <= 0.25, worst


def test_pow_dd_uses_accurate_phase_results():
    """pow_dd (fast phase first) equals the accurate phase alone."""
    rng = np.random.default_rng(5)
    for x in rng.uniform(0.6, 1.2, 2000):
        assert oracle.pow_dd(float(x), GAMMA) == oracle.pow_dd_accurate(float(x), GAMMA)
    assert math.isnan(oracle.pow_dd(-1.0, GAMMA))
