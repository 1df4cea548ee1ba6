"""Error behaviour of the C ABI on the GPU: every call returns a status code
and the context stays usable afterwards (no exits, no traps)."""
import numpy as np
import pytest

from conftest import golden_state, load_golden

pytestmark = pytest.mark.gpu


def test_bad_arguments_and_unsupported_combinations():
    import nebulasem_gb300 as ng
    g = load_golden("g3_2")
    s = ng.Solver(g, dt=float(g["dt"]))
    s.set_state(golden_state(g, "u0"))
    lib, ctx = s._lib, s._ctx
    assert lib.nsem_step(ctx, -1, ng.SSPRK3, ng.FP64) == 1            # BAD_ARG
    assert lib.nsem_step(ctx, 1, 7, ng.FP64) == 1                     # unknown scheme
    assert lib.nsem_step(ctx, 1, ng.SSPRK3, 9) == 1                   # unknown precision
    assert lib.nsem_step(ctx, 1, ng.REF_SEGREGATED, ng.MIXED) == 5    # UNSUPPORTED
    assert lib.nsem_step(ctx, 0, ng.SSPRK3, ng.FP64) == 0             # nothing to do
    assert lib.nsem_last_error(ctx)
    assert lib.nsem_adjoint(ctx, None, None, None) == 1               # NULL arrays
    # the context still works
    before = s.get_state()
    s.step(2)
    after = s.get_state()
    assert not np.array_equal(before[4], after[4])
    s.close()


def test_nonfinite_state_is_reported_and_context_recovers():
    import nebulasem_gb300 as ng
    g = load_golden("g3_2")
    u = golden_state(g, "up")
    bad = [a.copy() for a in u]
    bad[4][17] = np.nan
    s = ng.Solver(g, dt=float(g["dt"]))
    for prec in (ng.FP64, ng.MIXED):
        s.set_state(bad)
        with pytest.raises(ng.NsemError) as e:
            s.step(1, prec=prec)
        assert e.value.status == 3                                     # NONFINITE
        # a clean state steps normally afterwards
        s.set_state(u)
        s.step(1, prec=prec)
        assert all(np.isfinite(a).all() for a in s.get_state())
    s.close()


def test_create_rejects_bad_parameters():
    import nebulasem_gb300 as ng
    g = load_golden("g3_2")
    with pytest.raises(ng.NsemError) as e:
        ng.Solver(g, dt=0.01, cp=700.0, cv=717.5)                      # cp < cv
    assert e.value.status == 1
    with pytest.raises(ng.NsemError) as e:
        ng.Solver(g, dt=0.01, viscosity=1.0, Pr=0.0)                   # viscous needs Pr > 0
    assert e.value.status == 1
