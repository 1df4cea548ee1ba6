"""Allocation-free conservation sums against nsem_diagnostics.

nsem_conservation_sums_noalloc() serves host codes that own all device
memory and may not let a library call cudaMalloc while they run (embedded
solvers with their own memory pool, time loops that must not synchronise the
device through an allocation).  It takes raw device buffers and works in one
fixed file-scope device array.  This test gives it device copies of a state
and the node geometry, calls it twice in a row through the C ABI, and checks
both results against the context-based nsem_diagnostics() at the tolerance
the diagnostics parity test uses (1e-13 relative).  It lives in its own file
that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden_state, load_golden

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _noalloc_fn(lib):
    fn = lib.nsem_conservation_sums_noalloc
    P = ctypes.c_void_p
    fn.argtypes = [P, P, P, P, P, P, P, P, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                   ctypes.c_double, P, P]
    fn.restype = ctypes.c_int
    return fn


def _check_case(mesh, u, gh, p_ref, dt):
    import torch

    import nebulasem_gb300 as ng

    s = ng.Solver(mesh, dt=dt)
    s.set_state(u)
    want = s.diagnostics()
    s.close()
    n = len(u[0])
    dev = [torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda") for a in u]
    cV = torch.tensor(np.ascontiguousarray(mesh["cV"][:n]), dtype=torch.float64, device="cuda")
    ghd = torch.tensor(np.ascontiguousarray(gh[:n]), dtype=torch.float64, device="cuda")
    prd = torch.tensor(np.ascontiguousarray(p_ref[:n]), dtype=torch.float64, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    fn = _noalloc_fn(ng.load())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [ctypes.c_void_p(t.data_ptr()) for t in dev]
    # warm-up call (resolves the array's address on this device), then the
    # device's free memory must not move across the checked calls
    assert fn(*args, ctypes.c_void_p(cV.data_ptr()), ctypes.c_void_p(ghd.data_ptr()),
              ctypes.c_void_p(prd.data_ptr()), n, 1e5, 1004.5, 717.5,
              ctypes.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2):
        out.fill_(-1.0)
        st = fn(*[ctypes.c_void_p(t.data_ptr()) for t in dev],
                ctypes.c_void_p(cV.data_ptr()), ctypes.c_void_p(ghd.data_ptr()),
                ctypes.c_void_p(prd.data_ptr()), n, 1e5, 1004.5, 717.5,
                ctypes.c_void_p(out.data_ptr()), stream)
        assert st == 0, f"call {call}: status {st}"
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, "the call changed the device's free memory"
        got = out.cpu().numpy()
        assert np.allclose(got, want, rtol=RTOL, atol=0), (call, got, want)
    # beyond the fixed capacity: refused before any device work
    st = fn(*[ctypes.c_void_p(t.data_ptr()) for t in dev],
            ctypes.c_void_p(cV.data_ptr()), ctypes.c_void_p(ghd.data_ptr()),
            ctypes.c_void_p(prd.data_ptr()), 4096 * 65536 + 1, 1e5, 1004.5, 717.5,
            ctypes.c_void_p(out.data_ptr()), stream)
    assert st == 7


def test_noalloc_sums_match_diagnostics_fixture():
    g = load_golden("c1_2d")
    _check_case(g, golden_state(g, "up"), g["gh"], g["p_ref"], float(g["dt"]))


def test_noalloc_sums_match_diagnostics_many_chunks():
    from nebulasem_gb300.mesh import workload

    m, u = workload("bubble3d_8_n4")
    _check_case(m, u, m["gh"], m["p_ref"], 0.0075)


def test_noalloc_sums_match_diagnostics_over_256_chunks():
    # 4.1 M nodes = 1000 chunks: the final pass strides over its partial sums
    # and merges several per thread
    from nebulasem_gb300.mesh import workload

    m, u = workload("bubble3d_32_n4")
    _check_case(m, u, m["gh"], m["p_ref"], 0.0075)
