"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(nsem_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("nsem_create", "nsem_destroy", "nsem_step", "nsem_tendency",
                     "nsem_set_state", "nsem_get_state", "nsem_diagnostics"):
        assert required in names


def test_library_exports_every_declared_symbol():
    import nebulasem_gb300
    lib = nebulasem_gb300.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    with open(os.path.join(ROOT, "include", "nsem.h")) as f:
        version = int(re.search(r"#define NSEM_ABI_VERSION (\d+)", f.read()).group(1))
    assert lib.nsem_abi_version() == version


def test_create_rejects_null_mesh():
    """A NULL mesh is refused with BAD_ARG before any CUDA call."""
    import nebulasem_gb300 as ng
    lib = ng.load()
    ctx = ctypes.c_void_p()
    pr = ng.Params()
    pr.P0, pr.T0, pr.cp, pr.cv, pr.dt = 1e5, 300.0, 1004.5, 717.5, 0.01
    st = lib.nsem_create(None, ctypes.byref(pr), ctypes.byref(ctx))
    assert st == 1
    assert b"NULL" in lib.nsem_last_error(ctx)
    lib.nsem_destroy(ctx)
