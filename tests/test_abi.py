"""C-ABI checks that need no GPU: the library builds, loads and exports every symbol the header
declares; host-side validation rejects bad configurations before touching the device."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fdtd_api.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fdtd_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from fdtd_gb300 import build, solver
    build.build()
    return solver.load_library()


def test_header_symbols_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s


def test_python_bindings_cover_header():
    from fdtd_gb300 import solver
    assert set(declared_symbols()) == set(solver.SIGNATURES)


def test_version(lib):
    assert b"sm_103a" in lib.fdtd_version()


def _grid(**kw):
    from fdtd_gb300 import solver
    g = solver.Grid()
    g.nx, g.ny, g.nz = kw.get("n", (32, 32, 32))
    g.dx = g.dy = g.dz = 1e-3
    g.dt = kw.get("dt", 1.9e-12)
    g.eps0, g.mu0, g.pi = 8.854e-12, 1.2566e-6, 3.1415
    for q, v in enumerate(kw.get("pml", (10,) * 6)):
        g.pml[q] = v
    return g


@pytest.mark.parametrize("kw,msg", [
    (dict(n=(2, 32, 32)), b"at least 3"),
    (dict(dt=-1.0), b"positive"),
    (dict(pml=(16, 16, 10, 10, 10, 10)), b"overlap"),
    (dict(pml=(-1, 10, 10, 10, 10, 10)), b"negative"),
])
def test_create_rejects_bad_grid(lib, kw, msg):
    h = ctypes.c_void_p()
    rc = lib.fdtd_create(ctypes.byref(_grid(**kw)), ctypes.byref(h))
    assert rc == 1  # FDTD_ERR_INVALID
    assert msg in lib.fdtd_last_error()
    assert not h.value


def test_null_handle_errors(lib):
    assert lib.fdtd_step(None, 1) == 1
    assert lib.fdtd_destroy(None) == 0
    assert lib.fdtd_current_step(None) == -1
    assert lib.fdtd_active_schedule(None) == -1
