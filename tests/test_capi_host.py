"""CPU tests of the C ABI: the library builds/loads, exports every declared symbol, and validates
arguments in host code (no GPU needed)."""
import ctypes
import os
import re

import pytest

import exadg_gb300 as E
from exadg_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return E.load_library()


def test_header_symbols_exported(lib):
    hdr = open(os.path.join(ROOT, "include", "exadg_gb300.h")).read()
    declared = set(re.findall(r"(?:exg_status|const char\*)\s+(exg_\w+)\s*\(", hdr))
    assert declared == set(E.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(lib, name), name


def test_status_strings(lib):
    assert lib.exg_status_string(0) == b"ok"
    assert lib.exg_status_string(3) == b"solver did not converge"


def test_mesh_validation(lib):
    d = E.MeshDesc()
    d.n_cells[:] = [0, 2, 2]
    d.hi[:] = [1, 1, 1]
    h = ctypes.c_void_p()
    assert lib.exg_mesh_create(ctypes.byref(d), ctypes.byref(h)) == E.EXG_ERR_INVALID
    assert b"n_cells" in lib.exg_last_error()
    d.n_cells[:] = [2, 2, 2]
    d.bc[:] = [0, 0, 7, 0, 0, 0]
    assert lib.exg_mesh_create(ctypes.byref(d), ctypes.byref(h)) == E.EXG_ERR_INVALID
    d.bc[:] = [0] * 6
    d.deform_amp = 0.1
    d.periodic[:] = [1, 0, 0]
    assert lib.exg_mesh_create(ctypes.byref(d), ctypes.byref(h)) == E.EXG_ERR_UNSUPPORTED


def test_operator_validation_host_only(lib):
    m = E.Mesh(2)
    h = ctypes.c_void_p()
    assert lib.exg_sipg_create(m.h, 0, 1.0, E.PREC_F64, ctypes.byref(h)) == E.EXG_ERR_UNSUPPORTED
    assert lib.exg_sipg_create(m.h, 9, 1.0, E.PREC_F64, ctypes.byref(h)) == E.EXG_ERR_UNSUPPORTED
    assert lib.exg_sipg_create(m.h, 2, 1.0, 7, ctypes.byref(h)) == E.EXG_ERR_INVALID
    # Cartesian operators are set up on the host: size query works without a GPU
    assert lib.exg_sipg_create(m.h, 3, 1.0, E.PREC_F64, ctypes.byref(h)) == E.EXG_OK
    n = ctypes.c_longlong()
    assert lib.exg_sipg_n_dofs(h, ctypes.byref(n)) == 0 and n.value == 8 * 64
    # null pointers and precision mismatches are rejected before any device work
    assert lib.exg_sipg_apply_f64(h, None, None, 1, None) == E.EXG_ERR_INVALID
    assert lib.exg_sipg_apply_f32(h, ctypes.c_void_p(16), ctypes.c_void_p(32), 1, None) == E.EXG_ERR_INVALID
    assert lib.exg_sipg_apply_f64(h, ctypes.c_void_p(16), ctypes.c_void_p(16), 1, None) == E.EXG_ERR_INVALID
    assert lib.exg_sipg_destroy(h) == 0


def test_default_descriptors(lib):
    d = E.MGDesc()
    assert lib.exg_mg_default_desc(ctypes.byref(d)) == 0
    assert (d.mg_precision, d.cheb_degree, d.smoothing_range, d.eig_iters) == (E.PREC_F32, 5, 20.0, 20)
    assert d.coarse_rel_tol == 1e-3
    c = E.CGDesc()
    assert lib.exg_cg_default_desc(ctypes.byref(c)) == 0
    assert (c.max_iter, c.rel_tol, c.abs_tol) == (10000, 1e-10, 1e-20)
