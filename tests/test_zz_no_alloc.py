"""exg_cg_solve_noalloc: the CG solve for callers that cannot allocate device memory while they
run (cudaMalloc / cudaFree synchronise the device and would stall a time loop with other streams
in flight; some host frameworks own the whole device pool).  Its work vectors live in a static
device array, so it must give the same answer as exg_cg_solve, call after call.

This file is collected last on purpose: a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

import exadg_gb300 as E
from tests.gpu_common import require_gpu, to_dev
from tests.helpers import splitmix_uniform

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precond", [1, 0])
def test_noalloc_cg_matches_allocating_cg_twice(precond):
    torch = require_gpu()
    L = E.load_library()
    mesh = E.Mesh((6, 5, 4), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0))
    op = E.LaplaceOperator(mesh, 3)  # 7,680 DoF
    d = E.CGDesc()
    assert L.exg_cg_default_desc(ctypes.byref(d)) == 0
    d.precond = precond
    d.rel_tol = 1e-10
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # two calls in a row share the static scratch
        b = to_dev(torch, splitmix_uniform(op.n_dofs, 10 + call))
        x_ref = op.initialize_dof_vector()
        r_ref = E.CGResult()
        st = L.exg_cg_solve(op.h, None, ctypes.byref(d), ctypes.c_void_p(b.data_ptr()),
                            ctypes.c_void_p(x_ref.data_ptr()), ctypes.byref(r_ref), stream)
        assert st == 0
        x = op.initialize_dof_vector()
        r = E.CGResult()
        st = L.exg_cg_solve_noalloc(op.h, ctypes.byref(d), ctypes.c_void_p(b.data_ptr()),
                                    ctypes.c_void_p(x.data_ptr()), ctypes.byref(r), stream)
        assert st == 0, L.exg_last_error()
        torch.cuda.synchronize()
        assert r.converged and abs(r.iterations - r_ref.iterations) <= 1
        err = float(torch.linalg.norm(x - x_ref) / torch.linalg.norm(x_ref))
        assert err <= 1e-8, err


def test_noalloc_rejects_oversized_problem():
    torch = require_gpu()
    L = E.load_library()
    op = E.LaplaceOperator(E.Mesh(21), 3)  # 9,261 cells x 64 = 592,704 DoF > 524,288
    d = E.CGDesc()
    L.exg_cg_default_desc(ctypes.byref(d))
    d.precond = 1
    b = op.initialize_dof_vector()
    x = op.initialize_dof_vector()
    st = L.exg_cg_solve_noalloc(op.h, ctypes.byref(d), ctypes.c_void_p(b.data_ptr()),
                                ctypes.c_void_p(x.data_ptr()), None,
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == E.EXG_ERR_INVALID
    assert b"524288" in L.exg_last_error()


def test_noalloc_refuses_point_jacobi_on_continuous_cartesian_operator():
    """That diagonal set-up would need a temporary device allocation, so the call is refused."""
    torch = require_gpu()
    L = E.load_library()
    op = E.ContinuousLaplaceOperator(E.Mesh(4), 2)
    d = E.CGDesc()
    L.exg_cg_default_desc(ctypes.byref(d))
    d.precond = 1
    b = op.initialize_dof_vector()
    x = op.initialize_dof_vector()
    st = L.exg_cg_solve_noalloc(op.h, ctypes.byref(d), ctypes.c_void_p(b.data_ptr()),
                                ctypes.c_void_p(x.data_ptr()), None,
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == E.EXG_ERR_UNSUPPORTED
    assert b"allocate" in L.exg_last_error()

