"""GPU parity of the diagonal-preconditioned and multigrid-preconditioned CG against the oracle:
iteration counts within +-1, Chebyshev eigenvalue estimates, V-cycle output, and the reference's
sine golden errors reproduced by the GPU solve."""
import json
import os

import numpy as np
import pytest

import exadg_gb300 as E
import oracle as O
from tests.gpu_common import rel, require_gpu, to_dev
from tests.helpers import splitmix_uniform

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sine_errors.json")))


def sine(k, curved, n=8):
    kw = dict(n_cells=(n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0),
              deform_amp=0.15 if curved else 0.0, deform_freq=2, deform_left=-1.0, deform_right=1.0,
              mapping_degree=3)
    return O.Problem(O.mesh_desc(**kw), k), E.Mesh(**kw)


def test_cg_jacobi_config_1():
    torch = require_gpu()
    kw = dict(n_cells=(8, 8, 8))
    p = O.Problem(O.mesh_desc(**kw), 3)
    op = E.LaplaceOperator(E.Mesh(**kw), 3)
    b = p.rhs(O.FN_SINE, np.pi)
    xo, ro = p.solve(b, precond=1)
    x = op.initialize_dof_vector()
    solver = E.KrylovSolver(op, None, precond=E.KrylovSolver.JACOBI)
    its = solver.solve(x, to_dev(torch, b))
    assert abs(its - ro.iterations) <= 1
    assert rel(x.cpu().numpy(), xo) <= 1e-8


@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_mg_levels_and_eigenvalues(mg_prec):
    torch = require_gpu()
    p, m = sine(4, False)
    op = E.LaplaceOperator(m, 4)
    mg = E.MultigridPreconditioner(op, mg_precision=mg_prec)
    omg = O.Multigrid(p, mg_float=1 if mg_prec == E.PREC_F32 else 0)
    info = mg.info()
    ol = omg.levels()
    assert info["n_levels"] == len(ol)
    for g, o in zip(info["levels"], ol):
        assert g["degree"] == o["degree"] and g["n_cells"] == o["n_cells"]
        if o["eig_iters"]:
            assert g["eig_iters"] == o["eig_iters"]
            assert g["lambda_max"] == pytest.approx(o["lambda_max"], rel=1e-9 if mg_prec == E.PREC_F64 else 1e-4)


@pytest.mark.parametrize("curved", [False, True])
def test_vcycle_matches_oracle_double(curved):
    torch = require_gpu()
    p, m = sine(3, curved)
    op = E.LaplaceOperator(m, 3)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64)
    omg = O.Multigrid(p, mg_float=0)
    for seed in (1, 2):
        r = splitmix_uniform(p.n_dofs, seed)
        z = mg.vmult(op.initialize_dof_vector(), to_dev(torch, r))
        assert rel(z.cpu().numpy(), omg.vmult(r)) <= 1e-9


@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_fused_smoother_and_graph_replay(curved, mg_prec):
    """Chebyshev steps and level residuals fused into the operator kernels, replayed as a CUDA
    graph, give the iterates of the separate vector kernels run eagerly, over a sequence of
    V-cycles (the coarse solver starts from its previous solution)."""
    torch = require_gpu()
    k = 4 if not curved else 3
    _, m = sine(k, curved, n=6)
    op = E.LaplaceOperator(m, k)
    fused = E.MultigridPreconditioner(op, mg_precision=mg_prec, fuse_smoother=True, use_graph=True)
    plain = E.MultigridPreconditioner(op, mg_precision=mg_prec, fuse_smoother=False, use_graph=False)
    tol = 1e-12 if mg_prec == E.PREC_F64 else 1e-5
    for seed in (3, 4, 5):
        r = to_dev(torch, splitmix_uniform(op.n_dofs, seed))
        a = fused.vmult(op.initialize_dof_vector(), r)
        b = plain.vmult(op.initialize_dof_vector(), r)
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) <= tol


@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("k", [2, 4, 5])
@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_sine_solve_golden_and_iterations(curved, k, mg_prec):
    torch = require_gpu()
    p, m = sine(k, curved)
    op = E.LaplaceOperator(m, k)
    mg = E.MultigridPreconditioner(op, mg_precision=mg_prec)
    b = p.rhs(O.FN_SINE, 3 * np.pi)
    x = op.initialize_dof_vector()
    solver = E.KrylovSolver(op, mg)
    its = solver.solve(x, to_dev(torch, b))
    xo, ro = O.Multigrid(p, mg_float=1 if mg_prec == E.PREC_F32 else 0).solve(b)
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    err = p.error(x.cpu().numpy(), O.FN_SINE, 3 * np.pi)
    gold = GOLD["curvilinear" if curved else "cartesian"]["relative_l2_error"][k - 1]
    assert abs(err - gold) <= 5e-6 * gold


def test_cg_reports_nonfinite_and_max_iter():
    torch = require_gpu()
    op = E.LaplaceOperator(E.Mesh(4), 2)
    b = to_dev(torch, splitmix_uniform(op.n_dofs, 1))
    x = op.initialize_dof_vector()
    s = E.KrylovSolver(op, None, precond=E.KrylovSolver.JACOBI, max_iter=2)
    s.solve(x, b, raise_on_failure=False)
    assert s.result["status"] == E.EXG_ERR_NOT_CONVERGED and s.result["iterations"] == 2
    b[5] = float("nan")
    x.zero_()
    s2 = E.KrylovSolver(op, None, precond=E.KrylovSolver.JACOBI)
    s2.solve(x, b, raise_on_failure=False)
    assert s2.result["status"] == E.EXG_ERR_NONFINITE


@pytest.mark.parametrize("precond", [E.KrylovSolver.MULTIGRID, E.KrylovSolver.JACOBI, E.KrylovSolver.NONE])
@pytest.mark.parametrize("warm", [False, True])
def test_device_loop_matches_host_loop(precond, warm):
    """The graph-driven CG (WHILE node, scalars on the device) takes the iterations of the host loop
    and returns the same solution; repeated solves replay the captured graph, and a change of
    preconditioner re-captures it."""
    torch = require_gpu()
    p, m = sine(3, False)
    op = E.LaplaceOperator(m, 3)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64) if precond == E.KrylovSolver.MULTIGRID else None
    b = to_dev(torch, p.rhs(O.FN_SINE, np.pi))
    for rep in range(2):
        x0 = to_dev(torch, 0.1 * splitmix_uniform(p.n_dofs, 7 + rep)) if warm else op.initialize_dof_vector()
        xs = []
        its = []
        for device_loop in (False, True):
            x = x0.clone()
            s = E.KrylovSolver(op, mg, precond=precond, device_loop=device_loop, max_iter=2000)
            its.append(s.solve(x, b))
            xs.append(x)
        assert its[0] == its[1]
        assert float(torch.linalg.norm(xs[0] - xs[1]) / torch.linalg.norm(xs[0])) <= 1e-13


def test_device_loop_status_codes():
    torch = require_gpu()
    op = E.LaplaceOperator(E.Mesh(4), 2)
    b = to_dev(torch, splitmix_uniform(op.n_dofs, 1))
    x = op.initialize_dof_vector()
    s = E.KrylovSolver(op, None, precond=E.KrylovSolver.JACOBI, max_iter=3, device_loop=True)
    s.solve(x, b, raise_on_failure=False)
    assert s.result["status"] == E.EXG_ERR_NOT_CONVERGED and s.result["iterations"] == 3
    x.zero_()
    s.solve(x, torch.zeros_like(b), raise_on_failure=False)  # converged at iteration 0
    assert s.result["status"] == 0 and s.result["iterations"] == 0


def test_inconsistent_singular_problem_reports_failure():
    """A periodic (singular) problem whose right-hand side has a mean, solved without mean
    projection: no solution exists; the solver stops at its iteration cap with a status instead
    of hanging or faulting, in both loop variants."""
    torch = require_gpu()
    m = E.Mesh(4, periodic=(1, 1, 1))
    op = E.LaplaceOperator(m, 2)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64, singular=False, coarse_max_iter=200)
    b = to_dev(torch, splitmix_uniform(op.n_dofs, 3) + 1.0)
    for device_loop in (True, False):
        x = op.initialize_dof_vector()
        s = E.KrylovSolver(op, mg, max_iter=50, device_loop=device_loop)
        s.solve(x, b, raise_on_failure=False)
        assert s.result["status"] in (E.EXG_ERR_NOT_CONVERGED, E.EXG_ERR_NONFINITE)
        assert s.result["iterations"] <= 50


def test_mismatched_vectors_are_rejected():
    """Raw pointers cross the C ABI, so the Python layer rejects vectors of the wrong size or type
    before any kernel could over-run them."""
    torch = require_gpu()
    op = E.LaplaceOperator(E.Mesh(3), 2)
    n = op.n_dofs
    good = op.initialize_dof_vector()
    for bad in (torch.zeros(n - 1, dtype=torch.float64, device="cuda"), torch.zeros(n, dtype=torch.float32, device="cuda")):
        with pytest.raises(E.ExgError):
            op.vmult(good, bad)
        with pytest.raises(E.ExgError):
            op.vmult(bad, good)
        with pytest.raises(E.ExgError):
            E.KrylovSolver(op, None, precond=E.KrylovSolver.JACOBI).solve(bad, good)
    with pytest.raises(E.ExgError):
        op.vmult(good, good, n_rhs=2)
    with pytest.raises(E.ExgError):
        op.vmult_host(torch.zeros(n - 1, dtype=torch.float64), torch.zeros(n, dtype=torch.float64))


def test_level_timings_match_vcycle():
    """The event-timed eager V-cycle gives the graph V-cycle's result and one positive time per
    level."""
    torch = require_gpu()
    p, m = sine(3, False)
    op = E.LaplaceOperator(m, 3)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64)
    r = to_dev(torch, splitmix_uniform(p.n_dofs, 4))
    ms = mg.level_timings(r)
    assert len(ms) == mg.info()["n_levels"] and all(t > 0 for t in ms)
    mg2 = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64)
    a = mg2.vmult(op.initialize_dof_vector(), r)
    mg3 = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64)
    b = torch.empty_like(r)
    mg3.level_timings(r, b)
    assert float(torch.linalg.norm(a - b) / torch.linalg.norm(a)) <= 1e-13


def _composed_vcycle(mg, src):
    """MultigridAlgorithm::v_cycle (multigrid_algorithm.h:172-240) written against the level
    objects of the C ABI: smoother vmult/step, level vmult, restrict_and_add, coarse solver,
    prolongate_and_add."""
    import torch

    nl = mg.info()["n_levels"]
    dt = mg.level_dtype
    defs = [torch.zeros(mg.level_n_dofs(l), dtype=dt, device="cuda") for l in range(nl)]
    sols = [torch.zeros_like(d) for d in defs]
    defs[-1].copy_(src.to(dt))

    def cycle(l):
        if l == 0:
            mg.coarse_solve(sols[0], defs[0])
            return
        mg.smooth(l, sols[l], defs[l], zero_start=True)
        t = torch.empty_like(defs[l])
        mg.level_vmult(l, t, sols[l])
        mg.restrict_and_add(l, defs[l - 1], defs[l] - t)
        cycle(l - 1)
        mg.prolongate_and_add(l, sols[l], sols[l - 1])
        mg.smooth(l, sols[l], defs[l], zero_start=False)

    cycle(nl - 1)
    return sols[-1].double()


@pytest.mark.parametrize("mg_type", [E.MG_PH, E.MG_CPH])
@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
@pytest.mark.parametrize("curved", [False, True])
def test_vcycle_from_level_objects(mg_type, mg_prec, curved):
    """The V-cycle assembled from the exported smoother, transfer, level-operator and coarse-solver
    entry points reproduces exg_mg_vmult (two fresh preconditioners, so both coarse solvers start
    from zero; the second input checks the warm start)."""
    torch = require_gpu()
    _, m = sine(3, curved, n=4)
    op = E.LaplaceOperator(m, 3)
    kw = dict(mg_precision=mg_prec, mg_type=mg_type, use_graph=False)
    a = E.MultigridPreconditioner(op, **kw)
    b = E.MultigridPreconditioner(op, **kw)
    tol = 1e-13 if mg_prec == E.PREC_F64 else 1e-6
    for seed in (1, 2):
        r = to_dev(torch, splitmix_uniform(op.n_dofs, seed))
        ref = a.vmult(op.initialize_dof_vector(), r)
        got = _composed_vcycle(b, r)
        assert float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref)) <= tol


def test_level_transfers_are_transposes():
    torch = require_gpu()
    _, m = sine(3, False, n=4)
    op = E.LaplaceOperator(m, 3)
    for mg_type in (E.MG_PH, E.MG_CPH):
        mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64, mg_type=mg_type)
        for l in range(1, mg.info()["n_levels"]):
            nf, nc = mg.level_n_dofs(l), mg.level_n_dofs(l - 1)
            f = to_dev(torch, splitmix_uniform(nf, 3 + l))
            c = to_dev(torch, splitmix_uniform(nc, 7 + l))
            Rf = mg.restrict_and_add(l, torch.zeros(nc, dtype=torch.float64, device="cuda"), f)
            Pc = mg.prolongate_and_add(l, torch.zeros(nf, dtype=torch.float64, device="cuda"), c)
            lhs, rhs = float(Rf @ c), float(f @ Pc)
            assert abs(lhs - rhs) <= 1e-11 * max(1.0, abs(lhs))


@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
@pytest.mark.parametrize("graph", [True, False])
def test_block_jacobi_smoother_vcycle_matches_oracle(mg_prec, graph):
    """Chebyshev preconditioned by block Jacobi (PreconditionerSmoother::BlockJacobi)."""
    torch = require_gpu()
    from tests.helpers import mesh_kwargs

    kw = mesh_kwargs("mixed", 4)
    p = O.Problem(O.mesh_desc(**kw), 3)
    op = E.LaplaceOperator(E.Mesh(**kw), 3)
    mg = E.MultigridPreconditioner(op, mg_precision=mg_prec, block_jacobi_smoother=True, use_graph=graph)
    omg = O.Multigrid(p, mg_float=1 if mg_prec == E.PREC_F32 else 0, smoother_block=1)
    for g, o in zip(mg.info()["levels"], omg.levels()):
        if o["eig_iters"]:
            assert g["lambda_max"] == pytest.approx(o["lambda_max"], rel=1e-9 if mg_prec == E.PREC_F64 else 1e-4)
    for seed in (1, 2):
        r = splitmix_uniform(p.n_dofs, seed)
        z = mg.vmult(op.initialize_dof_vector(), to_dev(torch, r))
        # FP32: the GPU applies the block inverse by fast diagonalisation, the oracle by a dense
        # inverse; both in float, so the smoother's polynomial sees different rounding (1e-4 level)
        assert rel(z.cpu().numpy(), omg.vmult(r)) <= (1e-9 if mg_prec == E.PREC_F64 else 2e-4)


@pytest.mark.parametrize("k", [3, 4])
def test_block_jacobi_smoother_solve_iterations(k):
    torch = require_gpu()
    p, m = sine(k, False)
    op = E.LaplaceOperator(m, k)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F32, block_jacobi_smoother=True)
    b = p.rhs(O.FN_SINE, 3 * np.pi)
    x = op.initialize_dof_vector()
    its = E.KrylovSolver(op, mg).solve(x, to_dev(torch, b))
    xo, ro = O.Multigrid(p, mg_float=1, smoother_block=1).solve(b)
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    gold = GOLD["cartesian"]["relative_l2_error"][k - 1]
    assert abs(p.error(x.cpu().numpy(), O.FN_SINE, 3 * np.pi) - gold) <= 5e-6 * gold


def test_block_jacobi_smoother_rejects_continuous_and_curved_levels():
    require_gpu()
    _, m = sine(3, False, n=4)
    with pytest.raises(E.ExgError):
        E.MultigridPreconditioner(E.LaplaceOperator(m, 3), mg_type=E.MG_CPH, block_jacobi_smoother=True)
    _, mc = sine(3, True, n=4)
    with pytest.raises(E.ExgError):
        E.MultigridPreconditioner(E.LaplaceOperator(mc, 3), block_jacobi_smoother=True)
