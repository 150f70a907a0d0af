"""GPU parity of the continuous (cphMG) levels against the oracle: the FE_Q lattice operator and
its diagonal, the cphMG V-cycle in FP64 and FP32, and cphMG-preconditioned solves (iterations
within +-1 of the oracle, the reference's sine golden errors)."""
import json
import os

import numpy as np
import pytest

import exadg_gb300 as E
import oracle as O
from tests.gpu_common import rel, require_gpu, to_dev
from tests.helpers import mesh_kwargs, splitmix_uniform

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sine_errors.json")))
KINDS = ["dirichlet", "mixed", "periodic", "partial_periodic", "anisotropic"]


def _singular(kind):
    return kind == "periodic"


def _pair(kw, k, prec, singular):
    oc = O.ContinuousProblem(O.mesh_desc(**kw), k, singular=singular)
    op = E.ContinuousLaplaceOperator(E.Mesh(**kw), k, precision=prec, singular=singular)
    assert op.n_dofs == oc.n_dofs
    return oc, op


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32])
def test_continuous_apply_matches_oracle(kind, k, prec):
    torch = require_gpu()
    n = 3 if k <= 4 else 2
    oc, op = _pair(mesh_kwargs(kind, n), k, prec, _singular(kind))
    x = splitmix_uniform(oc.n_dofs, 21)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x, op.dtype)).cpu().numpy()
    if prec == E.PREC_F64:
        assert rel(y, oc.apply(x)) <= 1e-13
    else:
        assert rel(y, oc.apply_f32(x.astype(np.float32))) <= 2e-6
    # identity rows of the constrained nodes, stored bit for bit
    c = oc.constrained()
    assert np.array_equal(y[c], x.astype(y.dtype)[c])


@pytest.mark.parametrize("n_cells,k", [((9, 5, 7), 4), ((33, 2, 3), 2), ((1, 1, 1), 3), ((5, 17, 4), 1),
                                       ((4, 3, 11), 5)])
@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 1), (1, 0, 1)])
def test_continuous_apply_ragged_tiles(n_cells, k, periodic):
    """Lattices that do not fill whole tiles, several tiles per direction, single cells (a periodic
    node that couples to itself across the wrapped cell)."""
    torch = require_gpu()
    kw = dict(n_cells=n_cells, periodic=periodic, bc=(0, 1, 1, 0, 0, 1))
    singular = all(periodic)
    oc, op = _pair(kw, k, E.PREC_F64, singular)
    x = splitmix_uniform(oc.n_dofs, 5)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x)).cpu().numpy()
    assert rel(y, oc.apply(x)) <= 1e-13
    d = op.calculate_inverse_diagonal(op.initialize_dof_vector()).cpu().numpy()
    assert rel(d, 1.0 / oc.diagonal()) <= 1e-13


@pytest.mark.parametrize("k,n", [(2, 52), (3, 20), (4, 20), (5, 12)])
@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32])
@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 0, 1)])
def test_continuous_apply_full_tiles(k, n, prec, periodic):
    """Lattices large enough for the full-size tiles (and, at k = 2, above the direct kernel's
    size limit), with the Chebyshev store fused."""
    torch = require_gpu()
    kw = dict(n_cells=(n, n, n), periodic=periodic, bc=(0, 1, 0, 0, 1, 0))
    oc, op = _pair(kw, k, prec, False)
    x = splitmix_uniform(oc.n_dofs, 31)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x, op.dtype)).cpu().numpy()
    ref = oc.apply(x) if prec == E.PREC_F64 else oc.apply_f32(x.astype(np.float32))
    assert rel(y, ref) <= (1e-13 if prec == E.PREC_F64 else 2e-6)


@pytest.mark.parametrize("kind", ["mixed", "periodic"])
def test_continuous_inverse_diagonal_and_residual(kind):
    torch = require_gpu()
    oc, op = _pair(mesh_kwargs(kind, 3), 3, E.PREC_F64, _singular(kind))
    assert rel(op.calculate_inverse_diagonal(op.initialize_dof_vector()).cpu().numpy(), 1.0 / oc.diagonal()) <= 1e-14
    of = E.ContinuousLaplaceOperator(E.Mesh(**mesh_kwargs(kind, 3)), 3, precision=E.PREC_F32,
                                     singular=_singular(kind))
    assert rel(of.calculate_inverse_diagonal(of.initialize_dof_vector()).cpu().numpy(), 1.0 / oc.diagonal()) <= 1e-6
    x = splitmix_uniform(oc.n_dofs, 1)
    b = splitmix_uniform(oc.n_dofs, 2)
    r = op.residual(op.initialize_dof_vector(), to_dev(torch, b), to_dev(torch, x)).cpu().numpy()
    assert rel(r, b - oc.apply(x)) <= 1e-13


def test_continuous_operator_rejects_dg_only_calls():
    require_gpu()
    m = E.Mesh(3)
    op = E.ContinuousLaplaceOperator(m, 2)
    with pytest.raises(E.ExgError):
        op.quadrature_points()
    with pytest.raises(E.ExgError):  # singular flag differs from the operator's
        E.MultigridPreconditioner(op, singular=True)
    with pytest.raises(E.ExgError):
        E.MultigridPreconditioner(op, mg_type=7)


def sine(k, n=8):
    kw = dict(n_cells=(n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0))
    return O.Problem(O.mesh_desc(**kw), k), E.Mesh(**kw)


@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_cphmg_levels_and_eigenvalues(mg_prec):
    require_gpu()
    p, m = sine(4)
    mg = E.MultigridPreconditioner(E.LaplaceOperator(m, 4), mg_precision=mg_prec, mg_type=E.MG_CPH)
    omg = O.Multigrid(p, mg_float=1 if mg_prec == E.PREC_F32 else 0, mg_type=1)
    info, ol = mg.info(), omg.levels()
    assert [(g["n_cells"], g["degree"], g["dg"]) for g in info["levels"]] == \
        [(o["n_cells"], o["degree"], o["dg"]) for o in ol]
    assert [g["dg"] for g in info["levels"]] == [False] * 5 + [True]
    for g, o in zip(info["levels"], ol):
        if o["eig_iters"]:
            assert g["eig_iters"] == o["eig_iters"]
            assert g["lambda_max"] == pytest.approx(o["lambda_max"], rel=1e-9 if mg_prec == E.PREC_F64 else 1e-4)


@pytest.mark.parametrize("kind,k", [("mixed", 3), ("periodic", 2), ("partial_periodic", 4), ("dirichlet", 1)])
def test_cphmg_vcycle_matches_oracle_double(kind, k):
    torch = require_gpu()
    kw = mesh_kwargs(kind, 4)
    p = O.Problem(O.mesh_desc(**kw), k)
    singular = _singular(kind)
    op = E.LaplaceOperator(E.Mesh(**kw), k)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64, mg_type=E.MG_CPH, singular=singular)
    omg = O.Multigrid(p, mg_float=0, mg_type=1, singular=int(singular))
    for seed in (1, 2, 3):  # a sequence: the coarse solver starts from its previous solution
        r = splitmix_uniform(p.n_dofs, seed)
        z = mg.vmult(op.initialize_dof_vector(), to_dev(torch, r))
        assert rel(z.cpu().numpy(), omg.vmult(r)) <= 1e-9


@pytest.mark.parametrize("fuse,graph", [(True, True), (False, False)])
def test_cphmg_vcycle_matches_oracle_float(fuse, graph):
    torch = require_gpu()
    p, m = sine(4, n=6)
    op = E.LaplaceOperator(m, 4)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F32, mg_type=E.MG_CPH, fuse_smoother=fuse,
                                   use_graph=graph)
    omg = O.Multigrid(p, mg_float=1, mg_type=1)
    for seed in (4, 5):
        r = splitmix_uniform(p.n_dofs, seed)
        z = mg.vmult(op.initialize_dof_vector(), to_dev(torch, r))
        assert rel(z.cpu().numpy(), omg.vmult(r)) <= 2e-5


@pytest.mark.parametrize("k", [2, 3, 5])
@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_cphmg_sine_solve_golden_and_iterations(k, mg_prec):
    torch = require_gpu()
    p, m = sine(k)
    op = E.LaplaceOperator(m, k)
    mg = E.MultigridPreconditioner(op, mg_precision=mg_prec, mg_type=E.MG_CPH)
    b = p.rhs(O.FN_SINE, 3 * np.pi)
    x = op.initialize_dof_vector()
    its = E.KrylovSolver(op, mg).solve(x, to_dev(torch, b))
    xo, ro = O.Multigrid(p, mg_float=1 if mg_prec == E.PREC_F32 else 0, mg_type=1).solve(b)
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    err = p.error(x.cpu().numpy(), O.FN_SINE, 3 * np.pi)
    gold = GOLD["cartesian"]["relative_l2_error"][k - 1]
    assert abs(err - gold) <= 5e-6 * gold


def test_cphmg_singular_periodic_solve():
    torch = require_gpu()
    kw = dict(n_cells=(8, 8, 8), periodic=(1, 1, 1))
    p = O.Problem(O.mesh_desc(**kw), 3)
    op = E.LaplaceOperator(E.Mesh(**kw), 3)
    b = splitmix_uniform(p.n_dofs, 8)
    b -= b.mean()
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F32, mg_type=E.MG_CPH, singular=True)
    x = op.initialize_dof_vector()
    its = E.KrylovSolver(op, mg).solve(x, to_dev(torch, b))
    xo, ro = O.Multigrid(p, mg_float=1, mg_type=1, singular=1).solve(b)
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    xg = x.cpu().numpy()
    assert rel(xg - xg.mean(), xo - xo.mean()) <= 1e-8


# ---- curved meshes: the continuous operator is the DG cell term assembled through the lattice


@pytest.mark.parametrize("k", [1, 2, 3, 5])
@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32])
def test_curved_continuous_apply_and_diagonal(k, prec):
    torch = require_gpu()
    kw = mesh_kwargs("curved", 3)
    oc, op = _pair(kw, k, prec, False)
    x = splitmix_uniform(oc.n_dofs, 41)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x, op.dtype)).cpu().numpy()
    d = op.calculate_inverse_diagonal(op.initialize_dof_vector()).cpu().numpy()
    if prec == E.PREC_F64:
        assert rel(y, oc.apply(x)) <= 1e-12
        assert rel(d, 1.0 / oc.diagonal()) <= 1e-12
    else:
        assert rel(y, oc.apply_f32(x.astype(np.float32))) <= 2e-5
        assert rel(d, 1.0 / oc.diagonal()) <= 2e-5
    c = oc.constrained()
    assert np.array_equal(y[c], x.astype(y.dtype)[c])


def curved_sine(k, n=8):
    kw = dict(n_cells=(n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0), deform_amp=0.15,
              deform_freq=2, deform_left=-1.0, deform_right=1.0, mapping_degree=3)
    return O.Problem(O.mesh_desc(**kw), k), E.Mesh(**kw)


@pytest.mark.parametrize("k", [2, 3])
def test_curved_cphmg_vcycle_matches_oracle(k):
    torch = require_gpu()
    p, m = curved_sine(k, n=4)
    op = E.LaplaceOperator(m, k)
    mg = E.MultigridPreconditioner(op, mg_precision=E.PREC_F64, mg_type=E.MG_CPH)
    omg = O.Multigrid(p, mg_float=0, mg_type=1)
    assert [g["dg"] for g in mg.info()["levels"]] == [o["dg"] for o in omg.levels()]
    for seed in (1, 2):
        r = splitmix_uniform(p.n_dofs, seed)
        z = mg.vmult(op.initialize_dof_vector(), to_dev(torch, r))
        assert rel(z.cpu().numpy(), omg.vmult(r)) <= 1e-9


@pytest.mark.parametrize("k", [2, 3, 5])
@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_curved_cphmg_sine_solve_golden_and_iterations(k, mg_prec):
    """The reference's curvilinear sine configuration (cphMG, MappingQ3, 8^3 cells)."""
    torch = require_gpu()
    p, m = curved_sine(k)
    op = E.LaplaceOperator(m, k)
    mg = E.MultigridPreconditioner(op, mg_precision=mg_prec, mg_type=E.MG_CPH)
    b = p.rhs(O.FN_SINE, 3 * np.pi)
    x = op.initialize_dof_vector()
    its = E.KrylovSolver(op, mg).solve(x, to_dev(torch, b))
    xo, ro = O.Multigrid(p, mg_float=1 if mg_prec == E.PREC_F32 else 0, mg_type=1).solve(b)
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    err = p.error(x.cpu().numpy(), O.FN_SINE, 3 * np.pi)
    gold = GOLD["curvilinear"]["relative_l2_error"][k - 1]
    assert abs(err - gold) <= 5e-6 * gold


# ---- the continuous discretization: CG on the continuous operator with continuous multigrid


@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("k", [2, 4])
@pytest.mark.parametrize("mg_prec", [E.PREC_F64, E.PREC_F32])
def test_continuous_discretization_multigrid_solve(curved, k, mg_prec):
    """The sine problem on FE_Q(k): b = P_c^T of the DG right-hand side (homogeneous data on the
    constrained nodes); CG + multigrid on FE_Q levels against the oracle (iterations +-1)."""
    torch = require_gpu()
    if curved:
        kw = dict(n_cells=(8, 8, 8), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0), deform_amp=0.15,
                  deform_freq=2, deform_left=-1.0, deform_right=1.0, mapping_degree=3)
        omega = 3 * np.pi
    else:
        kw = dict(n_cells=(8, 8, 8))
        omega = np.pi
    oc = O.ContinuousProblem(O.mesh_desc(**kw), k)
    dg = O.Problem(O.mesh_desc(**kw), k)
    b = np.bincount(oc.dg_map(), weights=dg.rhs(O.FN_SINE, omega), minlength=oc.n_dofs) * ~oc.constrained()
    op = E.ContinuousLaplaceOperator(E.Mesh(**kw), k)
    mg = E.MultigridPreconditioner(op, mg_precision=mg_prec)
    info = mg.info()
    assert not any(l["dg"] for l in info["levels"]) and info["levels"][-1]["degree"] == k
    x = op.initialize_dof_vector()
    its = E.KrylovSolver(op, mg).solve(x, to_dev(torch, b))
    omg = oc.multigrid(mg_float=1 if mg_prec == E.PREC_F32 else 0)
    xo, ro = oc.solve(b, mg=omg, rel_tol=1e-10)
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    assert rel(x.cpu().numpy(), xo) <= 1e-8

