"""CPU tests of the oracle: independent assembled apply, diagonal, symmetry, transfers."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import mesh_kwargs, splitmix_uniform


@pytest.mark.parametrize("kind", ["dirichlet", "mixed", "periodic", "partial_periodic", "anisotropic", "curved"])
@pytest.mark.parametrize("k", [1, 2, 3])
def test_sumfactorized_matches_assembled(kind, k):
    p = O.Problem(O.mesh_desc(**mesh_kwargs(kind, 2)), k)
    x = splitmix_uniform(p.n_dofs, 7)
    y = p.apply(x)
    ya = p.assembled_apply(x)
    assert np.linalg.norm(y - ya) <= 1e-13 * np.linalg.norm(ya)


@pytest.mark.parametrize("kind", ["mixed", "periodic", "curved"])
@pytest.mark.parametrize("k", [1, 2, 4])
def test_diagonal_matches_unit_vectors(kind, k):
    p = O.Problem(O.mesh_desc(**mesh_kwargs(kind, 2)), k)
    d = p.diagonal()
    db = p.diagonal_bruteforce()
    assert np.linalg.norm(d - db) <= 1e-13 * np.linalg.norm(db)


@pytest.mark.parametrize("kind", ["mixed", "curved", "periodic"])
def test_operator_symmetric_positive(kind):
    p = O.Problem(O.mesh_desc(**mesh_kwargs(kind, 3)), 3)
    a = splitmix_uniform(p.n_dofs, 1)
    b = splitmix_uniform(p.n_dofs, 2)
    assert abs(a @ p.apply(b) - b @ p.apply(a)) <= 1e-12 * abs(a @ p.apply(a))
    assert a @ p.apply(a) > 0


def test_penalty_cartesian_values():
    # tau_c = surface/volume with weight 1 on boundary faces: interior 3/h, one boundary face 3.5/h
    p = O.Problem(O.mesh_desc(n_cells=(4, 4, 4)), 2)
    tau = p.penalty().reshape(4, 4, 4)
    h = 0.25
    assert tau[1, 1, 1] == pytest.approx(3.0 / h, rel=1e-14)
    assert tau[1, 1, 0] == pytest.approx(3.5 / h, rel=1e-14)
    assert tau[0, 0, 0] == pytest.approx(4.5 / h, rel=1e-14)


def test_transfer_p_and_h_consistency():
    # prolongation is exact for coarse polynomials; restriction is its transpose
    for kc, kf, Nc, Nf in [(1, 2, (2, 2, 2), (2, 2, 2)), (2, 4, (1, 2, 1), (1, 2, 1)), (3, 3, (1, 1, 2), (2, 2, 4))]:
        nc = int(np.prod(Nc)) * (kc + 1) ** 3
        nf = int(np.prod(Nf)) * (kf + 1) ** 3
        u = splitmix_uniform(nc, 3)
        w = splitmix_uniform(nf, 4)
        Pu = O.transfer(kc, kf, Nc, Nf, u)
        Rw = O.transfer(kc, kf, Nc, Nf, w, restrict=True)
        assert abs(w @ Pu - u @ Rw) <= 1e-12 * np.linalg.norm(w) * np.linalg.norm(Pu)
    # a constant is prolongated to a constant
    one = np.ones(8 * 8)
    assert np.allclose(O.transfer(1, 1, (2, 2, 2), (4, 4, 4), one), 1.0)


def test_tridiagonal_eigenvalues():
    import ctypes
    rng = np.random.default_rng(0)
    d = rng.uniform(1, 3, 12)
    e = rng.uniform(-0.5, 0.5, 11)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    out = np.empty(12)
    O.lib().orc_tridiag_eigs(12, O._dp(d), O._dp(e), O._dp(out))
    assert np.allclose(out, np.linalg.eigvalsh(T), rtol=1e-12, atol=1e-12)


def test_cg_jacobi_config_1():
    # unit cube, 8^3 cells, k = 3, u = sin(pi x) sin(pi y) sin(pi z): CG + Jacobi to 1e-10
    p = O.Problem(O.mesh_desc(n_cells=8), 3)
    b = p.rhs(O.FN_SINE, np.pi)
    x, r = p.solve(b, precond=1, rel_tol=1e-10, abs_tol=1e-20)
    assert r.converged
    assert p.n_dofs == 32768
    assert p.error(x, O.FN_SINE, np.pi) < 1e-4


def test_mg_preconditioned_cg_converges_fast():
    p = O.Problem(O.mesh_desc(n_cells=8, lo=(-1,) * 3, hi=(1,) * 3, bc=(0, 1, 0, 0, 0, 0)), 4)
    b = p.rhs(O.FN_SINE, 3 * np.pi)
    x, r = p.solve(b, precond=2)
    assert r.converged and r.iterations < 20
    mg = O.Multigrid(p)
    lv = mg.levels()
    assert [l["degree"] for l in lv] == [1, 1, 1, 2, 4]
    assert [l["n_cells"][0] for l in lv] == [2, 4, 8, 8, 8]


@pytest.mark.parametrize("kind", ["mixed", "periodic", "curved"])
def test_block_jacobi_inverts_the_cell_blocks(kind):
    """The oracle's block Jacobi (dense cell-block inverses) undoes the operator's diagonal blocks,
    which are obtained here independently as cell-restricted applies of the full operator."""
    p = O.Problem(O.mesh_desc(**mesh_kwargs(kind, 2)), 2)
    x = splitmix_uniform(p.n_dofs, 3)
    n3 = 27
    bx = np.zeros_like(x)
    for c in range(p.n_dofs // n3):
        v = np.zeros_like(x)
        v[c * n3:(c + 1) * n3] = x[c * n3:(c + 1) * n3]
        bx[c * n3:(c + 1) * n3] = p.apply(v)[c * n3:(c + 1) * n3]
    assert np.linalg.norm(p.block_jacobi(bx) - x) <= 1e-12 * np.linalg.norm(x)


def test_block_jacobi_smoothed_multigrid_converges():
    p = O.Problem(O.mesh_desc(**mesh_kwargs("mixed", 4)), 3)
    b = splitmix_uniform(p.n_dofs, 5)
    x1, r1 = p.solve(b, smoother_block=0, mg_float=0)
    x2, r2 = p.solve(b, smoother_block=1, mg_float=0)
    assert r1.converged and r2.converged and r2.iterations <= r1.iterations + 1
    assert np.linalg.norm(x1 - x2) <= 1e-8 * np.linalg.norm(x1)
