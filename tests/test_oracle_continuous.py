"""CPU tests of the oracle's continuous (cphMG) levels: the lattice operator is pinned to the DG
SIPG operator through the Galerkin identity A_CG = P_c^T A_DG P_c on the unconstrained nodes, and
the transfers are checked for exactness on polynomials and for transposition."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import mesh_kwargs, splitmix_uniform

KINDS = ["dirichlet", "mixed", "periodic", "partial_periodic", "anisotropic", "curved"]


def _singular(kind):
    return kind == "periodic"


def _node_coords(mesh, k, n_nodes, d):
    gl, _, _ = O.fe1d(k + 1)
    h = (mesh.hi[d] - mesh.lo[d]) / mesh.n_cells[d]
    g = np.arange(n_nodes)
    e, l = g // k, g % k
    return mesh.lo[d] + (e + gl[l]) * h


def _lattice_shape(mesh, k):
    return tuple(mesh.n_cells[d] * k + (0 if mesh.periodic[d] else 1) for d in range(3))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_galerkin_identity_with_dg_operator(kind, k):
    m = O.mesh_desc(**mesh_kwargs(kind, 2))
    cg = O.ContinuousProblem(m, k, singular=_singular(kind))
    dg = O.Problem(m, k)
    free = ~cg.constrained()
    u = splitmix_uniform(cg.n_dofs, 11) * free
    mp = cg.dg_map()
    y_dg = dg.apply(u[mp])
    galerkin = np.bincount(mp, weights=y_dg, minlength=cg.n_dofs)
    y = cg.apply(u)
    assert np.linalg.norm((y - galerkin)[free]) <= 1e-12 * np.linalg.norm(galerkin[free])
    # identity rows on the constrained nodes, whose src entries are not read by the free rows
    v = splitmix_uniform(cg.n_dofs, 12)
    yv = cg.apply(v)
    assert np.array_equal(yv[~free], v[~free])
    assert np.allclose(yv[free], cg.apply(v * free)[free], rtol=0, atol=1e-12 * np.abs(yv).max())


@pytest.mark.parametrize("kind", ["mixed", "periodic", "partial_periodic", "curved"])
@pytest.mark.parametrize("k", [1, 3])
def test_diagonal_and_symmetry(kind, k):
    m = O.mesh_desc(**mesh_kwargs(kind, 2))
    cg = O.ContinuousProblem(m, k, singular=_singular(kind))
    n = cg.n_dofs
    eye_diag = np.array([cg.apply(np.eye(1, n, i)[0])[i] for i in range(n)])
    assert np.allclose(cg.diagonal(), eye_diag, rtol=1e-13, atol=0)
    a, b = splitmix_uniform(n, 1), splitmix_uniform(n, 2)
    assert abs(a @ cg.apply(b) - b @ cg.apply(a)) <= 1e-12 * abs(a @ cg.apply(a))
    assert a @ cg.apply(a) > 0


def test_single_periodic_cell_diagonal():
    # one periodic cell: a node couples to itself across the wrapped cell ends
    m = O.mesh_desc(n_cells=(1, 3, 2), periodic=(1, 1, 1))
    cg = O.ContinuousProblem(m, 2, singular=True)
    n = cg.n_dofs
    eye_diag = np.array([cg.apply(np.eye(1, n, i)[0])[i] for i in range(n)])
    assert np.allclose(cg.diagonal(), eye_diag, rtol=1e-13, atol=0)


def test_lattice_sizes_and_constraints():
    m = O.mesh_desc(**mesh_kwargs("mixed", 2))  # Neumann at x = +1
    cg = O.ContinuousProblem(m, 2)
    shape = _lattice_shape(m, 2)
    assert cg.n_dofs == np.prod(shape)
    c = cg.constrained().reshape(shape[::-1])  # [z][y][x]
    assert c[:, :, 0].all() and not c[1:-1, 1:-1, -1].any() and c[0].all() and c[-1].all()
    p = O.ContinuousProblem(O.mesh_desc(**mesh_kwargs("periodic", 2)), 3, singular=True)
    cp = p.constrained()
    assert cp[0] and cp.sum() == 1


@pytest.mark.parametrize("case", ["p_dirichlet", "p_neumann", "h_neumann", "h_periodic"])
def test_lattice_transfer_exact_on_polynomials(case):
    if case.startswith("p"):
        bc = (0,) * 6 if case == "p_dirichlet" else (1,) * 6
        m = O.mesh_desc(n_cells=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=bc)
        Nc, kc, kf = (2, 3, 2), 2, 4
    elif case == "h_neumann":
        m = O.mesh_desc(n_cells=(4, 2, 4), lo=(0, 0, 0), hi=(1, 1, 1), bc=(1,) * 6)
        Nc, kc, kf = (2, 1, 2), 1, 1
    else:
        m = O.mesh_desc(n_cells=(4, 4, 2), periodic=(1, 1, 1))
        Nc, kc, kf = (2, 2, 1), 1, 1
    mc = O.mesh_desc(Nc, lo=tuple(m.lo), hi=tuple(m.hi), periodic=tuple(m.periodic), bc=tuple(m.bc))
    if case == "p_dirichlet":
        f = lambda x, y, z: x * (1 - x) * y * (1 - y) * z * (1 - z)  # noqa: E731  (Q2, zero on the boundary)
    elif case == "h_periodic":
        f = lambda x, y, z: 1.0 + 0 * x * y * z  # noqa: E731  (constants are the periodic Q1 polynomials)
    else:
        f = lambda x, y, z: (1 + x) * (2 + y) * (3 - z)  # noqa: E731
    sc, sf = _lattice_shape(mc, kc), _lattice_shape(m, kf)
    xc = np.meshgrid(*[_node_coords(mc, kc, sc[d], d) for d in range(3)], indexing="ij")
    xf = np.meshgrid(*[_node_coords(m, kf, sf[d], d) for d in range(3)], indexing="ij")
    uc = f(*xc).transpose(2, 1, 0).ravel()  # x fastest
    uf = f(*xf).transpose(2, 1, 0).ravel()
    singular = case == "h_periodic"
    Pu = O.lattice_transfer(m, Nc, kc, kf, False, uc, singular=singular)
    free = ~O.ContinuousProblem(m, kf, singular=singular).constrained()
    if singular:
        # the pinned coarse node is read as zero: compare with the prolongated pinned-free function
        uc_pinned = uc.copy()
        uc_pinned[0] = 0.0
        ref = O.lattice_transfer(m, Nc, kc, kf, False, uc_pinned, singular=True)
        assert np.allclose(Pu, ref)
        assert np.allclose(Pu[free & (np.abs(ref - uf) < 1e-12)], uf[free & (np.abs(ref - uf) < 1e-12)])
    else:
        assert np.allclose(Pu[free], uf[free], rtol=0, atol=1e-13)
        assert np.all(Pu[~free] == 0)
    # restriction is the transpose
    w = splitmix_uniform(len(uf), 5)
    Rw = O.lattice_transfer(m, Nc, kc, kf, False, w, restrict=True, singular=singular)
    assert abs(w @ Pu - uc @ Rw) <= 1e-12 * np.linalg.norm(w) * np.linalg.norm(Pu)


@pytest.mark.parametrize("kind", ["mixed", "periodic"])
def test_c_transfer_embeds_continuous_function(kind):
    m = O.mesh_desc(**mesh_kwargs(kind, 2))
    k = 3
    cg = O.ContinuousProblem(m, k, singular=_singular(kind))
    u = splitmix_uniform(cg.n_dofs, 9)
    Pu = O.lattice_transfer(m, tuple(m.n_cells), k, k, True, u, singular=_singular(kind))
    free = ~cg.constrained()
    assert np.array_equal(Pu, (u * free)[cg.dg_map()])
    w = splitmix_uniform(len(Pu), 4)
    Rw = O.lattice_transfer(m, tuple(m.n_cells), k, k, True, w, restrict=True, singular=_singular(kind))
    assert np.allclose(Rw, np.bincount(cg.dg_map(), weights=w, minlength=cg.n_dofs) * free)


def test_cphmg_levels():
    p = O.Problem(O.mesh_desc(n_cells=(8, 8, 8)), 4)
    lv = O.Multigrid(p, mg_type=1).levels()
    got = [(l["n_cells"][0], l["degree"], l["dg"]) for l in lv]
    assert got == [(2, 1, False), (4, 1, False), (8, 1, False), (8, 2, False), (8, 4, False), (8, 4, True)]
    lv1 = O.Multigrid(O.Problem(O.mesh_desc(n_cells=(4, 4, 4)), 1), mg_type=1).levels()
    assert [(l["n_cells"][0], l["degree"], l["dg"]) for l in lv1] == [(2, 1, False), (4, 1, False), (4, 1, True)]


@pytest.mark.parametrize("kind,k", [("mixed", 3), ("periodic", 2), ("dirichlet", 4), ("curved", 3)])
@pytest.mark.parametrize("mg_float", [0, 1])
def test_cphmg_solve_matches_phmg_solution(kind, k, mg_float):
    m = O.mesh_desc(**mesh_kwargs(kind, 4))
    p = O.Problem(m, k)
    b = splitmix_uniform(p.n_dofs, 3)
    singular = _singular(kind)
    if singular:
        b -= b.mean()
    kw = dict(rel_tol=1e-10, singular=int(singular), mg_float=mg_float)
    x1, r1 = p.solve(b, mg_type=0, **kw)
    x2, r2 = p.solve(b, mg_type=1, **kw)
    assert r1.converged and r2.converged
    if singular:
        x1 -= x1.mean()
        x2 -= x2.mean()
    assert np.linalg.norm(x1 - x2) <= 1e-8 * np.linalg.norm(x1)
    assert r2.iterations <= 40


@pytest.mark.parametrize("kind", ["mixed", "curved"])
def test_continuous_discretization_multigrid(kind):
    """CG on FE_Q(k) preconditioned by the continuous multigrid (cphMG's list without the DG top)
    converges to the unpreconditioned CG solution."""
    m = O.mesh_desc(**mesh_kwargs(kind, 4))
    k = 3
    cg = O.ContinuousProblem(m, k)
    b = splitmix_uniform(cg.n_dofs, 17) * ~cg.constrained()
    mg = cg.multigrid(mg_float=0)
    lv = mg.levels()
    assert not any(l["dg"] for l in lv) and lv[-1]["degree"] == k and lv[-2]["degree"] == 1
    x, r = cg.solve(b, mg=mg, rel_tol=1e-12)
    x0, r0 = cg.solve(b, rel_tol=1e-12, max_iter=5000)
    assert r.converged and r0.converged and r.iterations < r0.iterations
    assert np.linalg.norm(x - x0) <= 1e-9 * np.linalg.norm(x0)
