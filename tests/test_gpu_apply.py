"""GPU parity of the SIPG operator apply against the oracle (C ABI through exadg_gb300).

Tolerances: FP64 and FP64-emulated (FP32-pair) arithmetic <= 1e-12 relative L2, FP32 <= 1e-5."""
import numpy as np
import pytest

import exadg_gb300 as E
import oracle as O
from tests.gpu_common import pair, rel, require_gpu, to_dev
from tests.helpers import mesh_kwargs, splitmix_uniform

pytestmark = pytest.mark.gpu

KINDS = ["dirichlet", "mixed", "periodic", "partial_periodic", "anisotropic"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6, 7, 8])
def test_apply_f64(kind, k):
    torch = require_gpu()
    p, m, op = pair(kind, 3, k)
    x = splitmix_uniform(p.n_dofs, 1)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x))
    assert rel(y.cpu().numpy(), p.apply(x)) <= 1e-12


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("k", [1, 2, 4, 5, 8])
def test_apply_f64_emulated(kind, k):
    torch = require_gpu()
    p, m, op = pair(kind, 3, k, E.PREC_F64E)
    x = splitmix_uniform(p.n_dofs, 2)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x))
    assert rel(y.cpu().numpy(), p.apply(x)) <= 1e-12


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("k", [1, 3, 4, 6, 8])
def test_apply_f32(kind, k):
    torch = require_gpu()
    p, m, op = pair(kind, 3, k, E.PREC_F32)
    x = splitmix_uniform(p.n_dofs, 3).astype(np.float32)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x, torch.float32))
    assert rel(y.cpu().numpy(), p.apply(x.astype(np.float64))) <= 1e-5


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F64E])
@pytest.mark.parametrize("kind", ["mixed", "periodic", "curved"])
@pytest.mark.parametrize("k", [2, 5])
def test_residual_fused(prec, kind, k):
    """r = b - A x from the operator's fused store against the oracle's A x."""
    torch = require_gpu()
    p, m, op = pair(kind, 3, k, prec)
    x = splitmix_uniform(p.n_dofs, 11)
    b = splitmix_uniform(p.n_dofs, 12)
    r = op.residual(op.initialize_dof_vector(), to_dev(torch, b), to_dev(torch, x))
    ref = b - p.apply(x)
    assert rel(r.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32, E.PREC_F64E])
@pytest.mark.parametrize("k", [2, 4])
def test_apply_multi_rhs(prec, k):
    torch = require_gpu()
    p, m, op = pair("mixed", 3, k, prec)
    dt = torch.float32 if prec == E.PREC_F32 else torch.float64
    X = np.stack([splitmix_uniform(p.n_dofs, s) for s in (1, 2, 3, 4)])
    Xd = to_dev(torch, X, dt)
    Y = op.vmult(op.initialize_dof_vector(4), Xd, n_rhs=4)
    for r in range(4):
        y1 = op.vmult(op.initialize_dof_vector(), Xd[r].contiguous())
        assert torch.equal(Y[r], y1)
        tol = 1e-5 if prec == E.PREC_F32 else 1e-12
        assert rel(Y[r].cpu().numpy(), p.apply(X[r].astype(np.float32 if prec == E.PREC_F32 else np.float64).astype(np.float64))) <= tol


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 8])
@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32, E.PREC_F64E])
def test_apply_curved(k, prec):
    torch = require_gpu()
    p, m, op = pair("curved", 3, k, prec)
    assert not op.cartesian
    dt = torch.float32 if prec == E.PREC_F32 else torch.float64
    x = splitmix_uniform(p.n_dofs, 5)
    if prec == E.PREC_F32:
        x = x.astype(np.float32).astype(np.float64)
    y = op.vmult(op.initialize_dof_vector(), to_dev(torch, x, dt))
    assert rel(y.cpu().numpy(), p.apply(x)) <= (1e-5 if prec == E.PREC_F32 else 1e-12)


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F64E])
@pytest.mark.parametrize("kind", ["mixed", "periodic", "curved", "anisotropic"])
@pytest.mark.parametrize("k", [1, 3, 5])
def test_inverse_diagonal(kind, k, prec):
    torch = require_gpu()
    p, m, op = pair(kind, 3, k, prec)
    d = op.calculate_inverse_diagonal(op.initialize_dof_vector())
    ref = 1.0 / p.diagonal()
    assert rel(d.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("k", [1, 3, 4])
def test_rhs_sine(curved, k):
    torch = require_gpu()
    p, m, op = pair("curved" if curved else "mixed", 3, k)
    cx, fx = op.quadrature_points()
    w = 3 * np.pi

    def u(x):
        return torch.sin(w * x[:, 0]) * torch.sin(w * x[:, 1]) * torch.sin(w * x[:, 2])

    f = 3 * w * w * u(cx)
    g = u(fx)
    h = w * torch.cos(w * fx[:, 0]) * torch.sin(w * fx[:, 1]) * torch.sin(w * fx[:, 2])
    b = op.rhs(f.contiguous(), g.contiguous(), h.contiguous())
    ref = p.rhs(O.FN_SINE, w)
    assert rel(b.cpu().numpy(), ref) <= 1e-12


def test_apply_large_mesh_properties():
    # full-size property checks (k = 4, 64^3 would need the full oracle): linearity and symmetry
    torch = require_gpu()
    m = E.Mesh(24)
    op = E.LaplaceOperator(m, 4)
    a = to_dev(torch, splitmix_uniform(op.n_dofs, 11))
    b = to_dev(torch, splitmix_uniform(op.n_dofs, 12))
    Aa = op.vmult(op.initialize_dof_vector(), a)
    Ab = op.vmult(op.initialize_dof_vector(), b)
    Aab = op.vmult(op.initialize_dof_vector(), (2.0 * a + b).contiguous())
    assert torch.linalg.norm(Aab - 2.0 * Aa - Ab) <= 1e-12 * torch.linalg.norm(Aab)
    assert abs(float(a @ Ab - b @ Aa)) <= 1e-12 * float(torch.linalg.norm(a) * torch.linalg.norm(Ab))
    assert float(a @ Aa) > 0


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32, E.PREC_F64E])
@pytest.mark.parametrize("kind", ["mixed", "periodic", "partial_periodic", "anisotropic"])
@pytest.mark.parametrize("k", [1, 2, 4, 7, 8])
def test_apply_every_launch_variant(prec, kind, k):
    """Every launch variant the autotuner can pick (cells in a row, bricks with shared-memory halo;
    partial bricks and periodic wrap inside a brick included) gives the oracle's result."""
    torch = require_gpu()
    p, m, op = pair(kind, 3, k, prec)
    dt = torch.float32 if prec == E.PREC_F32 else torch.float64
    x = splitmix_uniform(p.n_dofs, 9)
    if prec == E.PREC_F32:
        x = x.astype(np.float32).astype(np.float64)
    ref = p.apply(x)
    xd = to_dev(torch, x, dt)
    best, timings = op.tune()
    variants = [v for v, _ in timings]
    assert len(variants) >= 5 and best in variants
    for v in variants:
        op.set_launch_config(v)
        y = op.vmult(op.initialize_dof_vector(), xd)
        assert rel(y.cpu().numpy(), ref) <= (1e-5 if prec == E.PREC_F32 else 1e-12), v


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F64E])
@pytest.mark.parametrize("kind", ["dirichlet", "periodic", "curved"])
@pytest.mark.parametrize("slabs", [1, 3, 7])
def test_apply_host_vectors(prec, kind, slabs):
    """Host-vector apply with copies pipelined by z-slabs (incl. periodic z and more slabs than
    planes) against the oracle, and equal to the device apply bit for bit."""
    torch = require_gpu()
    p, m, op = pair(kind, 5, 3, prec)
    x = splitmix_uniform(p.n_dofs, 21)
    xh = torch.tensor(x).pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    op.vmult_host(yh, xh, n_slabs=slabs)
    torch.cuda.synchronize()
    assert rel(yh.numpy(), p.apply(x)) <= 1e-12
    yd = op.vmult(op.initialize_dof_vector(), to_dev(torch, x))
    assert torch.equal(yd.cpu(), yh)


TINY = [dict(n_cells=(1, 1, 1)), dict(n_cells=(1, 1, 1), periodic=(1, 1, 1)),
        dict(n_cells=(1, 3, 2), periodic=(1, 0, 1), bc=(0, 0, 1, 0, 0, 0)), dict(n_cells=(5, 1, 1), periodic=(0, 1, 0)),
        dict(n_cells=(2, 1, 3), bc=(1, 0, 0, 1, 0, 0)),
        dict(n_cells=(1, 2, 1), deform_amp=0.1, deform_freq=1, mapping_degree=2)]


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32, E.PREC_F64E])
@pytest.mark.parametrize("mesh", range(len(TINY)))
@pytest.mark.parametrize("k", [1, 3])
def test_apply_tiny_and_ragged_meshes(prec, mesh, k):
    """Single-cell and one-cell-thick meshes (a periodic direction of one cell is its own
    neighbour), blocks larger than the mesh, every launch variant, the host-vector apply."""
    torch = require_gpu()
    kw = TINY[mesh]
    p = O.Problem(O.mesh_desc(**kw), k)
    op = E.LaplaceOperator(E.Mesh(**kw), k, 1.0, prec)
    dt = torch.float32 if prec == E.PREC_F32 else torch.float64
    x = splitmix_uniform(p.n_dofs, 5)
    if prec == E.PREC_F32:
        x = x.astype(np.float32).astype(np.float64)
    ref = p.apply(x)
    tol = 1e-5 if prec == E.PREC_F32 else 1e-12
    xd = to_dev(torch, x, dt)
    variants = [v for v, _ in op.tune()[1]] if op.cartesian else [0]
    for v in variants:
        if op.cartesian:
            op.set_launch_config(v)
        y = op.vmult(op.initialize_dof_vector(), xd)
        assert rel(y.cpu().numpy(), ref) <= tol, v
    if prec != E.PREC_F32:
        xh = torch.tensor(x).pin_memory()
        yh = torch.empty_like(xh).pin_memory()
        op.vmult_host(yh, xh, n_slabs=4)
        torch.cuda.synchronize()
        assert rel(yh.numpy(), ref) <= tol


@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32, E.PREC_F64E])
@pytest.mark.parametrize("kind", ["mixed", "periodic", "curved"])
@pytest.mark.parametrize("k", [1, 4])
def test_every_dof_written_once_and_deterministic(prec, kind, k):
    """Element-centric kernels write each DoF from exactly one thread: a destination pre-filled
    with NaN is fully overwritten by every launch variant (and by the host-vector slabs), and
    repeated applies are bitwise identical (no write races, no atomics)."""
    torch = require_gpu()
    p, m, op = pair(kind, 5, k, prec)
    dt = torch.float32 if prec == E.PREC_F32 else torch.float64
    x = to_dev(torch, splitmix_uniform(p.n_dofs, 13), dt)
    variants = [v for v, _ in op.tune()[1]] if op.cartesian else [0]
    first = None
    for v in variants:
        if op.cartesian:
            op.set_launch_config(v)
        outs = []
        for _ in range(2):
            y = torch.full_like(x, float("nan"))
            op.vmult(y, x)
            assert not torch.isnan(y).any(), v
            outs.append(y)
        assert torch.equal(outs[0], outs[1]), v
        first = outs[0] if first is None else first
    if prec != E.PREC_F32:
        xh = x.cpu().pin_memory()
        yh = torch.full_like(xh, float("nan")).pin_memory()
        op.vmult_host(yh, xh, n_slabs=3)
        torch.cuda.synchronize()
        assert not torch.isnan(yh).any()


@pytest.mark.parametrize("kind", ["dirichlet", "mixed", "periodic", "partial_periodic", "anisotropic"])
@pytest.mark.parametrize("k", [1, 2, 3, 5, 8])
@pytest.mark.parametrize("prec", [E.PREC_F64, E.PREC_F32])
def test_block_jacobi_matches_oracle(kind, k, prec):
    """Fast-diagonalisation block inverse against the oracle's densely inverted cell blocks."""
    torch = require_gpu()
    kw = mesh_kwargs(kind, 2 if k >= 5 else 3)
    p = O.Problem(O.mesh_desc(**kw), k)
    op = E.LaplaceOperator(E.Mesh(**kw), k, 1.0, prec)
    r = splitmix_uniform(p.n_dofs, 13)
    z = op.apply_inverse_block_diagonal(op.initialize_dof_vector(), to_dev(torch, r, op.dtype)).cpu().numpy()
    assert rel(z, p.block_jacobi(r)) <= (1e-10 if prec == E.PREC_F64 else 1e-4)


@pytest.mark.parametrize("device_loop", [True, False])
def test_cg_block_jacobi_iterations(device_loop):
    torch = require_gpu()
    kw = dict(n_cells=(8, 8, 8))
    p = O.Problem(O.mesh_desc(**kw), 3)
    op = E.LaplaceOperator(E.Mesh(**kw), 3)
    b = p.rhs(O.FN_SINE, np.pi)
    xo, ro = p.solve(b, precond=3)
    x = op.initialize_dof_vector()
    its = E.KrylovSolver(op, None, precond=E.KrylovSolver.BLOCK_JACOBI, device_loop=device_loop).solve(
        x, to_dev(torch, b))
    assert abs(its - ro.iterations) <= 1, (its, ro.iterations)
    assert rel(x.cpu().numpy(), xo) <= 1e-8


def test_block_jacobi_rejects_curved_and_single_periodic_cell():
    torch = require_gpu()
    for kw in (mesh_kwargs("curved", 2), dict(n_cells=(1, 3, 3), periodic=(1, 0, 0))):
        op = E.LaplaceOperator(E.Mesh(**kw), 2)
        with pytest.raises(E.ExgError):
            op.apply_inverse_block_diagonal(op.initialize_dof_vector(), op.initialize_dof_vector())
    del torch
