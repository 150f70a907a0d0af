"""Poisson driver on the GPU library: problem set-up, operator throughput and solves.

Mirrors `Poisson::Driver` (poisson/driver.cpp:54-232): `apply_operator` measures DoF/s with the
semantics of `measure_operator_evaluation_time` (operators/throughput_parameters.h:40-87 -- the
minimum over outer repetitions of the average over inner repetitions, repeated until at least
`min_seconds` have passed), here timed with CUDA events on the launch stream; `solve` assembles
the right-hand side from analytic functions evaluated at the quadrature points and runs PCG.
"""
import math
import time

import exadg_gb300 as E


def measure_operator_evaluation_time(evaluate, n_inner=100, n_outer=1, min_seconds=1.0, stream=None):
    """Seconds per operator evaluation (CUDA-event device time)."""
    import torch

    s = stream or torch.cuda.current_stream()
    best = float("inf")
    t_start = time.perf_counter()
    while True:
        for _ in range(n_outer):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(n_inner):
                evaluate()
            e1.record(s)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3 / n_inner)
        if time.perf_counter() - t_start >= min_seconds:
            return best


def sine_functions(omega, neumann_dir=0):
    """u = prod sin(omega x_d), f = 3 omega^2 u, Neumann datum du/dx_dir (sine application,
    applications/poisson/sine/application.h:32-98)."""
    import torch

    def u(x):
        return torch.sin(omega * x[:, 0]) * torch.sin(omega * x[:, 1]) * torch.sin(omega * x[:, 2])

    def f(x):
        return 3.0 * omega * omega * u(x)

    def h(x):
        g = [torch.sin(omega * x[:, d]) for d in range(3)]
        g[neumann_dir] = omega * torch.cos(omega * x[:, neumann_dir])
        return g[0] * g[1] * g[2]

    return u, f, h


def assemble_rhs(op, f=None, g=None, h=None):
    """b from functions of the quadrature points (callables on [n, 3] FP64 tensors)."""
    cx, fx = op.quadrature_points()
    fq = f(cx).contiguous() if f else None
    gq = g(fx).contiguous() if g else None
    hq = h(fx).contiguous() if h else None
    return op.rhs(fq, gq, hq)


class PoissonProblem:
    """Operator + multigrid + CG on one mesh (Poisson::Operator::setup / solve,
    poisson/spatial_discretization/operator.cpp:261-473)."""

    def __init__(self, mesh_kwargs, degree, outer_precision=E.PREC_F64, mg_precision=E.PREC_F32,
                 use_graph=True, coarse_double=False, singular=False, tune=True, ip_factor=1.0, mg_type=E.MG_PH):
        t0 = time.perf_counter()
        self.mesh = E.Mesh(**mesh_kwargs)
        self.op = E.LaplaceOperator(self.mesh, degree, ip_factor, outer_precision)
        self.rhs_op = self.op if outer_precision == E.PREC_F64 else None
        if tune and self.op.cartesian:
            self.op.tune()
        self.mg = E.MultigridPreconditioner(self.op, mg_precision=mg_precision, use_graph=use_graph,
                                            coarse_double=coarse_double, singular=singular, mg_type=mg_type)
        self.setup_seconds = time.perf_counter() - t0
        self.degree = degree
        self.mesh_kwargs = mesh_kwargs
        self.ip_factor = ip_factor

    def rhs_operator(self):
        if self.rhs_op is None:
            self.rhs_op = E.LaplaceOperator(self.mesh, self.degree, self.ip_factor, E.PREC_F64)
        return self.rhs_op

    def solve(self, b, x=None, rel_tol=1e-10, abs_tol=1e-20, max_iter=10000):
        import torch

        if x is None:
            x = self.op.initialize_dof_vector()
        solver = E.KrylovSolver(self.op, self.mg, rel_tol=rel_tol, abs_tol=abs_tol, max_iter=max_iter)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its = solver.solve(x, b)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        r = dict(solver.result)
        r["wall_seconds"] = wall
        r["iterations"] = its
        return x, r


def unit_cube(n, periodic=False):
    if periodic:
        return dict(n_cells=(n, n, n), periodic=(1, 1, 1))
    return dict(n_cells=(n, n, n))


def deformed_unit_cube(n, amp=0.08, freq=2, mapping_degree=None, degree=5):
    return dict(n_cells=(n, n, n), deform_amp=amp, deform_freq=freq, deform_left=0.0, deform_right=1.0,
                mapping_degree=mapping_degree or degree)


def solve_unit_cube_sine(n, degree, outer_precision, mg_precision, curved=False, use_graph=True, rel_tol=1e-10,
                         mg_type=E.MG_PH):
    """-Laplace u = f on [0,1]^3, u = prod sin(pi x_d) (Dirichlet data = u), returns timings."""
    import torch

    kw = deformed_unit_cube(n, degree=degree) if curved else unit_cube(n)
    prob = PoissonProblem(kw, degree, outer_precision, mg_precision, use_graph=use_graph, mg_type=mg_type)
    u, f, _ = sine_functions(math.pi)
    b = assemble_rhs(prob.rhs_operator(), f=f, g=u)
    x, r = prob.solve(b, rel_tol=rel_tol)
    r["setup_seconds"] = prob.setup_seconds
    r["n_dofs"] = prob.op.n_dofs
    info = prob.mg.info()
    r["levels"] = [(l["n_cells"][0], l["degree"], "DG" if l["dg"] else "CG") for l in info["levels"]]
    r["coarse_iterations"] = info["coarse_iterations"]
    del prob
    torch.cuda.synchronize()
    return x, r
