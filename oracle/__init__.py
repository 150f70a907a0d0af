"""CPU oracle for the SIPG Laplace hot path -- TEST INFRASTRUCTURE ONLY.

Python bindings (ctypes) for ``oracle/oracle.cpp``, a CPU restatement of ExaDG's matrix-free
SIPG Laplace operator, its right-hand side, diagonal, Chebyshev/multigrid preconditioner and CG
solver (reference files are cited in the C++ source).  Only ``tests/``, ``__graft_entry__.smoke``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use this module, and only as
the checker or the timed CPU baseline.  The product library (``exadg_gb300``) never imports it.

Parity pin: ``tests/test_oracle_golden.py`` reproduces the relative L2 errors printed by the
reference's sine application tests (Cartesian and curvilinear meshes, k = 1..7).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_SRC = os.path.join(_HERE, "oracle.cpp")

FN_ZERO = 0
FN_SINE = 1


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("n_cells", ctypes.c_int * 3),
        ("lo", ctypes.c_double * 3),
        ("hi", ctypes.c_double * 3),
        ("periodic", ctypes.c_int * 3),
        ("bc", ctypes.c_int * 6),
        ("deform_amp", ctypes.c_double),
        ("deform_freq", ctypes.c_int),
        ("deform_left", ctypes.c_double),
        ("deform_right", ctypes.c_double),
        ("mapping_degree", ctypes.c_int),
    ]


class SolverDesc(ctypes.Structure):
    _fields_ = [
        ("precond", ctypes.c_int),
        ("rel_tol", ctypes.c_double),
        ("abs_tol", ctypes.c_double),
        ("max_iter", ctypes.c_int),
        ("mg_float", ctypes.c_int),
        ("cheb_degree", ctypes.c_int),
        ("smoothing_range", ctypes.c_double),
        ("eig_iters", ctypes.c_int),
        ("coarse_rel_tol", ctypes.c_double),
        ("coarse_abs_tol", ctypes.c_double),
        ("coarse_max_iter", ctypes.c_int),
        ("coarse_double", ctypes.c_int),
        ("min_coarse_cells", ctypes.c_int),
        ("singular", ctypes.c_int),
        ("mg_type", ctypes.c_int),
        ("smoother_block", ctypes.c_int),
    ]


class SolverResult(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("r0", ctypes.c_double),
        ("rn", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("n10", ctypes.c_double),
    ]


def build(force=False):
    """Compile the oracle shared library with g++ (OpenMP)."""
    os.makedirs(_BUILD, exist_ok=True)
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC):
        return _LIB_PATH
    cmd = ["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-o", _LIB_PATH, _SRC]
    subprocess.check_call(cmd)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        F = ctypes.POINTER(ctypes.c_float)
        I = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.c_int, ctypes.c_double]
        L.orc_destroy.argtypes = [P]
        L.orc_n_dofs.restype = ctypes.c_long
        L.orc_n_dofs.argtypes = [P]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_apply_f64.argtypes = [P, D, D]
        L.orc_apply_f32.argtypes = [P, F, F]
        L.orc_penalty.argtypes = [P, D]
        L.orc_diagonal_f64.argtypes = [P, D]
        L.orc_diagonal_f32.argtypes = [P, F]
        L.orc_diagonal_bruteforce.argtypes = [P, D]
        L.orc_assembled_apply.argtypes = [P, D, D]
        L.orc_block_jacobi.argtypes = [P, D, D]
        L.orc_rhs.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, D]
        L.orc_error.restype = ctypes.c_double
        L.orc_error.argtypes = [P, D, ctypes.c_int, ctypes.c_double]
        L.orc_interpolate.argtypes = [P, ctypes.c_int, ctypes.c_double, D]
        L.orc_default_solver_desc.argtypes = [ctypes.POINTER(SolverDesc)]
        L.orc_mg_create.restype = P
        L.orc_mg_create.argtypes = [P, ctypes.POINTER(SolverDesc)]
        L.orc_mg_destroy.argtypes = [P]
        L.orc_mg_vmult.argtypes = [P, D, D]
        L.orc_mg_n_levels.restype = ctypes.c_int
        L.orc_mg_n_levels.argtypes = [P]
        L.orc_mg_level.argtypes = [P, ctypes.c_int, I, I, D, I]
        L.orc_mg_coarse_iterations.restype = ctypes.c_long
        L.orc_mg_coarse_iterations.argtypes = [P]
        L.orc_solve.restype = ctypes.c_int
        L.orc_solve.argtypes = [P, ctypes.POINTER(SolverDesc), D, D, ctypes.POINTER(SolverResult)]
        L.orc_solve_with_mg.restype = ctypes.c_int
        L.orc_solve_with_mg.argtypes = [P, P, ctypes.POINTER(SolverDesc), D, D, ctypes.POINTER(SolverResult)]
        L.orc_chebyshev.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, D, D, D]
        L.orc_transfer.argtypes = [ctypes.c_int, ctypes.c_int, I, I, ctypes.c_int, D, D]
        L.orc_fe1d.argtypes = [ctypes.c_int, D, D, D]
        L.orc_tridiag_eigs.argtypes = [ctypes.c_int, D, D, D]
        L.orc_cg_create.restype = P
        L.orc_cg_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.c_int, ctypes.c_int]
        L.orc_cg_destroy.argtypes = [P]
        L.orc_cg_n_dofs.restype = ctypes.c_long
        L.orc_cg_n_dofs.argtypes = [P]
        L.orc_cg_apply_f64.argtypes = [P, D, D]
        L.orc_cg_apply_f32.argtypes = [P, F, F]
        L.orc_cg_diagonal_f64.argtypes = [P, D]
        L.orc_cg_constrained.argtypes = [P, ctypes.POINTER(ctypes.c_ubyte)]
        L.orc_cg_dg_map.argtypes = [P, ctypes.POINTER(ctypes.c_long)]
        L.orc_lattice_transfer.argtypes = [ctypes.POINTER(MeshDesc), I, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, D, D]
        L.orc_cg_mg_create.restype = P
        L.orc_cg_mg_create.argtypes = [P, ctypes.POINTER(SolverDesc)]
        L.orc_cg_solve.restype = ctypes.c_int
        L.orc_cg_solve.argtypes = [P, P, ctypes.POINTER(SolverDesc), D, D, ctypes.POINTER(SolverResult)]
        L.orc_mg_level_dg.restype = ctypes.c_int
        L.orc_mg_level_dg.argtypes = [P, ctypes.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def mesh_desc(n_cells, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), periodic=(0, 0, 0), bc=(0,) * 6,
              deform_amp=0.0, deform_freq=1, deform_left=0.0, deform_right=1.0, mapping_degree=1):
    if isinstance(n_cells, int):
        n_cells = (n_cells,) * 3
    m = MeshDesc()
    m.n_cells[:] = list(n_cells)
    m.lo[:] = list(lo)
    m.hi[:] = list(hi)
    m.periodic[:] = list(periodic)
    m.bc[:] = list(bc)
    m.deform_amp = deform_amp
    m.deform_freq = deform_freq
    m.deform_left = deform_left
    m.deform_right = deform_right
    m.mapping_degree = mapping_degree
    return m


def solver_desc(**kw):
    d = SolverDesc()
    lib().orc_default_solver_desc(ctypes.byref(d))
    for k, v in kw.items():
        setattr(d, k, v)
    return d


class Problem:
    """SIPG Laplace problem on a structured hex mesh (oracle side)."""

    def __init__(self, mesh, degree, ip_factor=1.0):
        self.mesh = mesh
        self.degree = degree
        self.h = lib().orc_create(ctypes.byref(mesh), degree, ip_factor)
        if not self.h:
            raise RuntimeError("oracle: problem creation failed")
        self.n_dofs = lib().orc_n_dofs(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def apply(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.empty_like(src)
        lib().orc_apply_f64(self.h, _dp(src), _dp(dst))
        return dst

    def apply_f32(self, src):
        src = np.ascontiguousarray(src, dtype=np.float32)
        dst = np.empty_like(src)
        lib().orc_apply_f32(self.h, _fp(src), _fp(dst))
        return dst

    def assembled_apply(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.empty_like(src)
        lib().orc_assembled_apply(self.h, _dp(src), _dp(dst))
        return dst

    def block_jacobi(self, src):
        """dst = blockdiag(A)^-1 src (cell blocks inverted densely)"""
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.empty_like(src)
        lib().orc_block_jacobi(self.h, _dp(src), _dp(dst))
        return dst

    def penalty(self):
        nc = int(np.prod(list(self.mesh.n_cells)))
        out = np.empty(nc)
        lib().orc_penalty(self.h, _dp(out))
        return out

    def diagonal(self):
        out = np.empty(self.n_dofs)
        lib().orc_diagonal_f64(self.h, _dp(out))
        return out

    def diagonal_f32(self):
        out = np.empty(self.n_dofs, dtype=np.float32)
        lib().orc_diagonal_f32(self.h, _fp(out))
        return out

    def diagonal_bruteforce(self):
        out = np.empty(self.n_dofs)
        lib().orc_diagonal_bruteforce(self.h, _dp(out))
        return out

    def rhs(self, fn=FN_SINE, omega=np.pi, with_f=True):
        b = np.empty(self.n_dofs)
        lib().orc_rhs(self.h, fn, omega, 1 if with_f else 0, _dp(b))
        return b

    def error(self, x, fn=FN_SINE, omega=np.pi):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return lib().orc_error(self.h, _dp(x), fn, omega)

    def interpolate(self, fn=FN_SINE, omega=np.pi):
        x = np.empty(self.n_dofs)
        lib().orc_interpolate(self.h, fn, omega, _dp(x))
        return x

    def solve(self, b, x0=None, **kw):
        d = solver_desc(**kw)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n_dofs) if x0 is None else np.array(x0, dtype=np.float64)
        r = SolverResult()
        lib().orc_solve(self.h, ctypes.byref(d), _dp(b), _dp(x), ctypes.byref(r))
        return x, r

    def chebyshev(self, b, x0=None, degree=5, smoothing_range=20.0, eig_iters=20, step=False):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n_dofs) if x0 is None else np.array(x0, dtype=np.float64)
        lam = ctypes.c_double()
        lib().orc_chebyshev(self.h, degree, smoothing_range, eig_iters, 1 if step else 0, _dp(b), _dp(x),
                            ctypes.byref(lam))
        return x, lam.value


class Multigrid:
    """phMG V-cycle preconditioner of the oracle (float or double levels)."""

    def __init__(self, problem, **kw):
        self.problem = problem
        self.desc = solver_desc(**kw)
        self.h = lib().orc_mg_create(problem.h, ctypes.byref(self.desc))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mg_destroy(self.h)
            self.h = None

    def vmult(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.empty_like(src)
        lib().orc_mg_vmult(self.h, _dp(src), _dp(dst))
        return dst

    def levels(self):
        out = []
        for l in range(lib().orc_mg_n_levels(self.h)):
            N = (ctypes.c_int * 3)()
            deg = ctypes.c_int()
            lam = ctypes.c_double()
            its = ctypes.c_int()
            lib().orc_mg_level(self.h, l, N, ctypes.byref(deg), ctypes.byref(lam), ctypes.byref(its))
            out.append(dict(n_cells=tuple(N), degree=deg.value, lambda_max=lam.value, eig_iters=its.value,
                            dg=bool(lib().orc_mg_level_dg(self.h, l))))
        return out

    def coarse_iterations(self):
        return lib().orc_mg_coarse_iterations(self.h)

    def solve(self, b, x0=None, **kw):
        d = solver_desc(**kw)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.problem.n_dofs) if x0 is None else np.array(x0, dtype=np.float64)
        r = SolverResult()
        lib().orc_solve_with_mg(self.problem.h, self.h, ctypes.byref(d), _dp(b), _dp(x), ctypes.byref(r))
        return x, r


def transfer(kc, kf, n_coarse, n_fine, src, restrict=False):
    """DG p- or h-transfer between two levels: prolongate_and_add / restrict_and_add into zeros."""
    Nc = (ctypes.c_int * 3)(*n_coarse)
    Nf = (ctypes.c_int * 3)(*n_fine)
    src = np.ascontiguousarray(src, dtype=np.float64)
    if restrict:
        out = np.zeros(int(np.prod(n_coarse)) * (kc + 1) ** 3)
    else:
        out = np.zeros(int(np.prod(n_fine)) * (kf + 1) ** 3)
    lib().orc_transfer(kc, kf, Nc, Nf, 1 if restrict else 0, _dp(src), _dp(out))
    return out


class ContinuousProblem:
    """Continuous Q_k Laplace operator on the node lattice of a Cartesian mesh (cphMG levels)."""

    def __init__(self, mesh, degree, singular=False):
        self.mesh = mesh
        self.degree = degree
        self.h = lib().orc_cg_create(ctypes.byref(mesh), degree, int(singular))
        self.n_dofs = lib().orc_cg_n_dofs(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cg_destroy(self.h)
            self.h = None

    def apply(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.empty_like(src)
        lib().orc_cg_apply_f64(self.h, _dp(src), _dp(dst))
        return dst

    def apply_f32(self, src):
        src = np.ascontiguousarray(src, dtype=np.float32)
        dst = np.empty_like(src)
        lib().orc_cg_apply_f32(self.h, _fp(src), _fp(dst))
        return dst

    def diagonal(self):
        out = np.empty(self.n_dofs)
        lib().orc_cg_diagonal_f64(self.h, _dp(out))
        return out

    def constrained(self):
        out = np.empty(self.n_dofs, dtype=np.uint8)
        lib().orc_cg_constrained(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
        return out.astype(bool)

    def multigrid(self, **kw):
        """multigrid for the continuous discretization (continuous p- then h-levels)"""
        mg = Multigrid.__new__(Multigrid)
        mg.problem = self
        mg.desc = solver_desc(**kw)
        mg.h = lib().orc_cg_mg_create(self.h, ctypes.byref(mg.desc))
        return mg

    def solve(self, b, mg=None, x0=None, **kw):
        """CG on the continuous operator (preconditioned by `mg` from multigrid(), or none)"""
        d = solver_desc(**kw)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n_dofs) if x0 is None else np.array(x0, dtype=np.float64)
        r = SolverResult()
        lib().orc_cg_solve(self.h, mg.h if mg is not None else None, ctypes.byref(d), _dp(b), _dp(x), ctypes.byref(r))
        return x, r

    def dg_map(self):
        """lattice node of every DG DoF of the same mesh and degree"""
        n = int(np.prod(list(self.mesh.n_cells))) * (self.degree + 1) ** 3
        out = np.empty(n, dtype=np.int64)
        lib().orc_cg_dg_map(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
        return out


def lattice_transfer(mesh, n_coarse, kc, kf, fine_dg, src, restrict=False, singular=False):
    """Transfer between a continuous level (n_coarse cells, degree kc) and the level of ``mesh``
    (degree kf; discontinuous when fine_dg): prolongate_and_add / restrict_and_add into zeros."""
    Nc = (ctypes.c_int * 3)(*n_coarse)
    mc = mesh_desc(tuple(n_coarse), lo=tuple(mesh.lo), hi=tuple(mesh.hi), periodic=tuple(mesh.periodic),
                   bc=tuple(mesh.bc))
    coarse_n = ContinuousProblem(mc, kc, singular).n_dofs
    if fine_dg:
        fine_n = int(np.prod(list(mesh.n_cells))) * (kf + 1) ** 3
    else:
        fine_n = ContinuousProblem(mesh, kf, singular).n_dofs
    src = np.ascontiguousarray(src, dtype=np.float64)
    out = np.zeros(coarse_n if restrict else fine_n)
    lib().orc_lattice_transfer(ctypes.byref(mesh), Nc, kc, kf, int(fine_dg), int(singular), int(restrict),
                               _dp(src), _dp(out))
    return out


def fe1d(n):
    gl = np.empty(n)
    gp = np.empty(n)
    gw = np.empty(n)
    lib().orc_fe1d(n, _dp(gl), _dp(gp), _dp(gw))
    return gl, gp, gw


def set_threads(n):
    lib().orc_set_threads(n)


def max_threads():
    return lib().orc_max_threads()
