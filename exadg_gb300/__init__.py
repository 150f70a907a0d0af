"""exadg_gb300 -- GB300-native matrix-free SIPG Laplace operator, multigrid and CG.

Python mirror of ExaDG's Poisson interfaces on top of the C ABI in ``include/exadg_gb300.h``
(``exadg_gb300/_lib/libexadg_gb300.so``).  Device vectors are torch CUDA tensors; torch is used
only for device memory and streams.  There is no CPU fallback: without the compiled library or a
GPU the classes raise.

Reference interfaces mirrored (paths relative to the ExaDG tree):
  LaplaceOperator.vmult / calculate_inverse_diagonal / rhs
      poisson/spatial_discretization/laplace_operator.h:228-350, operators/operator_base.h:175-213
  MultigridPreconditioner.vmult / update
      poisson/preconditioners/multigrid_preconditioner.cpp:37-149,
      solvers_and_preconditioners/preconditioners/preconditioner_base.h:33-67
  KrylovSolver.solve
      solvers_and_preconditioners/solvers/iterative_solvers_dealii_wrapper.h:136-221
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libexadg_gb300.so")

EXG_OK = 0
EXG_ERR_INVALID = 1
EXG_ERR_CUDA = 2
EXG_ERR_NOT_CONVERGED = 3
EXG_ERR_NONFINITE = 4
EXG_ERR_UNSUPPORTED = 5
EXG_ERR_NEEDS_UPDATE = 6

PREC_F64 = 0
PREC_F32 = 1
PREC_F64E = 2
MG_PH = 0  # phMG: DG on every level
MG_CPH = 1  # cphMG: continuous levels below the finest DG level

BC_DIRICHLET = 0
BC_NEUMANN = 1


class ExgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("exadg_gb300 status %d: %s" % (status, msg))
        self.status = status


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


class MGDesc(ctypes.Structure):
    _fields_ = [
        ("mg_precision", ctypes.c_int),
        ("cheb_degree", ctypes.c_int),
        ("smoothing_range", ctypes.c_double),
        ("eig_iters", ctypes.c_int),
        ("coarse_rel_tol", ctypes.c_double),
        ("coarse_abs_tol", ctypes.c_double),
        ("coarse_max_iter", ctypes.c_int),
        ("coarse_double", ctypes.c_int),
        ("min_coarse_cells", ctypes.c_int),
        ("singular", ctypes.c_int),
        ("use_graph", ctypes.c_int),
        ("fuse_smoother", ctypes.c_int),
        ("mg_type", ctypes.c_int),
        ("smoother_preconditioner", ctypes.c_int),
    ]


class MGInfo(ctypes.Structure):
    _fields_ = [
        ("n_levels", ctypes.c_int),
        ("degree", ctypes.c_int * 32),
        ("n_cells", (ctypes.c_int * 3) * 32),
        ("lambda_max", ctypes.c_double * 32),
        ("eig_iters", ctypes.c_int * 32),
        ("coarse_iterations", ctypes.c_longlong),
        ("vcycles", ctypes.c_longlong),
        ("dg", ctypes.c_int * 32),
    ]


class CGDesc(ctypes.Structure):
    _fields_ = [
        ("max_iter", ctypes.c_int),
        ("abs_tol", ctypes.c_double),
        ("rel_tol", ctypes.c_double),
        ("precond", ctypes.c_int),
        ("device_loop", ctypes.c_int),
    ]


class CGResult(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("r0", ctypes.c_double),
        ("rn", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("n10", ctypes.c_double),
        ("seconds", ctypes.c_double),
    ]


# every symbol declared in include/exadg_gb300.h
EXPORTED_SYMBOLS = [
    "exg_mesh_create", "exg_mesh_destroy", "exg_sipg_create", "exg_continuous_create", "exg_sipg_destroy",
    "exg_sipg_n_dofs",
    "exg_sipg_info", "exg_sipg_tune", "exg_sipg_set_launch_config", "exg_sipg_apply_f64", "exg_sipg_apply_f32",
    "exg_sipg_residual_f64", "exg_sipg_apply_host_f64", "exg_sipg_inverse_diagonal_f64",
    "exg_sipg_apply_inverse_block_diagonal_f64", "exg_sipg_apply_inverse_block_diagonal_f32",
    "exg_sipg_inverse_diagonal_f32", "exg_sipg_quadrature_points", "exg_sipg_rhs", "exg_mg_default_desc",
    "exg_mg_create", "exg_mg_destroy", "exg_mg_vmult", "exg_mg_info_get", "exg_mg_level_timings",
    "exg_mg_level_n_dofs", "exg_mg_level_apply", "exg_mg_smooth", "exg_mg_restrict_add", "exg_mg_prolongate_add",
    "exg_mg_coarse_solve", "exg_cg_default_desc", "exg_cg_solve",
    "exg_cg_solve_noalloc", "exg_device_fma_peaks", "exg_status_string", "exg_last_error",
    "exg_cnn_create", "exg_cnn_destroy", "exg_cnn_n_params", "exg_cnn_params", "exg_cnn_forward",
    "exg_cnn_backward", "exg_cnn_train_step", "exg_cnn_adam", "exg_cnn_optimizer_state", "exg_dg_pack", "exg_dg_unpack_add", "exg_dg_pack_diff",
    "exg_dg_features", "exg_dg_ls_step",
]

_lib = None


def load_library(path=LIB_PATH):
    """Load the compiled library (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ExgError(EXG_ERR_INVALID, "compiled library %s not found; run exadg_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I = ctypes.c_int
    D = ctypes.c_double
    LL = ctypes.c_longlong
    PP = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "exg_mesh_create": [ctypes.POINTER(MeshDesc), PP],
        "exg_mesh_destroy": [P],
        "exg_sipg_create": [P, I, D, I, PP],
        "exg_continuous_create": [P, I, I, I, PP],
        "exg_sipg_destroy": [P],
        "exg_sipg_n_dofs": [P, ctypes.POINTER(LL)],
        "exg_sipg_info": [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)],
        "exg_sipg_tune": [P, I, ctypes.POINTER(I), ctypes.POINTER(ctypes.c_float), ctypes.POINTER(I), P],
        "exg_sipg_set_launch_config": [P, I],
        "exg_sipg_apply_f64": [P, P, P, I, P],
        "exg_sipg_apply_f32": [P, P, P, I, P],
        "exg_sipg_residual_f64": [P, P, P, P, P],
        "exg_sipg_apply_inverse_block_diagonal_f64": [P, P, P, P],
        "exg_sipg_apply_inverse_block_diagonal_f32": [P, P, P, P],
        "exg_sipg_apply_host_f64": [P, P, P, I, P],
        "exg_sipg_inverse_diagonal_f64": [P, P, P],
        "exg_sipg_inverse_diagonal_f32": [P, P, P],
        "exg_sipg_quadrature_points": [P, P, P, ctypes.POINTER(LL), ctypes.POINTER(LL), P],
        "exg_sipg_rhs": [P, P, P, P, P, P],
        "exg_mg_default_desc": [ctypes.POINTER(MGDesc)],
        "exg_mg_create": [P, ctypes.POINTER(MGDesc), PP],
        "exg_mg_destroy": [P],
        "exg_mg_vmult": [P, P, P, P],
        "exg_mg_info_get": [P, ctypes.POINTER(MGInfo)],
        "exg_mg_level_timings": [P, P, P, ctypes.POINTER(ctypes.c_float), I, ctypes.POINTER(I), P],
        "exg_mg_level_n_dofs": [P, I, ctypes.POINTER(LL), ctypes.POINTER(I)],
        "exg_mg_level_apply": [P, I, P, P, P],
        "exg_mg_smooth": [P, I, P, P, I, P],
        "exg_mg_restrict_add": [P, I, P, P, P],
        "exg_mg_prolongate_add": [P, I, P, P, P],
        "exg_mg_coarse_solve": [P, P, P, P],
        "exg_cg_default_desc": [ctypes.POINTER(CGDesc)],
        "exg_cg_solve": [P, P, ctypes.POINTER(CGDesc), P, P, ctypes.POINTER(CGResult), P],
        "exg_cg_solve_noalloc": [P, ctypes.POINTER(CGDesc), P, P, ctypes.POINTER(CGResult), P],
        "exg_device_fma_peaks": [ctypes.POINTER(D), ctypes.POINTER(D), P],
        "exg_cnn_create": [ctypes.POINTER(I), I, I, I, ctypes.c_ulonglong, PP],
        "exg_cnn_destroy": [P],
        "exg_cnn_n_params": [P, ctypes.POINTER(LL)],
        "exg_cnn_params": [P, PP, PP],
        "exg_cnn_forward": [P, P, P, P],
        "exg_cnn_backward": [P, P, P, P],
        "exg_cnn_train_step": [P, P, P, ctypes.c_float, ctypes.POINTER(ctypes.c_float), P],
        "exg_cnn_adam": [P, ctypes.c_float, P],
        "exg_cnn_optimizer_state": [P, PP, PP, ctypes.POINTER(ctypes.POINTER(LL))],
        "exg_dg_pack": [P, P, I, I, LL, P, P],
        "exg_dg_unpack_add": [P, P, D, I, LL, P, P],
        "exg_dg_pack_diff": [P, P, D, I, LL, P, P],
        "exg_dg_features": [P, P, P, P, I, LL, D, P, P, P],
        "exg_dg_ls_step": [P, P, P, P, P, P, LL, P, P, P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.exg_status_string.argtypes = [ctypes.c_int]
    L.exg_status_string.restype = ctypes.c_char_p
    L.exg_last_error.argtypes = []
    L.exg_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def _check(status):
    if status != EXG_OK:
        L = load_library()
        raise ExgError(status, L.exg_last_error().decode())


def _ptr(t):
    if t is None:
        return None
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ExgError(EXG_ERR_INVALID, "expected a CUDA tensor")
    if not t.is_contiguous():
        raise ExgError(EXG_ERR_INVALID, "expected a contiguous tensor")
    return ctypes.c_void_p(t.data_ptr())


def _sized(t, n, dtype, what):
    """Rejects tensors the kernels would over-run or misread (size, dtype): raw pointers cross the
    C ABI, so the checks happen here."""
    import torch

    if not isinstance(t, torch.Tensor):
        raise ExgError(EXG_ERR_INVALID, "%s: expected a torch tensor" % what)
    if t.dtype != dtype:
        raise ExgError(EXG_ERR_INVALID, "%s: dtype %s, expected %s" % (what, t.dtype, dtype))
    if t.numel() < n:
        raise ExgError(EXG_ERR_INVALID, "%s: %d entries, expected %d" % (what, t.numel(), n))
    return t


def _host_ptr(t, dtype_name="float64"):
    import torch

    if not isinstance(t, torch.Tensor) or t.is_cuda or not t.is_contiguous() or t.dtype != getattr(torch, dtype_name):
        raise ExgError(EXG_ERR_INVALID, "expected a contiguous host %s tensor" % dtype_name)
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def device_fma_peaks(stream=None):
    """(FP64, FP32) FMA throughput of the current device in TFLOP/s, measured."""
    f64 = ctypes.c_double()
    f32 = ctypes.c_double()
    _check(load_library().exg_device_fma_peaks(ctypes.byref(f64), ctypes.byref(f32), _stream(stream)))
    return f64.value, f32.value


class Mesh:
    """Structured hex mesh of a box (subdivided_hyper_rectangle), optional DeformedCubeManifold."""

    def __init__(self, n_cells, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), periodic=(0, 0, 0), bc=(0,) * 6,
                 deform_amp=0.0, deform_freq=1, deform_left=0.0, deform_right=1.0, mapping_degree=1):
        if isinstance(n_cells, int):
            n_cells = (n_cells,) * 3
        d = MeshDesc()
        d.n_cells[:] = list(n_cells)
        d.lo[:] = list(lo)
        d.hi[:] = list(hi)
        d.periodic[:] = list(periodic)
        d.bc[:] = list(bc)
        d.deform_amp = deform_amp
        d.deform_freq = deform_freq
        d.deform_left = deform_left
        d.deform_right = deform_right
        d.mapping_degree = mapping_degree
        self.desc = d
        self.n_cells = tuple(n_cells)
        h = ctypes.c_void_p()
        _check(load_library().exg_mesh_create(ctypes.byref(d), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.exg_mesh_destroy(self.h)
            self.h = None


class LaplaceOperator:
    """SIPG Laplace operator (Poisson::LaplaceOperator) on FE_DGQ(degree), QGauss(degree+1)."""

    def __init__(self, mesh, degree, ip_factor=1.0, precision=PREC_F64, _continuous_singular=None):
        self.mesh = mesh
        self.degree = degree
        self.precision = precision
        h = ctypes.c_void_p()
        if _continuous_singular is None:
            _check(load_library().exg_sipg_create(mesh.h, degree, ip_factor, precision, ctypes.byref(h)))
        else:
            _check(load_library().exg_continuous_create(mesh.h, degree, precision, int(_continuous_singular),
                                                        ctypes.byref(h)))
        self.h = h
        n = ctypes.c_longlong()
        _check(_lib.exg_sipg_n_dofs(h, ctypes.byref(n)))
        self.n_dofs = n.value
        c = ctypes.c_int()
        _check(_lib.exg_sipg_info(h, None, None, ctypes.byref(c)))
        self.cartesian = bool(c.value)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.exg_sipg_destroy(self.h)
            self.h = None

    @property
    def dtype(self):
        import torch

        return torch.float32 if self.precision == PREC_F32 else torch.float64

    def initialize_dof_vector(self, n_rhs=1):
        import torch

        shape = (self.n_dofs,) if n_rhs == 1 else (n_rhs, self.n_dofs)
        return torch.zeros(shape, dtype=self.dtype, device="cuda")

    def vmult(self, dst, src, n_rhs=1, stream=None):
        """dst = A src (dst overwritten), operator_base.cpp:156-168."""
        f = _lib.exg_sipg_apply_f32 if self.precision == PREC_F32 else _lib.exg_sipg_apply_f64
        n = self.n_dofs * n_rhs
        _check(f(self.h, _ptr(_sized(src, n, self.dtype, "src")), _ptr(_sized(dst, n, self.dtype, "dst")), n_rhs,
                 _stream(stream)))
        return dst

    apply = vmult

    def vmult_host(self, dst_host, src_host, n_slabs=8, stream=None):
        """dst_host = A src_host for FP64 host tensors (pinned for copy/compute overlap); queued on
        `stream`, complete when it synchronises."""
        import torch

        for t, what in ((src_host, "src"), (dst_host, "dst")):
            _sized(t, self.n_dofs, torch.float64, what)
        _check(_lib.exg_sipg_apply_host_f64(self.h, _host_ptr(src_host), _host_ptr(dst_host), n_slabs,
                                            _stream(stream)))
        return dst_host

    def residual(self, r, b, x, stream=None):
        """r = b - A x in one kernel (FP64-storage operators)."""
        import torch

        for t, what in ((r, "r"), (b, "b"), (x, "x")):
            _sized(t, self.n_dofs, torch.float64, what)
        _check(_lib.exg_sipg_residual_f64(self.h, _ptr(b), _ptr(x), _ptr(r), _stream(stream)))
        return r

    def apply_inverse_block_diagonal(self, dst, src, stream=None):
        """dst = blockdiag(A)^-1 src (block Jacobi; Cartesian meshes), in the operator's storage
        precision (FP32 operators: float vectors, else double)."""
        f = (_lib.exg_sipg_apply_inverse_block_diagonal_f32 if self.precision == PREC_F32
             else _lib.exg_sipg_apply_inverse_block_diagonal_f64)
        _check(f(self.h, _ptr(_sized(src, self.n_dofs, self.dtype, "src")),
                 _ptr(_sized(dst, self.n_dofs, self.dtype, "dst")), _stream(stream)))
        return dst

    def calculate_inverse_diagonal(self, diag, stream=None):
        f = _lib.exg_sipg_inverse_diagonal_f32 if self.precision == PREC_F32 else _lib.exg_sipg_inverse_diagonal_f64
        _check(f(self.h, _ptr(_sized(diag, self.n_dofs, self.dtype, "diag")), _stream(stream)))
        return diag

    def tune(self, n_rhs=1, stream=None):
        """Autotune the launch variant (cells per block) for this degree / precision / n_rhs."""
        best = ctypes.c_int()
        buf = (ctypes.c_float * 16)()
        cnt = ctypes.c_int(8)
        _check(_lib.exg_sipg_tune(self.h, n_rhs, ctypes.byref(best), buf, ctypes.byref(cnt), _stream(stream)))
        return best.value, [(int(buf[2 * i]), float(buf[2 * i + 1])) for i in range(min(cnt.value, 8))]

    def set_launch_config(self, cpb):
        _check(_lib.exg_sipg_set_launch_config(self.h, cpb))

    def quadrature_points(self, stream=None):
        """Cell points [n_cells, (k+1)^3, 3] and face points [n_cells, 6, (k+1)^2, 3] (FP64)."""
        import torch

        ncp = ctypes.c_longlong()
        nfp = ctypes.c_longlong()
        _check(_lib.exg_sipg_quadrature_points(self.h, None, None, ctypes.byref(ncp), ctypes.byref(nfp),
                                               _stream(stream)))
        cx = torch.empty((ncp.value, 3), dtype=torch.float64, device="cuda")
        fx = torch.empty((nfp.value, 3), dtype=torch.float64, device="cuda")
        _check(_lib.exg_sipg_quadrature_points(self.h, _ptr(cx), _ptr(fx), ctypes.byref(ncp), ctypes.byref(nfp),
                                               _stream(stream)))
        return cx, fx

    def rhs(self, f_cell=None, g_face=None, h_face=None, stream=None):
        """b = (f, v) - inhomogeneous boundary part, from function values at the quadrature points."""
        import torch

        ncp = ctypes.c_longlong()
        nfp = ctypes.c_longlong()
        _check(_lib.exg_sipg_quadrature_points(self.h, None, None, ctypes.byref(ncp), ctypes.byref(nfp),
                                               _stream(stream)))
        for t, n, what in ((f_cell, ncp.value, "f_cell"), (g_face, nfp.value, "g_face"), (h_face, nfp.value, "h_face")):
            if t is not None:
                _sized(t, n, torch.float64, what)
        b = self.initialize_dof_vector()
        _check(_lib.exg_sipg_rhs(self.h, _ptr(f_cell), _ptr(g_face), _ptr(h_face), _ptr(b), _stream(stream)))
        return b


class ContinuousLaplaceOperator(LaplaceOperator):
    """Continuous Laplace operator on FE_Q(degree), as on the continuous
    levels of cphMG (LaplaceOperator with a continuous DoFHandler): DoFs are the lattice nodes
    (N_d * degree + 1 per direction, N_d * degree when periodic, x fastest); constrained DoFs
    (Dirichlet sides, DoF 0 when singular) keep dst = src."""

    def __init__(self, mesh, degree, precision=PREC_F64, singular=False):
        super().__init__(mesh, degree, 1.0, precision, _continuous_singular=bool(singular))


class MultigridPreconditioner:
    """phMG / cphMG V-cycle preconditioner (MultigridPreconditionerBase::vmult).

    mg_type: MG_PH (DG on every level) or MG_CPH (continuous FE_Q levels below the finest DG
    level, the reference's default for the sine and Taylor-Green applications)."""

    def __init__(self, operator, mg_precision=PREC_F32, cheb_degree=5, smoothing_range=20.0, eig_iters=20,
                 coarse_rel_tol=1e-3, coarse_abs_tol=1e-12, coarse_max_iter=10000, coarse_double=False,
                 min_coarse_cells=2, singular=False, use_graph=True, fuse_smoother=True, mg_type=0,
                 block_jacobi_smoother=False):
        d = MGDesc()
        _check(load_library().exg_mg_default_desc(ctypes.byref(d)))
        d.mg_precision = mg_precision
        d.cheb_degree = cheb_degree
        d.smoothing_range = smoothing_range
        d.eig_iters = eig_iters
        d.coarse_rel_tol = coarse_rel_tol
        d.coarse_abs_tol = coarse_abs_tol
        d.coarse_max_iter = coarse_max_iter
        d.coarse_double = int(coarse_double)
        d.min_coarse_cells = min_coarse_cells
        d.singular = int(singular)
        d.use_graph = int(use_graph)
        d.fuse_smoother = int(fuse_smoother)
        d.mg_type = int(mg_type)
        d.smoother_preconditioner = 1 if block_jacobi_smoother else 0
        self.desc = d
        self.operator = operator
        h = ctypes.c_void_p()
        _check(_lib.exg_mg_create(operator.h, ctypes.byref(d), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.exg_mg_destroy(self.h)
            self.h = None

    def vmult(self, dst, src, stream=None):
        import torch

        n = self.operator.n_dofs
        _check(_lib.exg_mg_vmult(self.h, _ptr(_sized(src, n, torch.float64, "src")),
                                 _ptr(_sized(dst, n, torch.float64, "dst")), _stream(stream)))
        return dst

    def level_timings(self, src, dst=None, stream=None):
        """ms per level (coarse first) of one eagerly run V-cycle on src."""
        import torch

        n = self.operator.n_dofs
        _sized(src, n, torch.float64, "src")
        dst = torch.empty_like(src) if dst is None else _sized(dst, n, torch.float64, "dst")
        buf = (ctypes.c_float * 32)()
        nl = ctypes.c_int()
        _check(_lib.exg_mg_level_timings(self.h, _ptr(src), _ptr(dst), buf, 32, ctypes.byref(nl), _stream(stream)))
        return [float(buf[i]) for i in range(nl.value)]

    # ---- the level objects (SmootherBase, MultigridTransferBase, CoarseGridSolverBase, level vmult)
    @property
    def level_dtype(self):
        import torch

        return torch.float32 if self.desc.mg_precision == PREC_F32 else torch.float64

    def level_n_dofs(self, level):
        n = ctypes.c_longlong()
        dg = ctypes.c_int()
        _check(_lib.exg_mg_level_n_dofs(self.h, level, ctypes.byref(n), ctypes.byref(dg)))
        return n.value

    def _lvec(self, t, level, what):
        return _sized(t, self.level_n_dofs(level), self.level_dtype, what)

    def level_vmult(self, level, dst, src, stream=None):
        _check(_lib.exg_mg_level_apply(self.h, level, _ptr(self._lvec(src, level, "src")),
                                       _ptr(self._lvec(dst, level, "dst")), _stream(stream)))
        return dst

    def smooth(self, level, x, rhs, zero_start, stream=None):
        """Chebyshev smoother of a level: vmult (zero_start) or step (x updated in place)."""
        _check(_lib.exg_mg_smooth(self.h, level, _ptr(self._lvec(rhs, level, "rhs")), _ptr(self._lvec(x, level, "x")),
                                  int(zero_start), _stream(stream)))
        return x

    def restrict_and_add(self, level, coarse, fine, stream=None):
        _check(_lib.exg_mg_restrict_add(self.h, level, _ptr(self._lvec(fine, level, "fine")),
                                        _ptr(self._lvec(coarse, level - 1, "coarse")), _stream(stream)))
        return coarse

    def prolongate_and_add(self, level, fine, coarse, stream=None):
        _check(_lib.exg_mg_prolongate_add(self.h, level, _ptr(self._lvec(coarse, level - 1, "coarse")),
                                          _ptr(self._lvec(fine, level, "fine")), _stream(stream)))
        return fine

    def coarse_solve(self, dst, src, stream=None):
        _check(_lib.exg_mg_coarse_solve(self.h, _ptr(self._lvec(src, 0, "src")), _ptr(self._lvec(dst, 0, "dst")),
                                        _stream(stream)))
        return dst

    def info(self):
        i = MGInfo()
        _check(_lib.exg_mg_info_get(self.h, ctypes.byref(i)))
        return dict(
            n_levels=i.n_levels,
            levels=[dict(degree=i.degree[l], n_cells=tuple(i.n_cells[l]), lambda_max=i.lambda_max[l],
                         eig_iters=i.eig_iters[l], dg=bool(i.dg[l])) for l in range(i.n_levels)],
            coarse_iterations=i.coarse_iterations,
            vcycles=i.vcycles,
        )


class KrylovSolver:
    """PCG (Krylov::KrylovSolver with SolverCG and ReductionControl)."""

    NONE, JACOBI, MULTIGRID, BLOCK_JACOBI = 0, 1, 2, 3

    def __init__(self, operator, preconditioner=None, max_iter=10000, abs_tol=1e-20, rel_tol=1e-10, precond=None,
                 device_loop=True):
        self.operator = operator
        self.preconditioner = preconditioner
        d = CGDesc()
        _check(load_library().exg_cg_default_desc(ctypes.byref(d)))
        d.max_iter = max_iter
        d.abs_tol = abs_tol
        d.rel_tol = rel_tol
        if precond is None:
            precond = self.MULTIGRID if preconditioner is not None else self.NONE
        d.precond = precond
        d.device_loop = int(device_loop)
        self.desc = d
        self.result = None

    def solve(self, dst, rhs, stream=None, raise_on_failure=True):
        """Solve A dst = rhs with dst as the initial guess; returns the iteration count."""
        import torch

        n = self.operator.n_dofs
        _sized(rhs, n, torch.float64, "rhs")
        _sized(dst, n, torch.float64, "dst")
        r = CGResult()
        mg = self.preconditioner.h if self.preconditioner is not None else None
        st = _lib.exg_cg_solve(self.operator.h, mg, ctypes.byref(self.desc), _ptr(rhs), _ptr(dst), ctypes.byref(r),
                               _stream(stream))
        self.result = dict(iterations=r.iterations, converged=bool(r.converged), r0=r.r0, rn=r.rn, rho=r.rho,
                           n10=r.n10, seconds=r.seconds, status=st)
        if st != EXG_OK and raise_on_failure:
            _check(st)
        return r.iterations
