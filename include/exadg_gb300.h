/*
 * exadg_gb300.h -- C ABI of the GB300-native SIPG Laplace operator, multigrid preconditioner and
 * CG solver.
 *
 * Conventions
 *   - Every function returns an exg_status (0 = EXG_OK) and never throws across the ABI.
 *   - Vector pointers are DEVICE pointers owned by the caller; handles are owned by the library.
 *   - Calls are ordered on the given CUDA stream (a cudaStream_t passed as void*, NULL = default
 *     stream).  One handle is used by one host thread at a time.
 *   - DoF ordering: cells lexicographic (x fastest), FE_DGQ(k) nodal values on Gauss-Lobatto
 *     points lexicographic within a cell (x fastest).
 *   - apply/vmult overwrite dst (zero_dst = true); src and dst must not alias.
 *
 * Each entry point names the ExaDG interface it replaces (paths relative to the ExaDG tree).
 */
#ifndef EXADG_GB300_H
#define EXADG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int exg_status;
enum {
  EXG_OK = 0,
  EXG_ERR_INVALID = 1,        /* bad argument (size, degree, pointer, descriptor) */
  EXG_ERR_CUDA = 2,           /* a CUDA call failed */
  EXG_ERR_NOT_CONVERGED = 3,  /* Krylov solver hit max_iter (deal.II SolverControl::NoConvergence) */
  EXG_ERR_NONFINITE = 4,      /* NaN / Inf residual (iterative_solvers_dealii_wrapper.h:210-211) */
  EXG_ERR_UNSUPPORTED = 5,    /* configuration not implemented */
  EXG_ERR_NEEDS_UPDATE = 6    /* preconditioner used before update() (multigrid_preconditioner_base.cpp:678-680) */
};

/* arithmetic of an operator instance */
enum {
  EXG_PREC_F64 = 0,   /* native FP64 */
  EXG_PREC_F32 = 1,   /* FP32 (multigrid levels) */
  EXG_PREC_F64E = 2   /* FP64 storage, FP32-pair ("double-float") arithmetic, ~1e-14 relative */
};

/* boundary types of the six box sides (x-, x+, y-, y+, z-, z+); ignored on periodic directions */
enum { EXG_BC_DIRICHLET = 0, EXG_BC_NEUMANN = 1 };

typedef struct {
  int n_cells[3];       /* cells per direction */
  double lo[3], hi[3];  /* box corners */
  int periodic[3];      /* 1 = periodic in that direction */
  int bc[6];            /* EXG_BC_* per side */
  double deform_amp;    /* DeformedCubeManifold deformation (grid/deformed_cube_manifold.h:47-59); 0 = affine */
  int deform_freq;
  double deform_left, deform_right;
  int mapping_degree;   /* MappingQ degree used for curvilinear meshes */
} exg_mesh_desc;

typedef struct exg_mesh exg_mesh;
typedef struct exg_op exg_op;
typedef struct exg_mg exg_mg;

/* Structured hex triangulation (replaces GridGenerator::subdivided_hyper_rectangle + manifold
 * setup, applications/poisson/sine/application.h:181-300; grid/deformed_cube_manifold.h:127-157). */
exg_status exg_mesh_create(const exg_mesh_desc* desc, exg_mesh** mesh);
exg_status exg_mesh_destroy(exg_mesh* mesh);

/* SIPG Laplace operator on FE_DGQ(degree), QGauss(degree+1)
 * (Poisson::LaplaceOperator::initialize, poisson/spatial_discretization/laplace_operator.cpp:33-51;
 *  penalty IP::calculate_penalty_parameter, operators/interior_penalty_parameter.h:45-97). */
exg_status exg_sipg_create(const exg_mesh* mesh, int degree, double ip_factor, int precision, exg_op** op);
/* Continuous Laplace operator on FE_Q(degree) (Gauss-Lobatto support points), as on the
 * continuous levels of cphMG: cell integrals with QGauss(degree+1), constrained
 * DoFs (Dirichlet sides; DoF 0 when singular != 0) keep dst = src
 * (LaplaceOperator with a continuous DoFHandler, laplace_operator.cpp:387-436;
 *  OperatorBase::apply, operators/operator_base.cpp:264-310; multigrid/constraints.h:130-197).
 * DoFs are the nodes of the lattice of N_d * degree + 1 points per direction (N_d * degree when
 * periodic), x fastest.  precision: EXG_PREC_F64 or EXG_PREC_F32.  The handle works with
 * exg_sipg_apply_f64/_f32, exg_sipg_residual_f64, exg_sipg_inverse_diagonal_f64/_f32,
 * exg_sipg_n_dofs, exg_sipg_destroy and exg_cg_solve (without multigrid). */
exg_status exg_continuous_create(const exg_mesh* mesh, int degree, int precision, int singular, exg_op** op);
exg_status exg_sipg_destroy(exg_op* op);
exg_status exg_sipg_n_dofs(const exg_op* op, long long* n_dofs);
exg_status exg_sipg_info(const exg_op* op, int* degree, int* precision, int* cartesian);

/* dst = A src for n_rhs vectors stored back to back (stride n_dofs)
 * (OperatorBase::vmult / apply, operators/operator_base.cpp:156-168, 264-310;
 *  Poisson::Operator::vmult, poisson/spatial_discretization/operator.cpp:425-430).
 * exg_sipg_apply_f64 runs on EXG_PREC_F64 and EXG_PREC_F64E operators, exg_sipg_apply_f32 on
 * EXG_PREC_F32 operators. */
exg_status exg_sipg_apply_f64(exg_op* op, const double* src, double* dst, int n_rhs, void* stream);
exg_status exg_sipg_apply_f32(exg_op* op, const float* src, float* dst, int n_rhs, void* stream);
/* dst = A src for FP64 HOST vectors (the vectors ExaDG holds): the library copies in, applies and
 * copies back, cutting the mesh into n_slabs slabs of z-planes so that the copies of one slab
 * overlap the apply of its neighbour (three internal streams, ordered after and before `stream`).
 * Returns once the work is queued; the result is in dst_host when `stream` has completed.  Pinned
 * host memory (cudaHostAlloc / cudaHostRegister) is needed for the overlap.  Overlapping calls on
 * the same operator share its device buffers and race.  FP64-storage operators
 * (OperatorBase::vmult on host vectors, operators/operator_base.cpp:156-168). */
exg_status exg_sipg_apply_host_f64(exg_op* op, const double* src_host, double* dst_host, int n_slabs,
                                   void* stream);
/* r = b - A x in one kernel (the residual step of the V-cycle and of its residual check,
 * multigrid/multigrid_algorithm.h:155-160, 215-216); r must not alias x.  FP64 storage operators. */
/* dst = blockdiag(A)^-1 src: the inverse of every cell's diagonal block, cell term plus the cell's
 * own side of its face terms (OperatorBase::apply_inverse_block_diagonal, operator_base.cpp:820-900;
 * the BlockJacobi preconditioner, preconditioners/block_jacobi_preconditioner.h).  Cartesian
 * meshes (at least two cells along a periodic direction); fast diagonalisation of the Kronecker
 * form, exact up to rounding.  Set up on the first call (synchronous), per precision. */
exg_status exg_sipg_apply_inverse_block_diagonal_f64(exg_op* op, const double* src, double* dst, void* stream);
exg_status exg_sipg_apply_inverse_block_diagonal_f32(exg_op* op, const float* src, float* dst, void* stream);

exg_status exg_sipg_residual_f64(exg_op* op, const double* b, const double* x, double* r, void* stream);

/* Autotuner: times the launch variants of the apply kernel (cells per thread block; one thread
 * per line of a cell) for this operator's degree, precision and n_rhs, keeps the fastest and
 * returns it in *launch_config; timings_ms receives (variant, median ms) pairs, *n_timings their
 * count (in: capacity).  No reference counterpart (deal.II picks its vectorisation at compile time,
 * operators/operator_base.h:116-117). */
exg_status exg_sipg_tune(exg_op* op, int n_rhs, int* launch_config, float* timings_ms, int* n_timings,
                         void* stream);
/* select a launch variant explicitly (0 = default) */
exg_status exg_sipg_set_launch_config(exg_op* op, int launch_config);

/* inverse diagonal, |d| <= 1e-10 -> 1
 * (OperatorBase::calculate_inverse_diagonal, operators/operator_base.cpp:251-262;
 *  utilities/invert_diagonal.h:35-46) */
exg_status exg_sipg_inverse_diagonal_f64(exg_op* op, double* d, void* stream);
exg_status exg_sipg_inverse_diagonal_f32(exg_op* op, float* d, void* stream);

/* Quadrature points where the caller evaluates f, g and h for the right-hand side:
 * cell points [n_cells][(k+1)^3][3] and boundary-face points [n_cells][6][(k+1)^2][3]
 * (entries of interior faces are unused). Sizes returned via n_cell_pts / n_face_pts. */
exg_status exg_sipg_quadrature_points(exg_op* op, double* cell_xyz, double* face_xyz,
                                      long long* n_cell_pts, long long* n_face_pts, void* stream);

/* b = (f, v) - (inhomogeneous boundary part): Dirichlet g and Neumann h values at the boundary
 * face points, f at the cell points; any of f/g/h may be NULL (zero)
 * (Poisson::Operator::rhs, operator.cpp:414-423; OperatorBase::rhs_add, operator_base.cpp:515-554;
 *  weak_boundary_conditions.h:34-234; RHSOperator, operators/rhs_operator.h). */
exg_status exg_sipg_rhs(exg_op* op, const double* f_cell, const double* g_face, const double* h_face,
                        double* b, void* stream);

typedef struct {
  int mg_precision;        /* EXG_PREC_F32 (reference default MultigridNumber = float) or EXG_PREC_F64 */
  int cheb_degree;         /* 5 (multigrid_parameters.h:169-217) */
  double smoothing_range;  /* 20 */
  int eig_iters;           /* 20 */
  double coarse_rel_tol;   /* 1e-3 (applications/poisson/sine/application.h:175-177) */
  double coarse_abs_tol;   /* 1e-12 */
  int coarse_max_iter;     /* 10000 */
  int coarse_double;       /* 1: coarse CG in FP64 even when the V-cycle is FP32 */
  int min_coarse_cells;    /* stop h-coarsening at this many cells per direction (2) */
  int singular;            /* subtract the mean in the coarse solve (coarse_grid_solvers.h:161-162) */
  int use_graph;           /* capture the V-cycle as one CUDA graph */
  int fuse_smoother;       /* 1: Chebyshev steps and the level residual are computed in the operator
                            * kernels' store (deal.II's pre/post-loop operations of a Chebyshev
                            * vmult); 0: separate vector kernels.  Both give the same iterates. */
  int mg_type;             /* EXG_MG_PH (0): DG on every level (phMG); EXG_MG_CPH (1): cphMG, a
                            * continuous FE_Q(k) level below the finest DG level and coarsening in
                            * the continuous space (multigrid_preconditioner_base.cpp:188-199;
                            * the default of applications/poisson/sine/application.h:167). */
  int smoother_preconditioner; /* 0: Chebyshev on point Jacobi (PreconditionerSmoother::PointJacobi,
                                * the default); 1: on block Jacobi (::BlockJacobi; DG levels of
                                * Cartesian meshes, phMG) */
} exg_mg_desc;

#define EXG_MG_PH 0
#define EXG_MG_CPH 1

typedef struct {
  int n_levels;
  int degree[32];
  int n_cells[32][3];
  double lambda_max[32];   /* Lanczos estimate before the 1.2 safety factor */
  int eig_iters[32];
  long long coarse_iterations;  /* accumulated coarse CG iterations */
  long long vcycles;
  int dg[32];              /* 1: discontinuous level, 0: continuous level (cphMG) */
} exg_mg_info;

/* phMG or cphMG (Bisect p-sequence) with Chebyshev-Jacobi smoothing and a coarse CG
 * (MultigridPreconditionerBase::initialize/vmult, multigrid/multigrid_preconditioner_base.cpp:55-95,
 *  673-683; MultigridAlgorithm::v_cycle, multigrid/multigrid_algorithm.h:172-240). */
exg_status exg_mg_default_desc(exg_mg_desc* desc);
/* fine: the DG operator (exg_sipg_create), or a continuous operator (exg_continuous_create: the
 * continuous discretization; levels FE_Q(k) -> ... -> FE_Q(1), then h-coarsening in FE_Q(1),
 * mg_type ignored, desc->singular must match the operator's). */
exg_status exg_mg_create(const exg_op* fine, const exg_mg_desc* desc, exg_mg** mg);
exg_status exg_mg_destroy(exg_mg* mg);
exg_status exg_mg_vmult(exg_mg* mg, const double* src, double* dst, void* stream);
exg_status exg_mg_info_get(const exg_mg* mg, exg_mg_info* info);

/* The multigrid's level objects behind the reference's component interfaces.  Level vectors are
 * device arrays in the multigrid precision (float when mg_precision = EXG_PREC_F32, else double);
 * level 0 is the coarsest.  Calls are stream-ordered.
 *   exg_mg_level_n_dofs: size of level l and whether it is a DG level.
 *   exg_mg_level_apply: dst = A_l src (the level operator's vmult, operator_base.cpp:156-168).
 *   exg_mg_smooth: SmootherBase::vmult (zero_start = 1: x = S(rhs) from zero) or ::step
 *     (zero_start = 0: x updated in place) of the Chebyshev smoother of level l >= 1
 *     (multigrid/smoothers/smoother_base.h:28-43, chebyshev_smoother.h:79-210).
 *   exg_mg_restrict_add / exg_mg_prolongate_add: MultigridTransferBase::restrict_and_add
 *     (coarse += R fine) / prolongate_and_add (fine += P coarse) between levels l-1 and l >= 1
 *     (multigrid/transfer_base.h:27-41, transfer.cpp:76-96).
 *   exg_mg_coarse_solve: CoarseGridSolverBase::operator() (coarse_grid_solvers.h:49-59, 157-224):
 *     dst = coarse CG(src), started from the previous coarse solution as in the V-cycle. */
exg_status exg_mg_level_n_dofs(const exg_mg* mg, int level, long long* n_dofs, int* is_dg);
exg_status exg_mg_level_apply(exg_mg* mg, int level, const void* src, void* dst, void* stream);
exg_status exg_mg_smooth(exg_mg* mg, int level, const void* rhs, void* x, int zero_start, void* stream);
exg_status exg_mg_restrict_add(exg_mg* mg, int level, const void* fine, void* coarse, void* stream);
exg_status exg_mg_prolongate_add(exg_mg* mg, int level, const void* coarse, void* fine, void* stream);
exg_status exg_mg_coarse_solve(exg_mg* mg, const void* src, void* dst, void* stream);
/* One V-cycle dst = M src run eagerly with CUDA events around each level's work (smoothing,
 * residual and transfers on the way down and up; level 0 = the coarse solve); ms[l] receives the
 * time of level l, coarse first, for up to `capacity` levels; *n_levels the number of levels.
 * Synchronises `stream`.  The per-level timer of the reference's V-cycle
 * (multigrid/multigrid_algorithm.h:41, 176-237, behind ENABLE_TIMING). */
exg_status exg_mg_level_timings(exg_mg* mg, const double* src, double* dst, float* ms, int capacity,
                                int* n_levels, void* stream);

typedef struct {
  int max_iter;        /* 10000 */
  double abs_tol;      /* 1e-20 */
  double rel_tol;      /* 1e-10 */
  int precond;         /* 0 none, 1 point Jacobi, 2 multigrid (mg handle), 3 block Jacobi
                        * (Cartesian DG operators; exg_sipg_apply_inverse_block_diagonal_f64) */
  int device_loop;     /* 1: the iterations run as one CUDA-graph launch (a WHILE node over the
                        * captured iteration, scalars and stopping test on the device); 0: host
                        * loop reading the reductions each iteration.  Same arithmetic. */
} exg_cg_desc;

typedef struct {
  int iterations;
  int converged;
  double r0, rn;       /* initial / final residual norm */
  double rho, n10;     /* convergence metrics (iterative_solvers_dealii_wrapper.h:63-78) */
  double seconds;      /* wall time of the solve (device-synchronised) */
} exg_cg_result;

/* PCG on A x = b with x as the initial guess (Krylov::KrylovSolver::solve ->
 * dealii::SolverCG + ReductionControl, solvers/iterative_solvers_dealii_wrapper.h:136-221).
 * Returns EXG_ERR_NOT_CONVERGED / EXG_ERR_NONFINITE instead of throwing. */
exg_status exg_cg_default_desc(exg_cg_desc* desc);
exg_status exg_cg_solve(exg_op* op, exg_mg* mg, const exg_cg_desc* desc, const double* b, double* x,
                        exg_cg_result* result, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Learned initial guess for the pressure-Poisson sequence (the extrapolation p0 = sum_i beta_i p^{n-i}
 * of TimeIntBDFDualSplitting::pressure_step, incompressible_navier_stokes/time_integration/
 * time_int_bdf_dual_splitting.cpp:489-498, plus a learned correction).  A cell-patch CNN on the
 * periodic cell grid: 1x1x1 c_in->c_hidden, 3x3x3 c_hidden->c_hidden, 3x3x3 c_hidden->c_out
 * (SiLU between layers) plus a linear 1x1x1 skip c_in->c_out; activations channel-major
 * [C][n_cells] in FP32.  No counterpart in the
 * reference (the learned correction is an addition); the fallback to plain extrapolation is the
 * caller's choice of the guess with the smaller initial residual.
 * ------------------------------------------------------------------------------------------- */
typedef struct exg_cnn exg_cnn;
exg_status exg_cnn_create(const int n_cells[3], int c_in, int c_hidden, int c_out, unsigned long long seed,
                          exg_cnn** cnn);
exg_status exg_cnn_destroy(exg_cnn* cnn);
exg_status exg_cnn_n_params(const exg_cnn* cnn, long long* n_params);
/* device pointers to the parameter vector (W1, b1, W2, b2, W3, b3, W4) and to its gradient */
exg_status exg_cnn_params(exg_cnn* cnn, float** params, float** grads);
exg_status exg_cnn_forward(exg_cnn* cnn, const float* x, float* y, void* stream);
/* gradient of <gy, y(x)> with respect to the parameters, written to the gradient vector */
exg_status exg_cnn_backward(exg_cnn* cnn, const float* x, const float* gy, void* stream);
/* one Adam step on the mean-squared error between y(x) and target; *loss = MSE before the step */
exg_status exg_cnn_train_step(exg_cnn* cnn, const float* x, const float* target, float lr, float* loss,
                              void* stream);
/* one Adam step with the gradient currently held by the network (from exg_cnn_backward) */
exg_status exg_cnn_adam(exg_cnn* cnn, float lr, void* stream);
/* the Adam state for checkpoints: device pointers to the first and second moments (n_params
 * floats each) and a host pointer to the step counter (read / write) */
exg_status exg_cnn_optimizer_state(exg_cnn* cnn, float** m, float** v, long long** step);
/* x[j*dpc + i][c] = vecs[j][c*dpc + i] * inv_scales[j] (vecs, inv_scales: device arrays) */
exg_status exg_dg_pack(const double* const* vecs, const double* inv_scales, int n_vec, int dofs_per_cell,
                       long long n_cells, float* x, void* stream);
/* dst[c*dpc + i] = base[c*dpc + i] + scale * y[i][c] */
exg_status exg_dg_unpack_add(const float* y, const double* base, double scale, int dofs_per_cell,
                             long long n_cells, double* dst, void* stream);
/* Network input of the learned guess, all on the device: the four features
 * f = (p0, p0 - p1, p0 - 2 p1 + p2, r) of the DG vectors p0, p1, p2 (newest first) and r, each
 * divided by a scale, x[j*dpc + i][c] = f_j[c*dpc + i] / scale[j]; scale[j] is the feature's root
 * mean square over the DoFs, except for the second difference when diff_scale > 0 (divided by
 * diff_scale, the scale of the predicted correction, so that the correction can reproduce it
 * exactly).  The 4 scales are written to `rms` (device doubles). */
exg_status exg_dg_features(const double* p0, const double* p1, const double* p2, const double* r,
                           int dofs_per_cell, long long n_cells, double diff_scale, float* x, double* rms,
                           void* stream);
/* Least-squares step along one or two corrections without a host round trip: with r = b - A base,
 * (ce, cf) minimise |r - ce A e - cf A f| (f, Af may be NULL: then cf = 0), x = base + ce e + cf f,
 * stats = {r.Ae, Ae.Ae, r.r, ce, cf, decrease of |r|^2} (6 device doubles).  The residual of x is
 * never larger than r; when the corrections do not reduce it, ce = cf = 0 and x = base (the
 * fallback).  Calls that overlap on the GPU race (shared reduction array); this and
 * exg_dg_features add no counterpart to the reference. */
exg_status exg_dg_ls_step(const double* r, const double* Ae, const double* e, const double* Af, const double* f,
                          const double* base, long long n, double* x, double* stats, void* stream);
/* t[i][c] = (a[c*dpc + i] - b[c*dpc + i]) * inv_scale */
exg_status exg_dg_pack_diff(const double* a, const double* b, double inv_scale, int dofs_per_cell,
                            long long n_cells, float* t, void* stream);

/* The same point-Jacobi / unpreconditioned CG as exg_cg_solve (desc->precond 0 or 1; point Jacobi
 * is refused for a continuous operator on a Cartesian mesh, whose diagonal set-up would allocate),
 * but it allocates nothing: its work vectors live in one statically allocated device array of about
 * 20 MiB that every GPU loading this library holds until the process exits.  For callers that
 * cannot call cudaMalloc / cudaFree while they run (a time loop with other streams in flight --
 * both calls synchronise the device --, a framework whose pool owns the device memory).
 * Limit: n_dofs <= 524288, otherwise EXG_ERR_INVALID.  The first call on a device looks up the
 * array's device address (make that first call before any stream capture).  All calls share the
 * array, so calls that overlap on the GPU race; each call clears what must start at zero.
 * No counterpart in the reference: an addition of this library. */
exg_status exg_cg_solve_noalloc(exg_op* op, const exg_cg_desc* desc, const double* b, double* x,
                                exg_cg_result* result, void* stream);

/* Measured FMA throughput of the current device (TFLOP/s, FMA = 2 flops) for the compute-side
 * roofline of the operator kernels.  No reference counterpart. */
exg_status exg_device_fma_peaks(double* f64_tflops, double* f32_tflops, void* stream);

const char* exg_status_string(exg_status status);
const char* exg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* EXADG_GB300_H */
