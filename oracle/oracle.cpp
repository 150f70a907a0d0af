// ============================================================================================
// oracle/oracle.cpp -- CPU restatement of ExaDG's SIPG Laplace hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests, the smoke check and the
// CPU-baseline leg of bench.py load it to check the CUDA product.  The product library never
// links, loads or calls anything in this directory.
//
// What it restates (reference paths are relative to the ExaDG source tree):
//   * FE_DGQ on Gauss-Lobatto nodes, QGauss(k+1)      operators/finite_element.h:60,
//                                                     operators/quadrature.h:45
//   * MappingQ(m) geometry through a chart manifold   grid/deformed_cube_manifold.h:47-59,127-157
//   * penalty parameter                               operators/interior_penalty_parameter.h:45-127
//   * SIPG cell / face / boundary integrals           poisson/spatial_discretization/
//                                                     laplace_operator.cpp:129-265,
//                                                     laplace_operator.h:128-197,
//                                                     weak_boundary_conditions.h:34-234
//   * operator loops, rhs, diagonal                   operators/operator_base.cpp:264-310,509-554,
//                                                     618-646,1349-1491; utilities/invert_diagonal.h
//   * Jacobi                                          preconditioners/jacobi_preconditioner.h:33-82
//   * Chebyshev smoother (deal.II PreconditionChebyshev, first kind, Lanczos estimate)
//                                                     multigrid/smoothers/chebyshev_smoother.h:79-210
//   * DG p / h transfers (MGTwoLevelTransfer)          multigrid/transfer.cpp:28-96
//   * V-cycle                                         multigrid/multigrid_algorithm.h:87-240
//   * level list (phMG, Bisect)                       multigrid/multigrid_preconditioner_base.cpp:97-323
//   * coarse CG + Jacobi                              multigrid/coarse_grid_solvers.h:157-224
//   * outer CG (deal.II SolverCG + ReductionControl)  solvers/iterative_solvers_dealii_wrapper.h:136-221
//   * relative L2 error with QGauss(k+3)              postprocessor/error_calculation.cpp:38-110
//   * cphMG level list, continuous FE_Q levels and     multigrid/multigrid_preconditioner_base.cpp:
//     their constraints, c/p/h transfers of the        188-199,520-545, multigrid/constraints.h:
//     continuous levels                                130-197, operators/operator_base.cpp:264-310
//   * block Jacobi (dense cell-block inverses) and     operators/operator_base.cpp:820-900,
//     Chebyshev smoothing on it                         multigrid/smoothers/chebyshev_smoother.h
//
// deal.II (>= 9.7, not vendored) supplies FEEvaluation, SolverCG, PreconditionChebyshev and
// MGTwoLevelTransfer; their published algorithms are restated here in plain loops.
//
// Parity pin: the relative L2 errors of the sine application (Cartesian and curvilinear, 8^3
// cells, k = 1..7, applications/poisson/sine/tests/{cartesian,curvilinear}.output) are reproduced
// by tests/test_oracle_golden.py.  An independent assembled-matrix apply cross-checks the
// sum-factorised apply on small meshes.  The continuous operator is pinned to the DG operator by
// the Galerkin identity A_CG = P_c^T A_DG P_c (tests/test_oracle_continuous.py).
//
// Ordering: cells lexicographic (x fastest), DoFs lexicographic within a cell (x fastest).
// ============================================================================================
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// -------------------------------------------------------------------------------------------
// 1D polynomial machinery (standard FE mathematics)
// -------------------------------------------------------------------------------------------
static double legendre(int n, double x, double* dp) {
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (n == 0) {
    if (dp) *dp = 0.0;
    return 1.0;
  }
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    double d2 = d0 + (2.0 * k - 1.0) * p1;
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  if (dp) *dp = d1;
  return p1;
}

// Gauss-Legendre points / weights mapped to [0,1]
static void gauss_rule(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double dp;
      double p = legendre(n, z, &dp);
      double dz = p / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double dp;
    legendre(n, z, &dp);
    double wi = 2.0 / ((1.0 - z * z) * dp * dp);
    // z is the i-th largest root on [-1,1]
    x[n - 1 - i] = 0.5 * (1.0 + z);
    x[i] = 0.5 * (1.0 - z);
    w[n - 1 - i] = 0.5 * wi;
    w[i] = 0.5 * wi;
  }
}

// Gauss-Lobatto points on [0,1]: endpoints plus the roots of P'_{n-1}
static std::vector<double> gauss_lobatto_points(int n) {
  std::vector<double> x(n);
  x[0] = 0.0;
  x[n - 1] = 1.0;
  int k = n - 1;
  for (int i = 1; i <= (n - 1) / 2; ++i) {
    double z = std::cos(M_PI * i / k);  // largest first
    for (int it = 0; it < 100; ++it) {
      // q(z) = P'_k(z); q'(z) = (2 z P'_k - k(k+1) P_k) / (1 - z^2)
      double dp;
      double p = legendre(k, z, &dp);
      double ddp = (2.0 * z * dp - k * (k + 1.0) * p) / (1.0 - z * z);
      double dz = dp / ddp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[n - 1 - i] = 0.5 * (1.0 + z);
    x[i] = 0.5 * (1.0 - z);
  }
  if (n % 2 == 1 && n > 2) x[n / 2] = 0.5;
  return x;
}

static double lagrange(const std::vector<double>& z, int i, double x) {
  double v = 1.0;
  for (size_t j = 0; j < z.size(); ++j)
    if ((int)j != i) v *= (x - z[j]) / (z[i] - z[j]);
  return v;
}

static double lagrange_deriv(const std::vector<double>& z, int i, double x) {
  double s = 0.0;
  for (size_t m = 0; m < z.size(); ++m) {
    if ((int)m == i) continue;
    double t = 1.0 / (z[i] - z[m]);
    for (size_t j = 0; j < z.size(); ++j)
      if ((int)j != i && j != m) t *= (x - z[j]) / (z[i] - z[j]);
    s += t;
  }
  return s;
}

// -------------------------------------------------------------------------------------------
// Mesh description: subdivided box, optional DeformedCubeManifold, per-side boundary types
// -------------------------------------------------------------------------------------------
}  // namespace orc

extern "C" {
typedef struct {
  int n_cells[3];
  double lo[3], hi[3];
  int periodic[3];
  int bc[6];  // per side x-,x+,y-,y+,z-,z+: 0 = Dirichlet, 1 = Neumann (ignored when periodic)
  double deform_amp;  // DeformedCubeManifold deformation (0 = affine box)
  int deform_freq;
  double deform_left, deform_right;
  int mapping_degree;
} orc_mesh_desc;

typedef struct {
  int precond;           // 0 none, 1 point Jacobi, 2 multigrid
  double rel_tol, abs_tol;
  int max_iter;
  int mg_float;          // 1: V-cycle in float (reference default), 0: double
  int cheb_degree;       // 5
  double smoothing_range;  // 20
  int eig_iters;         // 20
  double coarse_rel_tol;   // 1e-3
  double coarse_abs_tol;   // 1e-12
  int coarse_max_iter;     // 10000
  int coarse_double;     // 1: coarse CG in double even when the V-cycle is float
  int min_coarse_cells;  // stop h-coarsening at this many cells per direction (2)
  int singular;          // subtract mean in the coarse solve (pure Neumann / periodic)
  int mg_type;           // 0: phMG (DG on every level), 1: cphMG (continuous levels below the finest)
  int smoother_block;    // Chebyshev preconditioned by block Jacobi (DG levels) instead of point Jacobi
} orc_solver_desc;

typedef struct {
  int iterations;
  int converged;
  double r0, rn, rho, n10;
} orc_solver_result;
}

namespace orc {

struct Mesh {
  orc_mesh_desc d;
  int N[3];
  double h[3];
  long n_cells() const { return (long)N[0] * N[1] * N[2]; }
  bool affine() const { return d.deform_amp == 0.0; }

  // chart coordinates of local reference point xi in cell c
  void chart(const int c[3], const double xi[3], double X[3]) const {
    for (int e = 0; e < 3; ++e) X[e] = d.lo[e] + (c[e] + xi[e]) * h[e];
  }
  // DeformedCubeManifold::push_forward, grid/deformed_cube_manifold.h:47-59
  void push_forward(const double X[3], double x[3]) const {
    double s = d.deform_amp;
    if (s != 0.0)
      for (int e = 0; e < 3; ++e)
        s *= std::sin(d.deform_freq * M_PI * (X[e] - d.deform_left) / (d.deform_right - d.deform_left));
    for (int e = 0; e < 3; ++e) x[e] = X[e] + s;
  }
  long idx(int i, int j, int k) const { return i + (long)N[0] * (j + (long)N[1] * k); }
  void coords(long c, int out[3]) const {
    out[0] = (int)(c % N[0]);
    out[1] = (int)((c / N[0]) % N[1]);
    out[2] = (int)(c / ((long)N[0] * N[1]));
  }
  // neighbour across face f = 2*dir + side; -1 = boundary
  long neighbor(long c, int f) const {
    int ci[3];
    coords(c, ci);
    int e = f / 2, s = f % 2;
    ci[e] += s ? 1 : -1;
    if (ci[e] < 0 || ci[e] >= N[e]) {
      if (!d.periodic[e]) return -1;
      ci[e] = (ci[e] + N[e]) % N[e];
    }
    return idx(ci[0], ci[1], ci[2]);
  }
  bool at_boundary(long c, int f) const { return neighbor(c, f) < 0; }
};

static Mesh make_mesh(const orc_mesh_desc& d) {
  Mesh m;
  m.d = d;
  for (int e = 0; e < 3; ++e) {
    m.N[e] = d.n_cells[e];
    m.h[e] = (d.hi[e] - d.lo[e]) / d.n_cells[e];
  }
  if (d.deform_amp != 0.0)
    for (int e = 0; e < 3; ++e)
      if (d.periodic[e]) throw std::runtime_error("periodic + deformation not supported");
  return m;
}

// -------------------------------------------------------------------------------------------
// Geometry at quadrature points (MappingQ(m) interpolating the manifold at GL support points)
// -------------------------------------------------------------------------------------------
static const int CELL_STRIDE = 13;  // Jinv[9] (Jinv[i][j] = d xi_i / d x_j), JxW, x[3]
static const int FACE_STRIDE = 16;  // Jinv[9], normal[3] (outward from this cell), JxW, x[3]

struct Geometry {
  Mesh mesh;
  int nq;
  bool uniform;  // affine with identical cells -> one copy
  std::vector<double> gq, gw;  // Gauss rule on [0,1]
  std::vector<double> cell;    // [cells][nq^3][CELL_STRIDE]
  std::vector<double> face;    // [cells][6][nq^2][FACE_STRIDE]
  const double* cell_data(long c) const {
    return cell.data() + (uniform ? 0 : c) * (long)nq * nq * nq * CELL_STRIDE;
  }
  const double* face_data(long c, int f) const {
    return face.data() + ((uniform ? 0 : c) * 6 + f) * (long)nq * nq * FACE_STRIDE;
  }
  // physical coordinates of a stored point (uniform meshes store cell 0 only)
  void point(long c, const double* x0, double out[3]) const {
    int ci[3] = {0, 0, 0};
    if (uniform) mesh.coords(c, ci);
    for (int e = 0; e < 3; ++e) out[e] = x0[e] + ci[e] * mesh.h[e];
  }
};

// evaluate x(xi) and J(xi) for one cell from its support points
struct MappingEval {
  int m1;
  std::vector<double> nodes;
  std::vector<double> P;  // [(m+1)^3][3]
  void init(const Mesh& mesh, long c) {
    int deg = mesh.d.mapping_degree;
    if (deg < 1) deg = 1;
    nodes = gauss_lobatto_points(deg + 1);
    m1 = deg + 1;
    P.resize((size_t)m1 * m1 * m1 * 3);
    int ci[3];
    mesh.coords(c, ci);
    for (int k = 0; k < m1; ++k)
      for (int j = 0; j < m1; ++j)
        for (int i = 0; i < m1; ++i) {
          double xi[3] = {nodes[i], nodes[j], nodes[k]}, X[3], x[3];
          mesh.chart(ci, xi, X);
          mesh.push_forward(X, x);
          for (int e = 0; e < 3; ++e) P[((size_t)(k * m1 + j) * m1 + i) * 3 + e] = x[e];
        }
  }
  void eval(const double xi[3], double x[3], double J[3][3]) const {
    double v[3][16], dv[3][16];
    for (int e = 0; e < 3; ++e)
      for (int a = 0; a < m1; ++a) {
        v[e][a] = lagrange(nodes, a, xi[e]);
        dv[e][a] = lagrange_deriv(nodes, a, xi[e]);
      }
    for (int e = 0; e < 3; ++e) {
      x[e] = 0;
      for (int f = 0; f < 3; ++f) J[e][f] = 0;
    }
    for (int k = 0; k < m1; ++k)
      for (int j = 0; j < m1; ++j)
        for (int i = 0; i < m1; ++i) {
          const double* p = &P[((size_t)(k * m1 + j) * m1 + i) * 3];
          double w = v[0][i] * v[1][j] * v[2][k];
          double w0 = dv[0][i] * v[1][j] * v[2][k];
          double w1 = v[0][i] * dv[1][j] * v[2][k];
          double w2 = v[0][i] * v[1][j] * dv[2][k];
          for (int e = 0; e < 3; ++e) {
            x[e] += w * p[e];
            J[e][0] += w0 * p[e];
            J[e][1] += w1 * p[e];
            J[e][2] += w2 * p[e];
          }
        }
  }
};

static double inverse3(const double J[3][3], double Ji[3][3]) {
  double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  double id = 1.0 / det;
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return det;
}

// tangential directions of a face normal to direction d (lower index first)
static inline void tangential(int d, int& t1, int& t2) {
  t1 = d == 0 ? 1 : 0;
  t2 = d == 2 ? 1 : 2;
}

static std::shared_ptr<Geometry> make_geometry(const Mesh& mesh, int nq) {
  auto g = std::make_shared<Geometry>();
  g->mesh = mesh;
  g->nq = nq;
  gauss_rule(nq, g->gq, g->gw);
  g->uniform = mesh.affine();
  long nc = g->uniform ? 1 : mesh.n_cells();
  long nq3 = (long)nq * nq * nq, nq2 = (long)nq * nq;
  g->cell.resize(nc * nq3 * CELL_STRIDE);
  g->face.resize(nc * 6 * nq2 * FACE_STRIDE);
#pragma omp parallel for schedule(dynamic, 16)
  for (long c = 0; c < nc; ++c) {
    MappingEval me;
    me.init(mesh, c);
    for (int q2 = 0; q2 < nq; ++q2)
      for (int q1 = 0; q1 < nq; ++q1)
        for (int q0 = 0; q0 < nq; ++q0) {
          double xi[3] = {g->gq[q0], g->gq[q1], g->gq[q2]}, x[3], J[3][3], Ji[3][3];
          me.eval(xi, x, J);
          double det = inverse3(J, Ji);
          double* p = &g->cell[(c * nq3 + (q2 * nq + q1) * nq + q0) * CELL_STRIDE];
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) p[i * 3 + j] = Ji[i][j];
          p[9] = std::fabs(det) * g->gw[q0] * g->gw[q1] * g->gw[q2];
          for (int e = 0; e < 3; ++e) p[10 + e] = x[e];
        }
    for (int f = 0; f < 6; ++f) {
      int d = f / 2, side = f % 2, t1, t2;
      tangential(d, t1, t2);
      for (int b = 0; b < nq; ++b)
        for (int a = 0; a < nq; ++a) {
          double xi[3];
          xi[d] = side;
          xi[t1] = g->gq[a];
          xi[t2] = g->gq[b];
          double x[3], J[3][3], Ji[3][3];
          me.eval(xi, x, J);
          double det = inverse3(J, Ji);
          // outward normal: n = J^{-T} nhat / |J^{-T} nhat|, nhat = +-e_d
          double sgn = side ? 1.0 : -1.0, n[3], nn = 0;
          for (int j = 0; j < 3; ++j) {
            n[j] = sgn * Ji[d][j];
            nn += n[j] * n[j];
          }
          nn = std::sqrt(nn);
          double* p = &g->face[((c * 6 + f) * nq2 + b * nq + a) * FACE_STRIDE];
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) p[i * 3 + j] = Ji[i][j];
          for (int j = 0; j < 3; ++j) p[9 + j] = n[j] / nn;
          p[12] = std::fabs(det) * nn * g->gw[a] * g->gw[b];
          for (int e = 0; e < 3; ++e) p[13 + e] = x[e];
        }
    }
  }
  return g;
}

// -------------------------------------------------------------------------------------------
// Tensor contractions along one direction of an (n0 x n1 x n2) array, x fastest.
// out has extent `rows` along `dir`; M is rows x cols (row-major).
// -------------------------------------------------------------------------------------------
template <class T>
static void sweep(const T* M, int rows, int cols, int dir, const int dims[3], const T* in, T* out,
                  bool transpose, bool add) {
  // forward: out[r] = sum_c M[r][c] in[c]; transpose: out[c'] = sum_r M[r][c'] in[r]
  int nin = dims[dir], nout = transpose ? cols : rows;
  int od[3] = {dims[0], dims[1], dims[2]};
  od[dir] = nout;
  long sin = 1, sout = 1;
  for (int e = 0; e < dir; ++e) {
    sin *= dims[e];
    sout *= od[e];
  }
  long outer = 1;
  for (int e = dir + 1; e < 3; ++e) outer *= dims[e];
  long inner = sin;  // == sout
  for (long o = 0; o < outer; ++o)
    for (long i = 0; i < inner; ++i) {
      const T* ip = in + o * sin * nin + i;
      T* op = out + o * sout * nout + i;
      for (int r = 0; r < nout; ++r) {
        T s = 0;
        for (int c = 0; c < nin; ++c) s += (transpose ? M[c * cols + r] : M[r * cols + c]) * ip[c * sin];
        if (add)
          op[r * sout] += s;
        else
          op[r * sout] = s;
      }
    }
}

// -------------------------------------------------------------------------------------------
// Functions for the manufactured problems (sine application, applications/poisson/sine/
// application.h:32-98; the unit-cube variant uses omega = pi)
// -------------------------------------------------------------------------------------------
enum FnKind { FN_ZERO = 0, FN_SINE = 1 };
struct Fn {
  int kind;
  double omega;
  double u(const double* x) const {
    if (kind == FN_ZERO) return 0.0;
    return std::sin(omega * x[0]) * std::sin(omega * x[1]) * std::sin(omega * x[2]);
  }
  double f(const double* x) const { return 3.0 * omega * omega * u(x); }
  // NeumannBoundary of the sine application: d u / d x (the Neumann side is x = +right)
  double neumann(const double* x) const {
    if (kind == FN_ZERO) return 0.0;
    return omega * std::cos(omega * x[0]) * std::sin(omega * x[1]) * std::sin(omega * x[2]);
  }
};

enum OpType { HOMOGENEOUS = 0, INHOMOGENEOUS = 1, FULL = 2 };

// -------------------------------------------------------------------------------------------
// SIPG Laplace operator in precision Number (element-centric evaluation of the reference's
// cell / face / boundary loops; each cell integrates only its own test functions, which is the
// reference's cell-based face-loop variant).
// -------------------------------------------------------------------------------------------
// what the multigrid levels need from an operator: the discontinuous SIPG operator (Laplace)
// and the continuous one (ContinuousLaplace, cphMG levels) both provide it
template <class Number>
struct LevelOp {
  virtual ~LevelOp() {}
  virtual long n_dofs() const = 0;
  virtual void apply(const Number* src, Number* dst) const = 0;
  virtual void diagonal(Number* diag) const = 0;
};

template <class Number>
struct Laplace : LevelOp<Number> {
  std::shared_ptr<Geometry> geo;
  int k, n, nq;
  double ip;
  std::vector<Number> S, D;         // nq x n shape values / gradients at Gauss points
  std::vector<Number> l0, l1, d0, d1;  // basis value / derivative at xi = 0 and 1
  std::vector<Number> tau_cell;     // per cell penalty (surface / volume)
  Number tau_factor;                // (k+1)^2 * IP_factor
  long n_cells() const { return geo->mesh.n_cells(); }
  long n_dofs() const override { return n_cells() * n * n * n; }

  void init(std::shared_ptr<Geometry> g, int degree, double ip_factor) {
    geo = g;
    k = degree;
    n = k + 1;
    nq = g->nq;
    ip = ip_factor;
    std::vector<double> z = gauss_lobatto_points(n);
    S.resize(nq * n);
    D.resize(nq * n);
    for (int q = 0; q < nq; ++q)
      for (int i = 0; i < n; ++i) {
        S[q * n + i] = (Number)lagrange(z, i, g->gq[q]);
        D[q * n + i] = (Number)lagrange_deriv(z, i, g->gq[q]);
      }
    l0.resize(n);
    l1.resize(n);
    d0.resize(n);
    d1.resize(n);
    for (int i = 0; i < n; ++i) {
      l0[i] = (Number)lagrange(z, i, 0.0);
      l1[i] = (Number)lagrange(z, i, 1.0);
      d0[i] = (Number)lagrange_deriv(z, i, 0.0);
      d1[i] = (Number)lagrange_deriv(z, i, 1.0);
    }
    // IP::get_penalty_factor, interior_penalty_parameter.h:110-127 (hypercube)
    tau_factor = (Number)(ip * (k + 1.0) * (k + 1.0));
    compute_penalty();
  }

  // IP::calculate_penalty_parameter, interior_penalty_parameter.h:45-97 (accumulates in Number)
  void compute_penalty() {
    const Mesh& m = geo->mesh;
    long nc = n_cells();
    tau_cell.resize(nc);
    long nq3 = (long)nq * nq * nq, nq2 = (long)nq * nq;
#pragma omp parallel for
    for (long c = 0; c < nc; ++c) {
      const double* cd = geo->cell_data(c);
      Number vol = 0;
      for (long q = 0; q < nq3; ++q) vol += (Number)cd[q * CELL_STRIDE + 9];
      Number surf = 0;
      for (int f = 0; f < 6; ++f) {
        Number factor = m.at_boundary(c, f) ? (Number)1.0 : (Number)0.5;
        const double* fd = geo->face_data(c, f);
        for (long q = 0; q < nq2; ++q) surf += (Number)fd[q * FACE_STRIDE + 12] * factor;
      }
      tau_cell[c] = surf / vol;
    }
  }

  Number face_tau(long c, long nb) const {
    // LaplaceKernel::reinit_face / reinit_boundary_face, laplace_operator.h:128-151
    if (nb < 0) return tau_cell[c] * tau_factor;
    return std::max(tau_cell[c], tau_cell[nb]) * tau_factor;
  }

  // evaluate value and reference gradient at the face q-points of face f of a cell
  void face_eval(const Number* u, int f, Number* val, Number* g0, Number* g1, Number* g2, Number* tmp) const {
    int d = f / 2, side = f % 2, t1, t2;
    tangential(d, t1, t2);
    const Number* lv = side ? l1.data() : l0.data();
    const Number* ld = side ? d1.data() : d0.data();
    // traces on the n x n face grid (t1 fastest)
    Number* tv = tmp;
    Number* tn = tmp + n * n;
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        Number sv = 0, sd = 0;
        for (int i = 0; i < n; ++i) {
          int ix[3];
          ix[d] = i;
          ix[t1] = a;
          ix[t2] = b;
          Number x = u[(ix[2] * n + ix[1]) * n + ix[0]];
          sv += lv[i] * x;
          sd += ld[i] * x;
        }
        tv[b * n + a] = sv;
        tn[b * n + a] = sd;
      }
    Number* w1 = tmp + 2 * n * n;  // nq x n
    Number* gref[3] = {g0, g1, g2};
    int dims[3] = {n, n, 1};
    int dq[3] = {nq, n, 1};
    // value: S x S
    sweep(S.data(), nq, n, 0, dims, tv, w1, false, false);
    sweep(S.data(), nq, n, 1, dq, w1, val, false, false);
    // normal-direction derivative: S x S of tn
    sweep(S.data(), nq, n, 0, dims, tn, w1, false, false);
    sweep(S.data(), nq, n, 1, dq, w1, gref[d], false, false);
    // tangential derivatives
    sweep(D.data(), nq, n, 0, dims, tv, w1, false, false);
    sweep(S.data(), nq, n, 1, dq, w1, gref[t1], false, false);
    sweep(S.data(), nq, n, 0, dims, tv, w1, false, false);
    sweep(D.data(), nq, n, 1, dq, w1, gref[t2], false, false);
  }

  // integrate coefficients (value coefficient cv, reference-gradient coefficients c0,c1,c2 at
  // face q-points) into the cell's n^3 test functions
  void face_integrate(int f, const Number* cv, const Number* c0, const Number* c1, const Number* c2,
                      Number* out, Number* tmp) const {
    int d = f / 2, side = f % 2, t1, t2;
    tangential(d, t1, t2);
    const Number* lv = side ? l1.data() : l0.data();
    const Number* ld = side ? d1.data() : d0.data();
    const Number* cr[3] = {c0, c1, c2};
    Number* tv = tmp;
    Number* tn = tmp + n * n;
    Number* w1 = tmp + 2 * n * n;
    int dq[3] = {nq, nq, 1};
    int dqn[3] = {nq, n, 1};
    // tv = (S x S)^T cv + (D x S)^T c_t1 + (S x D)^T c_t2 ; tn = (S x S)^T c_d
    sweep(S.data(), nq, n, 1, dq, cv, w1, true, false);
    sweep(S.data(), nq, n, 0, dqn, w1, tv, true, false);
    sweep(S.data(), nq, n, 1, dq, cr[t1], w1, true, false);
    sweep(D.data(), nq, n, 0, dqn, w1, tv, true, true);
    sweep(D.data(), nq, n, 1, dq, cr[t2], w1, true, false);
    sweep(S.data(), nq, n, 0, dqn, w1, tv, true, true);
    sweep(S.data(), nq, n, 1, dq, cr[d], w1, true, false);
    sweep(S.data(), nq, n, 0, dqn, w1, tn, true, false);
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a)
        for (int i = 0; i < n; ++i) {
          int ix[3];
          ix[d] = i;
          ix[t1] = a;
          ix[t2] = b;
          out[(ix[2] * n + ix[1]) * n + ix[0]] += lv[i] * tv[b * n + a] + ld[i] * tn[b * n + a];
        }
  }

  // cell integral of LaplaceOperator::do_cell_integral (laplace_operator.cpp:129-137)
  void cell_term(long c, const Number* u, Number* out, Number* buf) const {
    long nq3 = (long)nq * nq * nq;
    Number* g[3] = {buf, buf + nq3, buf + 2 * nq3};
    Number* t1 = buf + 3 * nq3;
    Number* t2 = t1 + nq3;
    int dn[3] = {n, n, n};
    int d1[3] = {nq, n, n};
    int d2[3] = {nq, nq, n};
    for (int e = 0; e < 3; ++e) {
      sweep(e == 0 ? D.data() : S.data(), nq, n, 0, dn, u, t1, false, false);
      sweep(e == 1 ? D.data() : S.data(), nq, n, 1, d1, t1, t2, false, false);
      sweep(e == 2 ? D.data() : S.data(), nq, n, 2, d2, t2, g[e], false, false);
    }
    const double* cd = geo->cell_data(c);
    for (long q = 0; q < nq3; ++q) {
      const double* p = cd + q * CELL_STRIDE;
      Number Ji[9];
      for (int i = 0; i < 9; ++i) Ji[i] = (Number)p[i];
      Number JxW = (Number)p[9];
      Number gr[3] = {g[0][q], g[1][q], g[2][q]}, gp[3];
      for (int j = 0; j < 3; ++j) gp[j] = Ji[0 * 3 + j] * gr[0] + Ji[1 * 3 + j] * gr[1] + Ji[2 * 3 + j] * gr[2];
      // submit_gradient(get_gradient(q)) -> reference coefficients JxW * Jinv * grad
      for (int i = 0; i < 3; ++i) g[i][q] = JxW * (Ji[i * 3 + 0] * gp[0] + Ji[i * 3 + 1] * gp[1] + Ji[i * 3 + 2] * gp[2]);
    }
    int e2[3] = {nq, nq, nq};
    int e1[3] = {nq, nq, n};
    int e0[3] = {nq, n, n};
    for (int e = 0; e < 3; ++e) {
      sweep(e == 2 ? D.data() : S.data(), nq, n, 2, e2, g[e], t2, true, false);
      sweep(e == 1 ? D.data() : S.data(), nq, n, 1, e1, t2, t1, true, false);
      sweep(e == 0 ? D.data() : S.data(), nq, n, 0, e0, t1, out, true, true);
    }
  }

  // face terms of one cell for all six faces (do_face_integral / do_boundary_integral)
  void face_terms(long c, const Number* src, Number* out, Number* buf, int optype, const Fn* bcfn) const {
    const Mesh& m = geo->mesh;
    long nq2 = (long)nq * nq, n3 = (long)n * n * n;
    Number* vo = buf;
    Number* go[3] = {buf + nq2, buf + 2 * nq2, buf + 3 * nq2};
    Number* vn = buf + 4 * nq2;
    Number* gn[3] = {buf + 5 * nq2, buf + 6 * nq2, buf + 7 * nq2};
    Number* cv = buf + 8 * nq2;
    Number* cc[3] = {buf + 9 * nq2, buf + 10 * nq2, buf + 11 * nq2};
    Number* tmp = buf + 12 * nq2;
    const Number* u = src ? src + c * n3 : nullptr;
    for (int f = 0; f < 6; ++f) {
      int d = f / 2, side = f % 2;
      long nb = m.neighbor(c, f);
      if (optype == INHOMOGENEOUS && nb >= 0) continue;
      const double* fo = geo->face_data(c, f);
      if (optype != INHOMOGENEOUS)
        face_eval(u, f, vo, go[0], go[1], go[2], tmp);
      else
        for (long q = 0; q < nq2; ++q) vo[q] = go[0][q] = go[1][q] = go[2][q] = Number(0);
      if (nb >= 0) {
        int fnb = 2 * d + (1 - side);
        const double* fn = geo->face_data(nb, fnb);
        face_eval(src + nb * n3, fnb, vn, gn[0], gn[1], gn[2], tmp);
        Number tau = face_tau(c, nb);
        bool own_minus = side == 1;
        const double* fm = own_minus ? fo : fn;  // the '-' side supplies normal and JxW
        for (long q = 0; q < nq2; ++q) {
          const double* pm = fm + q * FACE_STRIDE;
          const double* po = fo + q * FACE_STRIDE;
          const double* pn = fn + q * FACE_STRIDE;
          Number nrm[3] = {(Number)pm[9], (Number)pm[10], (Number)pm[11]};
          Number JxW = (Number)pm[12];
          Number ndo = 0, ndn = 0;
          for (int j = 0; j < 3; ++j) {
            Number gpo = (Number)po[0 * 3 + j] * go[0][q] + (Number)po[1 * 3 + j] * go[1][q] + (Number)po[2 * 3 + j] * go[2][q];
            Number gpn = (Number)pn[0 * 3 + j] * gn[0][q] + (Number)pn[1 * 3 + j] * gn[1][q] + (Number)pn[2 * 3 + j] * gn[2][q];
            ndo += nrm[j] * gpo;
            ndn += nrm[j] * gpn;
          }
          Number um = own_minus ? vo[q] : vn[q], up = own_minus ? vn[q] : vo[q];
          Number nm = own_minus ? ndo : ndn, np = own_minus ? ndn : ndo;
          // LaplaceKernel::calculate_gradient_flux / calculate_value_flux (laplace_operator.h:180-197)
          Number gflux = Number(-0.5) * (um - up);
          Number vflux = Number(0.5) * (nm + np) - tau * (um - up);
          Number sv = own_minus ? -vflux : vflux;
          // submit_normal_derivative(gflux) with the '-' normal, submit_value(sv)
          cv[q] = JxW * sv;
          for (int i = 0; i < 3; ++i)
            cc[i][q] = JxW * gflux * ((Number)po[i * 3 + 0] * nrm[0] + (Number)po[i * 3 + 1] * nrm[1] + (Number)po[i * 3 + 2] * nrm[2]);
        }
      } else {
        Number tau = face_tau(c, -1);
        int bctype = m.d.bc[f];  // 0 Dirichlet, 1 Neumann
        for (long q = 0; q < nq2; ++q) {
          const double* po = fo + q * FACE_STRIDE;
          Number nrm[3] = {(Number)po[9], (Number)po[10], (Number)po[11]};
          Number JxW = (Number)po[12];
          Number ndo = 0;
          for (int j = 0; j < 3; ++j) {
            Number gpo = (Number)po[0 * 3 + j] * go[0][q] + (Number)po[1 * 3 + j] * go[1][q] + (Number)po[2 * 3 + j] * go[2][q];
            ndo += nrm[j] * gpo;
          }
          // weak_boundary_conditions.h:34-234
          Number um = optype == INHOMOGENEOUS ? Number(0) : vo[q];
          Number nm = optype == INHOMOGENEOUS ? Number(0) : ndo;
          Number up, np;
          if (bctype == 0) {
            double xq[3];
            geo->point(c, po + 13, xq);
            Number gval = (optype == HOMOGENEOUS || !bcfn) ? Number(0) : (Number)bcfn->u(xq);
            up = optype == HOMOGENEOUS ? -um : -um + Number(2) * gval;
            np = nm;
          } else {
            double xq[3];
            geo->point(c, po + 13, xq);
            Number hval = (optype == HOMOGENEOUS || !bcfn) ? Number(0) : (Number)bcfn->neumann(xq);
            up = um;
            np = optype == HOMOGENEOUS ? -nm : -nm + Number(2) * hval;
          }
          Number gflux = Number(-0.5) * (um - up);
          Number vflux = Number(0.5) * (nm + np) - tau * (um - up);
          cv[q] = -JxW * vflux;
          for (int i = 0; i < 3; ++i)
            cc[i][q] = JxW * gflux * ((Number)po[i * 3 + 0] * nrm[0] + (Number)po[i * 3 + 1] * nrm[1] + (Number)po[i * 3 + 2] * nrm[2]);
        }
      }
      face_integrate(f, cv, cc[0], cc[1], cc[2], out, tmp);
    }
  }

  size_t buf_size() const {
    long nq3 = (long)nq * nq * nq, nq2 = (long)nq * nq;
    return (size_t)(5 * nq3 + 12 * nq2 + 2 * n * n + nq * n + 64);
  }

  // OperatorBase::apply (zero_dst = true), operator_base.cpp:264-310
  void apply(const Number* src, Number* dst) const override {
    long nc = n_cells(), n3 = (long)n * n * n;
#pragma omp parallel
    {
      std::vector<Number> buf(buf_size()), out(n3);
#pragma omp for schedule(static)
      for (long c = 0; c < nc; ++c) {
        std::fill(out.begin(), out.end(), Number(0));
        cell_term(c, src + c * n3, out.data(), buf.data());
        face_terms(c, src, out.data(), buf.data(), HOMOGENEOUS, nullptr);
        std::copy(out.begin(), out.end(), dst + c * n3);
      }
    }
  }

  // OperatorBase::rhs + RHSOperator::evaluate_add (operator.cpp:414-423, operator_base.cpp:509-554)
  void rhs(const Fn& fn, bool with_f, Number* b) const {
    long nc = n_cells(), n3 = (long)n * n * n, nq3 = (long)nq * nq * nq;
#pragma omp parallel
    {
      std::vector<Number> buf(buf_size()), tmp(n3), zero(1);
      std::vector<Number> fq(nq3), t1(nq3), t2(nq3);
#pragma omp for schedule(static)
      for (long c = 0; c < nc; ++c) {
        std::fill(tmp.begin(), tmp.end(), Number(0));
        // inhomogeneous boundary part (no gather: values are the boundary data only)
        face_terms(c, nullptr, tmp.data(), buf.data(), INHOMOGENEOUS, &fn);
        Number* bc = b + c * n3;
        for (long i = 0; i < n3; ++i) bc[i] = -tmp[i];
        if (with_f) {
          const double* cd = geo->cell_data(c);
          for (long q = 0; q < nq3; ++q) {
            double xq[3];
            geo->point(c, cd + q * CELL_STRIDE + 10, xq);
            fq[q] = (Number)(fn.f(xq) * cd[q * CELL_STRIDE + 9]);
          }
          int e2[3] = {nq, nq, nq}, e1[3] = {nq, nq, n}, e0[3] = {nq, n, n};
          sweep(S.data(), nq, n, 2, e2, fq.data(), t2.data(), true, false);
          sweep(S.data(), nq, n, 1, e1, t2.data(), t1.data(), true, false);
          sweep(S.data(), nq, n, 0, e0, t1.data(), bc, true, true);
        }
      }
    }
  }

  // diagonal by sum factorisation (cell + own-side face terms), MatrixFreeTools::compute_diagonal
  void diagonal(Number* diag) const override {
    const Mesh& m = geo->mesh;
    long nc = n_cells(), n3 = (long)n * n * n, nq3 = (long)nq * nq * nq, nq2 = (long)nq * nq;
    // elementwise products of the 1D matrices (nq x n)
    std::vector<Number> SS(nq * n), SD(nq * n), DD(nq * n);
    for (int i = 0; i < nq * n; ++i) {
      SS[i] = S[i] * S[i];
      SD[i] = S[i] * D[i];
      DD[i] = D[i] * D[i];
    }
    auto mat = [&](int kk, int ll, int e) -> const Number* {
      bool a = kk == e, b = ll == e;
      return a && b ? DD.data() : (a || b ? SD.data() : SS.data());
    };
#pragma omp parallel
    {
      std::vector<Number> G(nq3), t1(nq3), t2(nq3), out(n3), A(nq2), B(nq2), w1(nq * n), tv(n * n), tn(n * n);
#pragma omp for schedule(static)
      for (long c = 0; c < nc; ++c) {
        std::fill(out.begin(), out.end(), Number(0));
        const double* cd = geo->cell_data(c);
        for (int kk = 0; kk < 3; ++kk)
          for (int ll = 0; ll < 3; ++ll) {
            for (long q = 0; q < nq3; ++q) {
              const double* p = cd + q * CELL_STRIDE;
              Number s = 0;
              for (int j = 0; j < 3; ++j) s += (Number)p[kk * 3 + j] * (Number)p[ll * 3 + j];
              G[q] = s * (Number)p[9];
            }
            int e2[3] = {nq, nq, nq}, e1[3] = {nq, nq, n}, e0[3] = {nq, n, n};
            sweep(mat(kk, ll, 2), nq, n, 2, e2, G.data(), t2.data(), true, false);
            sweep(mat(kk, ll, 1), nq, n, 1, e1, t2.data(), t1.data(), true, false);
            sweep(mat(kk, ll, 0), nq, n, 0, e0, t1.data(), out.data(), true, true);
          }
        for (int f = 0; f < 6; ++f) {
          int d = f / 2, side = f % 2, t1d, t2d;
          tangential(d, t1d, t2d);
          long nb = m.neighbor(c, f);
          int bctype = m.d.bc[f];
          if (nb < 0 && bctype == 1) continue;  // Neumann: no homogeneous contribution
          const double* fo = geo->face_data(c, f);
          const double* fm = fo;
          bool own_minus = true;
          if (nb >= 0 && side == 0) {
            fm = geo->face_data(nb, 2 * d + 1);
            own_minus = false;
          }
          Number tau = face_tau(c, nb);
          // alpha: coefficient of v (n.grad phi), beta: coefficient of v^2, per q
          // interior: s * JxW- * v (n-.grad) + tau JxW- v^2, s = -1 if own is '-' else +1
          // Dirichlet: -2 JxW v (n.grad) + 2 tau JxW v^2
          const Number* lv = side ? l1.data() : l0.data();
          const Number* ld = side ? d1.data() : d0.data();
          for (int comp = 0; comp < 4; ++comp) {
            // comp 0: beta S^2 S^2 (times lv^2); comp 1: alpha c_t1 SD S^2 (lv^2);
            // comp 2: alpha c_t2 S^2 SD (lv^2); comp 3: alpha c_d S^2 S^2 (lv*ld)
            for (long q = 0; q < nq2; ++q) {
              const double* pm = fm + q * FACE_STRIDE;
              const double* po = fo + q * FACE_STRIDE;
              Number nrm[3] = {(Number)pm[9], (Number)pm[10], (Number)pm[11]};
              Number JxW = (Number)pm[12];
              Number alpha, beta;
              if (nb >= 0) {
                alpha = (own_minus ? Number(-1) : Number(1)) * JxW;
                beta = tau * JxW;
              } else {
                alpha = Number(-2) * JxW;
                beta = Number(2) * tau * JxW;
              }
              int dir = comp == 1 ? t1d : (comp == 2 ? t2d : d);
              Number cdir = (Number)po[dir * 3 + 0] * nrm[0] + (Number)po[dir * 3 + 1] * nrm[1] + (Number)po[dir * 3 + 2] * nrm[2];
              A[q] = comp == 0 ? beta : alpha * cdir;
            }
            const Number* m1 = comp == 1 ? SD.data() : SS.data();
            const Number* m2 = comp == 2 ? SD.data() : SS.data();
            int dq[3] = {nq, nq, 1}, dqn[3] = {nq, n, 1};
            sweep(m2, nq, n, 1, dq, A.data(), w1.data(), true, false);
            sweep(m1, nq, n, 0, dqn, w1.data(), tv.data(), true, false);
            for (int b = 0; b < n; ++b)
              for (int a = 0; a < n; ++a)
                for (int i = 0; i < n; ++i) {
                  int ix[3];
                  ix[d] = i;
                  ix[t1d] = a;
                  ix[t2d] = b;
                  Number w = comp == 3 ? lv[i] * ld[i] : lv[i] * lv[i];
                  out[(ix[2] * n + ix[1]) * n + ix[0]] += w * tv[b * n + a];
                }
          }
        }
        std::copy(out.begin(), out.end(), diag + c * n3);
      }
    }
  }

  // brute force: diagonal of the cell-local operator by unit vectors (small meshes only)
  void diagonal_bruteforce(Number* diag) const {
    long nc = n_cells(), n3 = (long)n * n * n;
    std::vector<Number> src(n_dofs(), Number(0)), buf(buf_size()), out(n3);
    for (long c = 0; c < nc; ++c)
      for (long i = 0; i < n3; ++i) {
        src[c * n3 + i] = 1;
        std::fill(out.begin(), out.end(), Number(0));
        cell_term(c, src.data() + c * n3, out.data(), buf.data());
        face_terms(c, src.data(), out.data(), buf.data(), HOMOGENEOUS, nullptr);
        diag[c * n3 + i] = out[i];
        src[c * n3 + i] = 0;
      }
  }
};

// -------------------------------------------------------------------------------------------
// Independent check: assembled matrix from naive quadrature (no sum factorisation)
// -------------------------------------------------------------------------------------------
static void assembled_apply(const Laplace<double>& op, const double* src, double* dst) {
  const Geometry& g = *op.geo;
  const Mesh& m = g.mesh;
  int n = op.n, nq = op.nq;
  long n3 = (long)n * n * n, nc = m.n_cells();
  std::vector<double> z = gauss_lobatto_points(n);
  auto phi = [&](int i, const double* xi, double* grad) {
    int a = i % n, b = (i / n) % n, c = i / (n * n);
    double v0 = lagrange(z, a, xi[0]), v1 = lagrange(z, b, xi[1]), v2 = lagrange(z, c, xi[2]);
    grad[0] = lagrange_deriv(z, a, xi[0]) * v1 * v2;
    grad[1] = v0 * lagrange_deriv(z, b, xi[1]) * v2;
    grad[2] = v0 * v1 * lagrange_deriv(z, c, xi[2]);
    return v0 * v1 * v2;
  };
  std::fill(dst, dst + op.n_dofs(), 0.0);
  std::vector<double> pv(n3), pg(3 * n3), nv(n3), ng(3 * n3);
  for (long c = 0; c < nc; ++c) {
    const double* cd = g.cell_data(c);
    for (int q2 = 0; q2 < nq; ++q2)
      for (int q1 = 0; q1 < nq; ++q1)
        for (int q0 = 0; q0 < nq; ++q0) {
          double xi[3] = {g.gq[q0], g.gq[q1], g.gq[q2]};
          const double* p = cd + ((q2 * nq + q1) * nq + q0) * CELL_STRIDE;
          for (long i = 0; i < n3; ++i) {
            double gr[3];
            phi((int)i, xi, gr);
            for (int j = 0; j < 3; ++j) pg[i * 3 + j] = p[0 * 3 + j] * gr[0] + p[1 * 3 + j] * gr[1] + p[2 * 3 + j] * gr[2];
          }
          double ux[3] = {0, 0, 0};
          for (long j = 0; j < n3; ++j)
            for (int e = 0; e < 3; ++e) ux[e] += pg[j * 3 + e] * src[c * n3 + j];
          for (long i = 0; i < n3; ++i)
            dst[c * n3 + i] += p[9] * (pg[i * 3] * ux[0] + pg[i * 3 + 1] * ux[1] + pg[i * 3 + 2] * ux[2]);
        }
    for (int f = 0; f < 6; ++f) {
      int d = f / 2, side = f % 2, t1, t2;
      tangential(d, t1, t2);
      long nb = m.neighbor(c, f);
      const double* fo = g.face_data(c, f);
      const double* fm = fo;
      if (nb >= 0 && side == 0) fm = g.face_data(nb, 2 * d + 1);
      double tau = nb >= 0 ? std::max((double)op.tau_cell[c], (double)op.tau_cell[nb]) * op.tau_factor
                           : op.tau_cell[c] * op.tau_factor;
      for (int b = 0; b < nq; ++b)
        for (int a = 0; a < nq; ++a) {
          double xi[3], xn[3];
          xi[d] = side;
          xi[t1] = g.gq[a];
          xi[t2] = g.gq[b];
          for (int e = 0; e < 3; ++e) xn[e] = xi[e];
          xn[d] = 1 - side;
          const double* po = fo + (b * nq + a) * FACE_STRIDE;
          const double* pm = fm + (b * nq + a) * FACE_STRIDE;
          const double* nrm = pm + 9;
          double JxW = pm[12];
          // own basis: value and normal derivative (with n-)
          for (long i = 0; i < n3; ++i) {
            double gr[3];
            pv[i] = phi((int)i, xi, gr);
            double s = 0;
            for (int j = 0; j < 3; ++j) s += nrm[j] * (po[0 * 3 + j] * gr[0] + po[1 * 3 + j] * gr[1] + po[2 * 3 + j] * gr[2]);
            pg[i] = s;
          }
          double uo = 0, ndo = 0;
          for (long j = 0; j < n3; ++j) {
            uo += pv[j] * src[c * n3 + j];
            ndo += pg[j] * src[c * n3 + j];
          }
          double un = 0, ndn = 0;
          if (nb >= 0) {
            const double* pn = g.face_data(nb, 2 * d + (1 - side)) + (b * nq + a) * FACE_STRIDE;
            for (long j = 0; j < n3; ++j) {
              double gr[3];
              double v = phi((int)j, xn, gr);
              double s = 0;
              for (int e = 0; e < 3; ++e) s += nrm[e] * (pn[0 * 3 + e] * gr[0] + pn[1 * 3 + e] * gr[1] + pn[2 * 3 + e] * gr[2]);
              un += v * src[nb * n3 + j];
              ndn += s * src[nb * n3 + j];
            }
          }
          // bilinear form of SIPG written directly: jump [u] = u- - u+, average {du/dn}
          double jump, avg;
          bool own_minus = (nb < 0) || side == 1;
          if (nb >= 0) {
            jump = own_minus ? uo - un : un - uo;
            avg = 0.5 * (ndo + ndn);
            // test function on own side: [v] = +-v, {dv/dn} = 0.5 dv/dn
            double sj = own_minus ? 1.0 : -1.0;
            for (long i = 0; i < n3; ++i)
              dst[c * n3 + i] += JxW * (-avg * sj * pv[i] - jump * 0.5 * pg[i] + tau * jump * sj * pv[i]);
          } else if (m.d.bc[f] == 0) {
            // Dirichlet (homogeneous): u+ = -u-, so [u] = 2u-, {du/dn} = du-/dn
            jump = 2 * uo;
            avg = ndo;
            for (long i = 0; i < n3; ++i) dst[c * n3 + i] += JxW * (-avg * pv[i] - jump * 0.5 * pg[i] + tau * jump * pv[i]);
          }
        }
    }
  }
}

// -------------------------------------------------------------------------------------------
// Continuous Q_k space on a Cartesian mesh (the continuous levels of cphMG)
//
// FE_Q(k) with Gauss-Lobatto support points (the same nodes as FE_DGQ(k)) on the node lattice
// of a box of N[0] x N[1] x N[2] equal cells: n_d = N_d k + 1 nodes per direction, N_d k when
// direction d is periodic (the last node plane is the first one).  Nodes are numbered x fastest.
// Constrained nodes (multigrid/constraints.h:130-197, multigrid_preconditioner_base.cpp:533-545):
// the nodes on Dirichlet sides, and node 0 when the operator is singular.
//
// Operator (OperatorBase::apply, operator_base.cpp:264-310, LaplaceOperator::do_cell_integral,
// laplace_operator.cpp): cell integrals only, (grad v, grad u) with k+1 Gauss points per
// direction; constrained entries of src are read as zero and dst = src on constrained nodes
// (the identity rows of the constrained DoFs).  On equal box cells the integral is the Kronecker
// sum A = K_x M_y M_z + M_x K_y M_z + M_x M_y K_z of the assembled 1D mass / stiffness
// matrices, applied as a = M_z x, b = K_z x, c = M_y a, d = K_y a + M_y b, A x = K_x c + M_x d.
// -------------------------------------------------------------------------------------------
struct Lattice {
  int N[3], k;
  int periodic[3];
  int dirichlet[6];
  bool pin_first;
  int n[3];
  double h[3];
  long size() const { return (long)n[0] * n[1] * n[2]; }
  bool constrained(int gx, int gy, int gz) const {
    int g[3] = {gx, gy, gz};
    for (int d = 0; d < 3; ++d)
      if (!periodic[d] && ((g[d] == 0 && dirichlet[2 * d]) || (g[d] == n[d] - 1 && dirichlet[2 * d + 1])))
        return true;
    return pin_first && gx == 0 && gy == 0 && gz == 0;
  }
  bool constrained(long i) const {
    return constrained((int)(i % n[0]), (int)((i / n[0]) % n[1]), (int)(i / ((long)n[0] * n[1])));
  }
};

static Lattice make_lattice(const orc_mesh_desc& m, int k, bool singular) {
  Lattice L;
  L.k = k;
  for (int d = 0; d < 3; ++d) {
    L.N[d] = m.n_cells[d];
    L.periodic[d] = m.periodic[d];
    L.n[d] = m.n_cells[d] * k + (m.periodic[d] ? 0 : 1);
    L.h[d] = (m.hi[d] - m.lo[d]) / m.n_cells[d];
  }
  for (int f = 0; f < 6; ++f) L.dirichlet[f] = (m.bc[f] == 0 && !m.periodic[f / 2]) ? 1 : 0;
  L.pin_first = singular;
  return L;
}

// assembled 1D matrix in band form: row g holds the entries of columns g + o, o = -k..k
// (column indices wrap on a periodic direction)
struct Band1D {
  int n, k;
  bool periodic;
  std::vector<double> a;  // [n][2k+1]
  double at(int g, int o) const { return a[(long)g * (2 * k + 1) + o + k]; }
  int col(int g, int o) const { return periodic ? ((g + o) % n + n) % n : g + o; }
};

// element matrices on a cell of length h: mass h (phi_i, phi_j), stiffness (phi_i', phi_j') / h,
// k+1 Gauss points (exact for both on an affine cell)
static void element_matrices_1d(int k, double h, std::vector<double>& Me, std::vector<double>& Ke) {
  std::vector<double> z = gauss_lobatto_points(k + 1), x, w;
  gauss_rule(k + 1, x, w);
  Me.assign((k + 1) * (k + 1), 0.0);
  Ke.assign((k + 1) * (k + 1), 0.0);
  for (int i = 0; i <= k; ++i)
    for (int j = 0; j <= k; ++j)
      for (int q = 0; q <= k; ++q) {
        Me[i * (k + 1) + j] += h * w[q] * lagrange(z, i, x[q]) * lagrange(z, j, x[q]);
        Ke[i * (k + 1) + j] += w[q] * lagrange_deriv(z, i, x[q]) * lagrange_deriv(z, j, x[q]) / h;
      }
}

static Band1D assemble_1d(const Lattice& L, int d, const std::vector<double>& E) {
  Band1D B;
  B.n = L.n[d];
  B.k = L.k;
  B.periodic = L.periodic[d];
  int k = L.k;
  B.a.assign((long)B.n * (2 * k + 1), 0.0);
  for (int e = 0; e < L.N[d]; ++e)
    for (int i = 0; i <= k; ++i) {
      int gi = e * k + i;
      if (B.periodic) gi %= B.n;
      for (int j = 0; j <= k; ++j) B.a[(long)gi * (2 * k + 1) + (j - i) + k] += E[i * (k + 1) + j];
    }
  return B;
}

// out = B along direction dir of a lattice array with extents dims
template <class Number>
static void band_apply(const Band1D& B, int dir, const int dims[3], const Number* in, Number* out) {
  long s[3] = {1, dims[0], (long)dims[0] * dims[1]};
  long total = (long)dims[0] * dims[1] * dims[2];
  int k = B.k;
#pragma omp parallel for
  for (long i = 0; i < total; ++i) {
    int g = (int)((i / s[dir]) % dims[dir]);
    long base = i - (long)g * s[dir];
    Number acc = 0;
    for (int o = -k; o <= k; ++o) {
      double v = B.at(g, o);
      if (v == 0.0) continue;
      int c = B.col(g, o);
      if (c < 0 || c >= B.n) continue;
      acc += (Number)v * in[base + (long)c * s[dir]];
    }
    out[i] = acc;
  }
}

// On a curved mesh (deformed cube) the same operator is the DG operator's cell term assembled
// through the lattice: gather the cell's nodes, (grad v, grad u) on the cell with its MappingQ
// geometry and k+1 Gauss points, sum into the nodes.
template <class Number>
struct ContinuousLaplace : LevelOp<Number> {
  Lattice L;
  Band1D M[3], K[3];
  std::unique_ptr<Laplace<Number>> cell;  // curved meshes: the cell term of the DG operator
  std::vector<long> map;                  // curved meshes: lattice node of each DG DoF
  long n_dofs() const override { return L.size(); }

  void init(const orc_mesh_desc& m, int degree, bool singular) {
    L = make_lattice(m, degree, singular);
    if (m.deform_amp != 0.0) {
      cell.reset(new Laplace<Number>());
      cell->init(make_geometry(make_mesh(m), degree + 1), degree, 1.0);
      dg_map(map);
      return;
    }
    for (int d = 0; d < 3; ++d) {
      std::vector<double> Me, Ke;
      element_matrices_1d(degree, L.h[d], Me, Ke);
      M[d] = assemble_1d(L, d, Me);
      K[d] = assemble_1d(L, d, Ke);
    }
  }

  // curved meshes: per cell f(u_cell) (the cell term, or its diagonal), summed into the nodes
  template <class F>
  void assemble(F&& f, std::vector<Number>& y) const {
    const long nc = cell->n_cells(), n3 = (long)(L.k + 1) * (L.k + 1) * (L.k + 1);
    std::vector<Number> dg(nc * n3);
#pragma omp parallel
    {
      std::vector<Number> buf(cell->buf_size()), out(n3);
#pragma omp for schedule(static)
      for (long c = 0; c < nc; ++c) {
        f(c, out.data(), buf.data());
        std::copy(out.begin(), out.end(), dg.begin() + c * n3);
      }
    }
    y.assign(L.size(), Number(0));
    for (long i = 0; i < (long)map.size(); ++i) y[map[i]] += dg[i];
  }

  void apply(const Number* src, Number* dst) const override {
    long N = L.size();
    if (cell) {
      std::vector<Number> x(N), y;
      for (long i = 0; i < N; ++i) x[i] = L.constrained(i) ? Number(0) : src[i];
      const long n3 = (long)(L.k + 1) * (L.k + 1) * (L.k + 1);
      assemble(
          [&](long c, Number* out, Number* buf) {
            std::vector<Number> u(n3);
            for (long q = 0; q < n3; ++q) u[q] = x[map[c * n3 + q]];
            std::fill(out, out + n3, Number(0));
            cell->cell_term(c, u.data(), out, buf);
          },
          y);
      for (long i = 0; i < N; ++i) dst[i] = L.constrained(i) ? src[i] : y[i];
      return;
    }
    std::vector<Number> x(N), a(N), b(N), c(N), d(N), t(N);
    for (long i = 0; i < N; ++i) x[i] = L.constrained(i) ? Number(0) : src[i];
    band_apply(M[2], 2, L.n, x.data(), a.data());
    band_apply(K[2], 2, L.n, x.data(), b.data());
    band_apply(M[1], 1, L.n, a.data(), c.data());
    band_apply(K[1], 1, L.n, a.data(), d.data());
    band_apply(M[1], 1, L.n, b.data(), t.data());
    for (long i = 0; i < N; ++i) d[i] += t[i];
    band_apply(K[0], 0, L.n, c.data(), a.data());
    band_apply(M[0], 0, L.n, d.data(), b.data());
    for (long i = 0; i < N; ++i) dst[i] = L.constrained(i) ? src[i] : a[i] + b[i];
  }

  // sum of the band entries of row g that land on column g (more than o = 0 only when a
  // periodic direction has a single cell)
  static double band_diag(const Band1D& B, int g) {
    double s = 0;
    for (int o = -B.k; o <= B.k; ++o)
      if (B.col(g, o) == g) s += B.at(g, o);
    return s;
  }

  void diagonal(Number* diag) const override {
    if (cell) {  // sum over the cells at a node of the cell term's diagonal entry
      const long n3 = (long)(L.k + 1) * (L.k + 1) * (L.k + 1);
      std::vector<Number> y;
      assemble(
          [&](long c, Number* out, Number* buf) {
            std::vector<Number> e(n3, Number(0)), col(n3);
            for (long j = 0; j < n3; ++j) {
              e[j] = Number(1);
              std::fill(col.begin(), col.end(), Number(0));
              cell->cell_term(c, e.data(), col.data(), buf);
              out[j] = col[j];
              e[j] = Number(0);
            }
          },
          y);
      for (long i = 0; i < L.size(); ++i) diag[i] = L.constrained(i) ? Number(1) : y[i];
      return;
    }
    for (long i = 0; i < L.size(); ++i) {
      int g[3] = {(int)(i % L.n[0]), (int)((i / L.n[0]) % L.n[1]), (int)(i / ((long)L.n[0] * L.n[1]))};
      if (L.constrained(g[0], g[1], g[2])) {
        diag[i] = Number(1);
        continue;
      }
      double m[3], kk[3];
      for (int d = 0; d < 3; ++d) {
        m[d] = band_diag(M[d], g[d]);
        kk[d] = band_diag(K[d], g[d]);
      }
      diag[i] = (Number)(kk[0] * m[1] * m[2] + m[0] * kk[1] * m[2] + m[0] * m[1] * kk[2]);
    }
  }

  // lattice node of each DG DoF (cell-wise, FE_DGQ nodes x fastest) of the same mesh and degree
  void dg_map(std::vector<long>& map) const {
    int k = L.k, n = k + 1;
    long nc = (long)L.N[0] * L.N[1] * L.N[2];
    map.resize(nc * n * n * n);
    for (long c = 0; c < nc; ++c) {
      int ci[3] = {(int)(c % L.N[0]), (int)((c / L.N[0]) % L.N[1]), (int)(c / ((long)L.N[0] * L.N[1]))};
      for (int q = 0; q < n * n * n; ++q) {
        int a[3] = {q % n, (q / n) % n, q / (n * n)};
        long idx = 0, stride = 1;
        for (int d = 0; d < 3; ++d) {
          int g = ci[d] * k + a[d];
          if (L.periodic[d]) g %= L.n[d];
          idx += g * stride;
          stride *= L.n[d];
        }
        map[c * n * n * n + q] = idx;
      }
    }
  }
};

// 1D interpolation between two lattices of one direction (rows: fine nodes; entries: coarse
// node, value).  p-transfer: same cells, degree kc -> kf; h-transfer: Nf = 2 Nc cells, fine cell
// ef in coarse cell ef / 2.  A node shared by two cells takes its row from the first cell (the
// values agree: the basis is interpolatory at the cell ends).
struct Prol1D {
  int nf, nc;
  std::vector<std::vector<std::pair<int, double>>> rows;
};

static Prol1D lattice_prolongation_1d(int Nc, int kc, int Nf, int kf, bool periodic) {
  Prol1D P;
  P.nf = Nf * kf + (periodic ? 0 : 1);
  P.nc = Nc * kc + (periodic ? 0 : 1);
  P.rows.assign(P.nf, {});
  std::vector<char> done(P.nf, 0);
  std::vector<double> zc = gauss_lobatto_points(kc + 1), zf = gauss_lobatto_points(kf + 1);
  bool is_h = Nf != Nc;
  for (int ef = 0; ef < Nf; ++ef)
    for (int i = 0; i <= kf; ++i) {
      int g = ef * kf + i;
      if (periodic) g %= P.nf;
      if (done[g]) continue;
      done[g] = 1;
      int ec = is_h ? ef / 2 : ef;
      double xi = is_h ? 0.5 * ((ef % 2) + zf[i]) : zf[i];
      for (int j = 0; j <= kc; ++j) {
        int cg = ec * kc + j;
        if (periodic) cg %= P.nc;
        P.rows[g].push_back({cg, lagrange(zc, j, xi)});
      }
    }
  return P;
}

// out = P along dir (transpose = false: in has the coarse extent along dir, out the fine one),
// or P^T (transpose = true: in fine, out coarse)
template <class Number>
static void prol_apply(const Prol1D& P, int dir, const int dims_in[3], const Number* in, Number* out,
                       bool transpose) {
  int dims_out[3] = {dims_in[0], dims_in[1], dims_in[2]};
  dims_out[dir] = transpose ? P.nc : P.nf;
  long si[3] = {1, dims_in[0], (long)dims_in[0] * dims_in[1]};
  long so[3] = {1, dims_out[0], (long)dims_out[0] * dims_out[1]};
  long total_out = (long)dims_out[0] * dims_out[1] * dims_out[2];
  std::fill(out, out + total_out, Number(0));
  long lines = total_out / dims_out[dir];
  for (long ln = 0; ln < lines; ++ln) {
    // base offsets of this line in both arrays
    long rem = ln, bo = 0, bi = 0;
    for (int d = 0; d < 3; ++d) {
      if (d == dir) continue;
      long c = rem % dims_out[d];
      rem /= dims_out[d];
      bo += c * so[d];
      bi += c * si[d];
    }
    for (int g = 0; g < P.nf; ++g)
      for (auto& e : P.rows[g]) {
        if (!transpose)
          out[bo + (long)g * so[dir]] += (Number)e.second * in[bi + (long)e.first * si[dir]];
        else
          out[bo + (long)e.first * so[dir]] += (Number)e.second * in[bi + (long)g * si[dir]];
      }
  }
}

template <class Number>
struct TransferBase {
  virtual ~TransferBase() {}
  virtual void prolongate_add(Number* dst, const Number* src) const = 0;
  virtual void restrict_add(Number* dst, const Number* src) const = 0;
};

// transfers of the continuous levels (deal.II MGTwoLevelTransfer on FE_Q, a third-party
// dependency; its published semantics): prolongation interpolates the coarse function, whose
// constrained nodes are read as zero, and adds it at the unconstrained fine nodes;
// restriction is the transpose (constrained fine entries ignored, contributions to constrained
// coarse nodes dropped).  Continuous -> continuous: the interpolation of a tensor-product
// function is the Kronecker product of the 1D interpolations.  Continuous -> discontinuous (the
// c-transfer, same mesh and degree): every DG node takes the value of its lattice node.
template <class Number>
struct LatticeTransfer : TransferBase<Number> {
  Lattice Lc, Lf;
  bool to_dg = false;
  Prol1D P[3];
  std::vector<long> map;  // c-transfer: lattice node of each DG DoF

  void setup(const Lattice& coarse, const Lattice* fine_cg, const ContinuousLaplace<Number>* same_mesh) {
    Lc = coarse;
    if (!fine_cg) {
      to_dg = true;
      same_mesh->dg_map(map);
      return;
    }
    Lf = *fine_cg;
    for (int d = 0; d < 3; ++d)
      P[d] = lattice_prolongation_1d(Lc.N[d], Lc.k, Lf.N[d], Lf.k, Lc.periodic[d]);
  }

  void prolongate_add(Number* dst, const Number* src) const override {
    long nc = Lc.size();
    std::vector<Number> u(nc);
    for (long i = 0; i < nc; ++i) u[i] = Lc.constrained(i) ? Number(0) : src[i];
    if (to_dg) {
      for (long i = 0; i < (long)map.size(); ++i) dst[i] += u[map[i]];
      return;
    }
    int d0[3] = {Lc.n[0], Lc.n[1], Lc.n[2]};
    int d1[3] = {Lf.n[0], Lc.n[1], Lc.n[2]};
    int d2[3] = {Lf.n[0], Lf.n[1], Lc.n[2]};
    std::vector<Number> a((long)d1[0] * d1[1] * d1[2]), b((long)d2[0] * d2[1] * d2[2]), c(Lf.size());
    prol_apply(P[0], 0, d0, u.data(), a.data(), false);
    prol_apply(P[1], 1, d1, a.data(), b.data(), false);
    prol_apply(P[2], 2, d2, b.data(), c.data(), false);
    for (long i = 0; i < Lf.size(); ++i)
      if (!Lf.constrained(i)) dst[i] += c[i];
  }

  void restrict_add(Number* dst, const Number* src) const override {
    long nc = Lc.size();
    std::vector<Number> v(nc, Number(0));
    if (to_dg) {
      for (long i = 0; i < (long)map.size(); ++i) v[map[i]] += src[i];
    } else {
      std::vector<Number> w(Lf.size());
      for (long i = 0; i < Lf.size(); ++i) w[i] = Lf.constrained(i) ? Number(0) : src[i];
      int d2[3] = {Lf.n[0], Lf.n[1], Lf.n[2]};
      int d1[3] = {Lf.n[0], Lf.n[1], Lc.n[2]};
      int d0[3] = {Lf.n[0], Lc.n[1], Lc.n[2]};
      std::vector<Number> a((long)d1[0] * d1[1] * d1[2]), b((long)d0[0] * d0[1] * d0[2]);
      prol_apply(P[2], 2, d2, w.data(), a.data(), true);
      prol_apply(P[1], 1, d1, a.data(), b.data(), true);
      prol_apply(P[0], 0, d0, b.data(), v.data(), true);
    }
    for (long i = 0; i < nc; ++i)
      if (!Lc.constrained(i)) dst[i] += v[i];
  }
};

// -------------------------------------------------------------------------------------------
// Vectors and Krylov pieces (deal.II SolverCG / ReductionControl semantics)
// -------------------------------------------------------------------------------------------
template <class T>
static double dot(const std::vector<T>& a, const std::vector<T>& b) {
  double s = 0;
#pragma omp parallel for reduction(+ : s)
  for (long i = 0; i < (long)a.size(); ++i) s += (double)a[i] * (double)b[i];
  return s;
}

struct CGResult {
  int its;
  bool converged;
  double r0, rn;
  std::vector<double> diag, offdiag;  // Lanczos tridiagonal
};

// generic PCG: A(x)->y, P(r)->z (may alias-free), with deal.II's ReductionControl check
// (iteration_status(it, |r|)): success if |r| <= max(abs_tol, rel_tol*|r0|); failure at max_iter
template <class T, class AOp, class POp>
static CGResult pcg(AOp&& A, POp&& P, const std::vector<T>& b, std::vector<T>& x, double rel_tol,
                    double abs_tol, int max_iter, bool track_eigs, bool fixed_iters = false) {
  long N = (long)b.size();
  std::vector<T> r(N), z(N), p(N), v(N);
  CGResult res{};
  bool zero_x = true;
  for (long i = 0; i < N; ++i)
    if (x[i] != T(0)) {
      zero_x = false;
      break;
    }
  if (zero_x)
    r = b;
  else {
    A(x, v);
#pragma omp parallel for
    for (long i = 0; i < N; ++i) r[i] = b[i] - v[i];
  }
  double rn = std::sqrt(dot(r, r));
  res.r0 = rn;
  res.rn = rn;
  double tol = fixed_iters ? abs_tol : std::max(abs_tol, rel_tol * rn);
  auto check = [&](int it, double val) -> int {
    if (fixed_iters) {
      if (it >= max_iter || val <= tol) return 1;
      return 0;
    }
    if (val <= tol) return 1;
    if (it >= max_iter || std::isnan(val)) return -1;
    return 0;
  };
  int st = check(0, rn);
  int it = 0;
  double rho_old = 0, alpha_old = 0;
  while (st == 0) {
    ++it;
    P(r, z);
    double rho = dot(r, z);
    double beta = 0;
    if (it == 1)
      p = z;
    else {
      beta = rho / rho_old;
#pragma omp parallel for
      for (long i = 0; i < N; ++i) p[i] = z[i] + (T)beta * p[i];
    }
    A(p, v);
    double pv = dot(p, v);
    double alpha = rho / pv;
#pragma omp parallel for
    for (long i = 0; i < N; ++i) {
      x[i] += (T)alpha * p[i];
      r[i] -= (T)alpha * v[i];
    }
    rn = std::sqrt(dot(r, r));
    if (track_eigs) {
      if (it == 1)
        res.diag.push_back(1.0 / alpha);
      else {
        res.diag.push_back(1.0 / alpha + beta / alpha_old);
        res.offdiag.push_back(std::sqrt(beta) / alpha_old);
      }
    }
    alpha_old = alpha;
    rho_old = rho;
    st = check(it, rn);
  }
  res.its = it;
  res.converged = st == 1;
  res.rn = rn;
  return res;
}

// eigenvalues of a symmetric tridiagonal matrix (implicit QL with Wilkinson shifts)
static std::vector<double> tridiag_eigenvalues(std::vector<double> d, std::vector<double> e) {
  int n = (int)d.size();
  e.resize(n, 0.0);
  for (int l = 0; l < n; ++l) {
    int iter = 0, mm;
    do {
      for (mm = l; mm < n - 1; ++mm) {
        double dd = std::fabs(d[mm]) + std::fabs(d[mm + 1]);
        if (std::fabs(e[mm]) <= 1e-15 * dd) break;
      }
      if (mm != l) {
        if (iter++ == 60) break;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[mm] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = mm - 1; i >= l; --i) {
          double f = s * e[i], b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) {
            d[i + 1] -= p;
            e[mm] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[mm] = 0.0;
      }
    } while (mm != l);
  }
  std::sort(d.begin(), d.end());
  return d;
}

// -------------------------------------------------------------------------------------------
// Multigrid (phMG, Bisect p-sequence, DG transfers, Chebyshev-Jacobi, coarse CG)
// -------------------------------------------------------------------------------------------
struct LevelInfo {
  int N[3];
  int degree;
  int dg;  // 1: discontinuous (FE_DGQ), 0: continuous (FE_Q)
};

// multigrid_preconditioner_base.cpp:137-307 (PSequenceType::Bisect): phMG keeps DG on every
// level; cphMG (c_transfer) puts a continuous level of the finest degree below the DG level
// (:188-199) and coarsens in the continuous space from there (h-levels at {1, continuous})
static std::vector<LevelInfo> mg_levels(const orc_mesh_desc& fine, int degree, int min_coarse, bool c_transfer) {
  std::vector<std::array<int, 3>> h;  // coarse to fine
  std::array<int, 3> Nc = {fine.n_cells[0], fine.n_cells[1], fine.n_cells[2]};
  h.push_back(Nc);
  while (Nc[0] % 2 == 0 && Nc[1] % 2 == 0 && Nc[2] % 2 == 0 && Nc[0] / 2 >= min_coarse &&
         Nc[1] / 2 >= min_coarse && Nc[2] / 2 >= min_coarse) {
    for (int e = 0; e < 3; ++e) Nc[e] /= 2;
    h.push_back(Nc);
  }
  std::reverse(h.begin(), h.end());
  std::vector<std::pair<int, int>> p;  // (degree, dg), fine to coarse
  int pp = degree;
  int dg = 1;
  if (c_transfer) {
    p.push_back({pp, 1});
    dg = 0;
  }
  do {
    p.push_back({pp, dg});
    pp = std::max(pp / 2, 1);
  } while (pp != p.back().first);
  std::reverse(p.begin(), p.end());
  std::vector<LevelInfo> lv;
  for (size_t i = 0; i + 1 < h.size(); ++i) lv.push_back({{h[i][0], h[i][1], h[i][2]}, p.front().first, p.front().second});
  for (auto q : p) lv.push_back({{h.back()[0], h.back()[1], h.back()[2]}, q.first, q.second});
  return lv;
}

// the inverse cell-diagonal blocks of a DG operator (block Jacobi, operator_base.cpp:820-900):
// each block (cell term + the cell's own side of its face terms) assembled from unit vectors in
// double, inverted by Gauss-Jordan elimination with partial pivoting, applied in Number
static void invert_dense(long n, std::vector<double>& A, std::vector<double>& inv) {
  inv.assign(n * n, 0.0);
  for (long i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (long p = 0; p < n; ++p) {
    long piv = p;
    for (long i = p + 1; i < n; ++i)
      if (std::fabs(A[i * n + p]) > std::fabs(A[piv * n + p])) piv = i;
    if (piv != p)
      for (long j = 0; j < n; ++j) {
        std::swap(A[p * n + j], A[piv * n + j]);
        std::swap(inv[p * n + j], inv[piv * n + j]);
      }
    const double d = A[p * n + p];
    for (long j = 0; j < n; ++j) {
      A[p * n + j] /= d;
      inv[p * n + j] /= d;
    }
    for (long i = 0; i < n; ++i) {
      if (i == p) continue;
      const double f = A[i * n + p];
      if (f == 0.0) continue;
      for (long j = 0; j < n; ++j) {
        A[i * n + j] -= f * A[p * n + j];
        inv[i * n + j] -= f * inv[p * n + j];
      }
    }
  }
}

template <class Number>
struct BlockInverse {
  long nc = 0, n3 = 0;
  std::vector<Number> inv;  // [cell][n3][n3]
  void init(const Laplace<double>& op) {
    nc = op.n_cells();
    n3 = (long)op.n * op.n * op.n;
    inv.resize(nc * n3 * n3);
    const long N = op.n_dofs();
#pragma omp parallel
    {
      std::vector<double> full(N, 0.0), buf(op.buf_size()), col(n3), A(n3 * n3), iv;
#pragma omp for schedule(static)
      for (long c = 0; c < nc; ++c) {
        for (long j = 0; j < n3; ++j) {
          full[c * n3 + j] = 1.0;
          std::fill(col.begin(), col.end(), 0.0);
          op.cell_term(c, full.data() + c * n3, col.data(), buf.data());
          op.face_terms(c, full.data(), col.data(), buf.data(), HOMOGENEOUS, nullptr);
          full[c * n3 + j] = 0.0;
          for (long i = 0; i < n3; ++i) A[i * n3 + j] = col[i];
        }
        invert_dense(n3, A, iv);
        for (long i = 0; i < n3 * n3; ++i) inv[c * n3 * n3 + i] = (Number)iv[i];
      }
    }
  }
  void apply(const Number* src, Number* dst) const {
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c)
      for (long i = 0; i < n3; ++i) {
        Number acc = 0;
        for (long j = 0; j < n3; ++j) acc += inv[(c * n3 + i) * n3 + j] * src[c * n3 + j];
        dst[c * n3 + i] = acc;
      }
  }
};

template <class Number>
struct Chebyshev {
  // deal.II PreconditionChebyshev (first kind), chebyshev_smoother.h:79-210
  const LevelOp<Number>* A;
  std::vector<Number> inv_diag;
  const BlockInverse<Number>* block = nullptr;  // PreconditionerSmoother::BlockJacobi when set
  int degree;
  double theta, delta, lambda_max, lambda_min;
  int eig_its;
  mutable std::vector<Number> t1, t2, old;

  void setup(const LevelOp<Number>* op, int deg, double range, int eig_iters) {
    A = op;
    degree = deg;
    long N = op->n_dofs();
    std::vector<Number> d(N);
    op->diagonal(d.data());
    inv_diag.resize(N);
    // invert_diagonal.h:35-46
    for (long i = 0; i < N; ++i) inv_diag[i] = std::fabs((double)d[i]) > 1e-10 ? Number(1) / d[i] : Number(1);
    t1.resize(N);
    t2.resize(N);
    old.resize(N);
    // eigenvalue estimate: CG on A x = b, b = (i % 11) - mean, x0 = 0, eig_iters steps
    std::vector<Number> b(N), x(N, Number(0));
    double mean = 0;
    for (long i = 0; i < N; ++i) {
      b[i] = (Number)(i % 11);
      mean += (double)b[i];
    }
    mean /= N;
    for (long i = 0; i < N; ++i) b[i] -= (Number)mean;
    auto Aop = [&](const std::vector<Number>& in, std::vector<Number>& out) { op->apply(in.data(), out.data()); };
    auto Pop = [&](const std::vector<Number>& in, std::vector<Number>& out) {
      if (block)
        block->apply(in.data(), out.data());
      else
        for (long i = 0; i < N; ++i) out[i] = inv_diag[i] * in[i];
    };
    CGResult r = pcg(Aop, Pop, b, x, 0.0, 1e-10, eig_iters, true, true);
    eig_its = r.its;
    std::vector<double> ev = tridiag_eigenvalues(r.diag, r.offdiag);
    lambda_max = ev.empty() ? 1.0 : ev.back();
    lambda_min = ev.empty() ? 1.0 : ev.front();
    double lmax = 1.2 * lambda_max;
    double alpha = range > 1.0 ? lmax / range : std::min(0.9 * lmax, lambda_min);
    delta = (lmax - alpha) * 0.5;
    theta = (lmax + alpha) * 0.5;
  }

  // x_{k+1} = (1+f1) x_k - f1 x_{k-1} + f2 P (b - A x_k)
  void iterate(std::vector<Number>& x, const std::vector<Number>& b, bool zero_start) const {
    long N = (long)x.size();
    // block Jacobi: t2 = P^-1 (b - t1) for the update (deal.II's preconditioner.vmult of the residual)
    auto block_residual = [&](bool with_t1) {
      for (long i = 0; i < N; ++i) t2[i] = with_t1 ? b[i] - t1[i] : b[i];
      std::vector<Number> z(N);
      block->apply(t2.data(), z.data());
      t2.swap(z);
    };
    int first;
    if (zero_start) {
      if (block) {
        block_residual(false);
        for (long i = 0; i < N; ++i) x[i] = (Number)(1.0 / theta) * t2[i];
      } else {
        for (long i = 0; i < N; ++i) x[i] = (Number)(1.0 / theta) * inv_diag[i] * b[i];
      }
      first = 0;
    } else {
      A->apply(x.data(), t1.data());
      Number f2 = (Number)(1.0 / theta);
      if (block) block_residual(true);
      for (long i = 0; i < N; ++i) {
        Number upd = block ? f2 * t2[i] : f2 * inv_diag[i] * (b[i] - t1[i]);
        old[i] = x[i];
        x[i] = x[i] + upd;
      }
      first = 1;
    }
    if (degree < 2 || std::fabs(delta) < 1e-40) return;
    double rhok = delta / theta, sigma = theta / delta;
    for (int k = 0; k < degree - 1; ++k) {
      A->apply(x.data(), t1.data());
      double rhokp = 1.0 / (2.0 * sigma - rhok);
      Number f1 = (Number)(rhokp * rhok), f2 = (Number)(2.0 * rhokp / delta);
      rhok = rhokp;
      int idx = k + 1 + first;
      if (block) block_residual(true);
      for (long i = 0; i < N; ++i) {
        Number pr = block ? t2[i] : inv_diag[i] * (b[i] - t1[i]);
        Number xn;
        if (idx == 1)
          xn = (Number(1) + f1) * x[i] + f2 * pr;  // x_{-1} = 0 after a zero start
        else
          xn = (Number(1) + f1) * x[i] - f1 * old[i] + f2 * pr;
        old[i] = x[i];
        x[i] = xn;
      }
    }
  }
};

// 1D prolongation matrices (fine n_f x coarse n_c)
static std::vector<double> p_prolongation(int kc, int kf) {
  std::vector<double> zc = gauss_lobatto_points(kc + 1), zf = gauss_lobatto_points(kf + 1);
  std::vector<double> P((kf + 1) * (kc + 1));
  for (int i = 0; i <= kf; ++i)
    for (int j = 0; j <= kc; ++j) P[i * (kc + 1) + j] = lagrange(zc, j, zf[i]);
  return P;
}
static std::vector<double> h_prolongation(int k, int child) {
  std::vector<double> z = gauss_lobatto_points(k + 1);
  std::vector<double> P((k + 1) * (k + 1));
  for (int i = 0; i <= k; ++i)
    for (int j = 0; j <= k; ++j) P[i * (k + 1) + j] = lagrange(z, j, 0.5 * (child + z[i]));
  return P;
}

template <class Number>
struct Transfer : TransferBase<Number> {
  // MGTwoLevelTransfer for DG (element-local interpolation; restriction = transpose)
  bool is_h;
  int Nf[3], Nc[3], nf, nc;
  std::vector<Number> P[2];  // p: P[0]; h: child 0/1
  void setup(const LevelInfo& coarse, const LevelInfo& fine) {
    is_h = coarse.N[0] != fine.N[0];
    for (int e = 0; e < 3; ++e) {
      Nf[e] = fine.N[e];
      Nc[e] = coarse.N[e];
    }
    nf = fine.degree + 1;
    nc = coarse.degree + 1;
    if (is_h)
      for (int ch = 0; ch < 2; ++ch) {
        auto m = h_prolongation(fine.degree, ch);
        P[ch].assign(m.begin(), m.end());
      }
    else {
      auto m = p_prolongation(coarse.degree, fine.degree);
      P[0].assign(m.begin(), m.end());
    }
  }
  // dst_fine += P src_coarse
  void prolongate_add(Number* dst, const Number* src) const override {
    long ncells_f = (long)Nf[0] * Nf[1] * Nf[2];
    long nf3 = (long)nf * nf * nf, nc3 = (long)nc * nc * nc;
#pragma omp parallel
    {
      std::vector<Number> a(nf * nf * nf), b(nf * nf * nf);
#pragma omp for
      for (long cf = 0; cf < ncells_f; ++cf) {
        int ci[3] = {(int)(cf % Nf[0]), (int)((cf / Nf[0]) % Nf[1]), (int)(cf / ((long)Nf[0] * Nf[1]))};
        long cc;
        int ch[3] = {0, 0, 0};
        if (is_h) {
          for (int e = 0; e < 3; ++e) ch[e] = ci[e] % 2;
          cc = ci[0] / 2 + (long)Nc[0] * (ci[1] / 2 + (long)Nc[1] * (ci[2] / 2));
        } else
          cc = cf;
        const Number* u = src + cc * nc3;
        int d0[3] = {nc, nc, nc}, d1[3] = {nf, nc, nc}, d2[3] = {nf, nf, nc};
        sweep(P[ch[0]].data(), nf, nc, 0, d0, u, a.data(), false, false);
        sweep(P[ch[1]].data(), nf, nc, 1, d1, a.data(), b.data(), false, false);
        sweep(P[ch[2]].data(), nf, nc, 2, d2, b.data(), a.data(), false, false);
        for (long i = 0; i < nf3; ++i) dst[cf * nf3 + i] += a[i];
      }
    }
  }
  // dst_coarse += P^T src_fine
  void restrict_add(Number* dst, const Number* src) const override {
    long ncells_c = (long)Nc[0] * Nc[1] * Nc[2];
    long nf3 = (long)nf * nf * nf, nc3 = (long)nc * nc * nc;
#pragma omp parallel
    {
      std::vector<Number> a(nf * nf * nf), b(nf * nf * nf), acc(nc3);
#pragma omp for
      for (long cc = 0; cc < ncells_c; ++cc) {
        std::fill(acc.begin(), acc.end(), Number(0));
        int ci[3] = {(int)(cc % Nc[0]), (int)((cc / Nc[0]) % Nc[1]), (int)(cc / ((long)Nc[0] * Nc[1]))};
        int nch = is_h ? 8 : 1;
        for (int c8 = 0; c8 < nch; ++c8) {
          int ch[3] = {c8 & 1, (c8 >> 1) & 1, (c8 >> 2) & 1};
          long cf;
          if (is_h)
            cf = (2 * ci[0] + ch[0]) + (long)Nf[0] * ((2 * ci[1] + ch[1]) + (long)Nf[1] * (2 * ci[2] + ch[2]));
          else {
            cf = cc;
            ch[0] = ch[1] = ch[2] = 0;
          }
          const Number* u = src + cf * nf3;
          int d2[3] = {nf, nf, nf}, d1[3] = {nf, nf, nc}, d0[3] = {nf, nc, nc};
          sweep(P[ch[2]].data(), nf, nc, 2, d2, u, a.data(), true, false);
          sweep(P[ch[1]].data(), nf, nc, 1, d1, a.data(), b.data(), true, false);
          sweep(P[ch[0]].data(), nf, nc, 0, d0, b.data(), acc.data(), true, true);
        }
        for (long i = 0; i < nc3; ++i) dst[cc * nc3 + i] += acc[i];
      }
    }
  }
};

template <class Number>
struct Multigrid {
  std::vector<LevelInfo> info;
  std::vector<std::unique_ptr<LevelOp<Number>>> ops;
  std::vector<std::unique_ptr<Chebyshev<Number>>> smoothers;
  std::vector<std::unique_ptr<BlockInverse<Number>>> blocks;  // block-Jacobi smoothing
  std::vector<std::unique_ptr<TransferBase<Number>>> transfers;  // transfers[l] between l-1 and l
  std::unique_ptr<LevelOp<double>> coarse_op_d;  // coarse operator in double (optional)
  std::vector<double> coarse_inv_diag_d;
  std::vector<Number> coarse_inv_diag;
  mutable std::vector<std::vector<Number>> defect, solution, t;
  mutable std::vector<double> coarse_sol_d;
  orc_solver_desc desc;
  mutable long coarse_its = 0, vcycles = 0;

  // operator of level l in precision T: SIPG on DG levels, the lattice operator on continuous ones
  template <class T>
  static std::unique_ptr<LevelOp<T>> make_op(const orc_mesh_desc& md, const LevelInfo& li, double ip, bool singular) {
    if (li.dg) {
      auto g = make_geometry(make_mesh(md), li.degree + 1);
      auto* op = new Laplace<T>();
      op->init(g, li.degree, ip);
      return std::unique_ptr<LevelOp<T>>(op);
    }
    auto* op = new ContinuousLaplace<T>();
    op->init(md, li.degree, singular);
    return std::unique_ptr<LevelOp<T>>(op);
  }

  // continuous_fine: the fine operator is the continuous one (a continuous discretization): the
  // cphMG level list without its DG top level
  void setup(const orc_mesh_desc& fine, int degree, double ip, const orc_solver_desc& d, bool continuous_fine = false) {
    desc = d;
    info = mg_levels(fine, degree, std::max(1, d.min_coarse_cells), d.mg_type == 1 || continuous_fine);
    if (continuous_fine) info.pop_back();
    int L = (int)info.size();
    ops.resize(L);
    smoothers.resize(L);
    transfers.resize(L);
    defect.resize(L);
    solution.resize(L);
    t.resize(L);
    for (int l = 0; l < L; ++l) {
      orc_mesh_desc md = fine;
      for (int e = 0; e < 3; ++e) md.n_cells[e] = info[l].N[e];
      ops[l] = make_op<Number>(md, info[l], ip, d.singular != 0);
      long N = ops[l]->n_dofs();
      defect[l].assign(N, Number(0));
      solution[l].assign(N, Number(0));
      t[l].assign(N, Number(0));
      if (l > 0) {
        smoothers[l].reset(new Chebyshev<Number>());
        if (d.smoother_block) {  // block Jacobi is defined for DG levels (operator_base.cpp:653)
          if (!info[l].dg) throw std::runtime_error("block-Jacobi smoothing needs DG levels");
          blocks.resize(L);
          auto g = make_geometry(make_mesh(md), info[l].degree + 1);
          Laplace<double> opd;
          opd.init(g, info[l].degree, ip);
          blocks[l].reset(new BlockInverse<Number>());
          blocks[l]->init(opd);
          smoothers[l]->block = blocks[l].get();
        }
        smoothers[l]->setup(ops[l].get(), d.cheb_degree, d.smoothing_range, d.eig_iters);
        const LevelInfo &ci = info[l - 1], &fi = info[l];
        if (ci.dg) {
          auto* tr = new Transfer<Number>();
          tr->setup(ci, fi);
          transfers[l].reset(tr);
        } else {
          orc_mesh_desc mc = fine;
          for (int e = 0; e < 3; ++e) mc.n_cells[e] = ci.N[e];
          Lattice lc = make_lattice(mc, ci.degree, d.singular != 0);
          auto* tr = new LatticeTransfer<Number>();
          if (fi.dg) {
            tr->setup(lc, nullptr, (const ContinuousLaplace<Number>*)ops[l - 1].get());
          } else {
            Lattice lf = make_lattice(md, fi.degree, d.singular != 0);
            tr->setup(lc, &lf, nullptr);
          }
          transfers[l].reset(tr);
        }
      }
      if (l == 0) {
        std::vector<Number> dg(N);
        ops[0]->diagonal(dg.data());
        coarse_inv_diag.resize(N);
        for (long i = 0; i < N; ++i) coarse_inv_diag[i] = std::fabs((double)dg[i]) > 1e-10 ? Number(1) / dg[i] : Number(1);
        if (d.coarse_double) {
          coarse_op_d = make_op<double>(md, info[0], ip, d.singular != 0);
          std::vector<double> dd(N);
          coarse_op_d->diagonal(dd.data());
          coarse_inv_diag_d.resize(N);
          for (long i = 0; i < N; ++i) coarse_inv_diag_d[i] = std::fabs(dd[i]) > 1e-10 ? 1.0 / dd[i] : 1.0;
          coarse_sol_d.assign(N, 0.0);
        }
      }
    }
  }

  // MGCoarseKrylov::operator(), coarse_grid_solvers.h:157-224: CG + Jacobi from the current
  // content of dst (the previous coarse solution), rel tol 1e-3
  void coarse(std::vector<Number>& dst, const std::vector<Number>& src) const {
    long N = (long)src.size();
    if (desc.coarse_double) {
      std::vector<double> r(src.begin(), src.end());
      if (desc.singular) {
        double mean = 0;
        for (double v : r) mean += v;
        mean /= N;
        for (double& v : r) v -= mean;
      }
      auto Aop = [&](const std::vector<double>& in, std::vector<double>& out) { coarse_op_d->apply(in.data(), out.data()); };
      auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) {
        for (long i = 0; i < N; ++i) out[i] = coarse_inv_diag_d[i] * in[i];
      };
      CGResult cr = pcg(Aop, Pop, r, coarse_sol_d, desc.coarse_rel_tol, desc.coarse_abs_tol, desc.coarse_max_iter, false);
      coarse_its += cr.its;
      for (long i = 0; i < N; ++i) dst[i] = (Number)coarse_sol_d[i];
    } else {
      std::vector<Number> r(src);
      if (desc.singular) {
        double mean = 0;
        for (Number v : r) mean += (double)v;
        mean /= N;
        for (Number& v : r) v -= (Number)mean;
      }
      auto Aop = [&](const std::vector<Number>& in, std::vector<Number>& out) { ops[0]->apply(in.data(), out.data()); };
      auto Pop = [&](const std::vector<Number>& in, std::vector<Number>& out) {
        for (long i = 0; i < N; ++i) out[i] = coarse_inv_diag[i] * in[i];
      };
      CGResult cr = pcg(Aop, Pop, r, dst, desc.coarse_rel_tol, desc.coarse_abs_tol, desc.coarse_max_iter, false);
      coarse_its += cr.its;
    }
  }

  // MultigridAlgorithm::v_cycle, multigrid_algorithm.h:172-240
  void v_cycle(int l) const {
    if (l == 0) {
      coarse(solution[0], defect[0]);
      return;
    }
    smoothers[l]->iterate(solution[l], defect[l], true);
    ops[l]->apply(solution[l].data(), t[l].data());
    long N = (long)t[l].size();
    for (long i = 0; i < N; ++i) t[l][i] = defect[l][i] - t[l][i];
    transfers[l]->restrict_add(defect[l - 1].data(), t[l].data());
    v_cycle(l - 1);
    transfers[l]->prolongate_add(solution[l].data(), solution[l - 1].data());
    smoothers[l]->iterate(solution[l], defect[l], false);
  }

  // MultigridAlgorithm::vmult, multigrid_algorithm.h:87-108
  void vmult(const double* src, double* dst) const {
    int L = (int)info.size();
    for (int l = 0; l < L - 1; ++l) std::fill(defect[l].begin(), defect[l].end(), Number(0));
    long N = (long)defect[L - 1].size();
    for (long i = 0; i < N; ++i) defect[L - 1][i] = (Number)src[i];
    v_cycle(L - 1);
    for (long i = 0; i < N; ++i) dst[i] = (double)solution[L - 1][i];
    ++vcycles;
  }
};

// -------------------------------------------------------------------------------------------
// relative L2 error, postprocessor/error_calculation.cpp:38-110 (QGauss(k+3))
// -------------------------------------------------------------------------------------------
static double relative_l2_error(const Mesh& mesh, int degree, const double* x, const Fn& fn) {
  int n = degree + 1, nq = degree + 3;
  auto g = make_geometry(mesh, nq);
  std::vector<double> z = gauss_lobatto_points(n);
  std::vector<double> S(nq * n);
  for (int q = 0; q < nq; ++q)
    for (int i = 0; i < n; ++i) S[q * n + i] = lagrange(z, i, g->gq[q]);
  long nc = mesh.n_cells(), n3 = (long)n * n * n, nq3 = (long)nq * nq * nq;
  double err = 0, nrm = 0;
#pragma omp parallel reduction(+ : err, nrm)
  {
    std::vector<double> a(nq * n * n), b(nq * nq * n), v(nq3);
#pragma omp for
    for (long c = 0; c < nc; ++c) {
      int d0[3] = {n, n, n}, d1[3] = {nq, n, n}, d2[3] = {nq, nq, n};
      sweep(S.data(), nq, n, 0, d0, x + c * n3, a.data(), false, false);
      sweep(S.data(), nq, n, 1, d1, a.data(), b.data(), false, false);
      sweep(S.data(), nq, n, 2, d2, b.data(), v.data(), false, false);
      const double* cd = g->cell_data(c);
      if (g->uniform) {
        // uniform geometry stores one cell; shift the quadrature points
        int ci[3];
        mesh.coords(c, ci);
        for (long q = 0; q < nq3; ++q) {
          const double* p = cd + q * CELL_STRIDE;
          double xq[3];
          for (int e = 0; e < 3; ++e) xq[e] = p[10 + e] + ci[e] * mesh.h[e];
          double ue = fn.u(xq);
          err += p[9] * (v[q] - ue) * (v[q] - ue);
          nrm += p[9] * ue * ue;
        }
      } else {
        for (long q = 0; q < nq3; ++q) {
          const double* p = cd + q * CELL_STRIDE;
          double ue = fn.u(p + 10);
          err += p[9] * (v[q] - ue) * (v[q] - ue);
          nrm += p[9] * ue * ue;
        }
      }
    }
  }
  return std::sqrt(err) / std::sqrt(nrm);
}

// -------------------------------------------------------------------------------------------
struct Problem {
  Mesh mesh;
  int degree;
  double ip;
  std::shared_ptr<Geometry> geo;
  std::unique_ptr<Laplace<double>> opd;
  std::unique_ptr<Laplace<float>> opf;
  const Laplace<float>& f32() {
    if (!opf) {
      opf.reset(new Laplace<float>());
      opf->init(geo, degree, ip);
    }
    return *opf;
  }
};

}  // namespace orc

// ============================================================================================
// C interface (ctypes)
// ============================================================================================
using namespace orc;

extern "C" {

void* orc_create(const orc_mesh_desc* m, int degree, double ip) {
  try {
    auto* p = new Problem();
    p->mesh = make_mesh(*m);
    p->degree = degree;
    p->ip = ip;
    p->geo = make_geometry(p->mesh, degree + 1);
    p->opd.reset(new Laplace<double>());
    p->opd->init(p->geo, degree, ip);
    return p;
  } catch (...) {
    return nullptr;
  }
}

void orc_destroy(void* h) { delete (Problem*)h; }
long orc_n_dofs(void* h) { return ((Problem*)h)->opd->n_dofs(); }
int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

void orc_apply_f64(void* h, const double* src, double* dst) { ((Problem*)h)->opd->apply(src, dst); }
void orc_apply_f32(void* h, const float* src, float* dst) { ((Problem*)h)->f32().apply(src, dst); }
void orc_penalty(void* h, double* tau) {
  auto& op = *((Problem*)h)->opd;
  for (long c = 0; c < op.n_cells(); ++c) tau[c] = op.tau_cell[c];
}
void orc_diagonal_f64(void* h, double* d) { ((Problem*)h)->opd->diagonal(d); }
void orc_diagonal_f32(void* h, float* d) { ((Problem*)h)->f32().diagonal(d); }
void orc_diagonal_bruteforce(void* h, double* d) { ((Problem*)h)->opd->diagonal_bruteforce(d); }

// OperatorBase::apply_inverse_block_diagonal (operator_base.cpp:820-900; block Jacobi): per cell the
// diagonal block A_cc (cell term + the cell's own side of its face terms, neighbours zero) is
// assembled column by column from unit vectors and inverted by Gauss-Jordan elimination with
// partial pivoting; dst_c = A_cc^-1 src_c
void orc_block_jacobi(void* h, const double* src, double* dst) {
  const Laplace<double>& op = *((Problem*)h)->opd;
  const long nc = op.n_cells(), n3 = (long)op.n * op.n * op.n, N = op.n_dofs();
#pragma omp parallel
  {
    std::vector<double> full(N, 0.0), buf(op.buf_size()), col(n3), A(n3 * n3), inv(n3 * n3);
#pragma omp for schedule(static)
    for (long c = 0; c < nc; ++c) {
      for (long j = 0; j < n3; ++j) {
        full[c * n3 + j] = 1.0;
        std::fill(col.begin(), col.end(), 0.0);
        op.cell_term(c, full.data() + c * n3, col.data(), buf.data());
        op.face_terms(c, full.data(), col.data(), buf.data(), HOMOGENEOUS, nullptr);
        full[c * n3 + j] = 0.0;
        for (long i = 0; i < n3; ++i) A[i * n3 + j] = col[i];
      }
      // Gauss-Jordan on [A | I]
      for (long i = 0; i < n3; ++i)
        for (long j = 0; j < n3; ++j) inv[i * n3 + j] = i == j ? 1.0 : 0.0;
      for (long p = 0; p < n3; ++p) {
        long piv = p;
        for (long i = p + 1; i < n3; ++i)
          if (std::fabs(A[i * n3 + p]) > std::fabs(A[piv * n3 + p])) piv = i;
        if (piv != p)
          for (long j = 0; j < n3; ++j) {
            std::swap(A[p * n3 + j], A[piv * n3 + j]);
            std::swap(inv[p * n3 + j], inv[piv * n3 + j]);
          }
        const double d = A[p * n3 + p];
        for (long j = 0; j < n3; ++j) {
          A[p * n3 + j] /= d;
          inv[p * n3 + j] /= d;
        }
        for (long i = 0; i < n3; ++i) {
          if (i == p) continue;
          const double f = A[i * n3 + p];
          if (f == 0.0) continue;
          for (long j = 0; j < n3; ++j) {
            A[i * n3 + j] -= f * A[p * n3 + j];
            inv[i * n3 + j] -= f * inv[p * n3 + j];
          }
        }
      }
      for (long i = 0; i < n3; ++i) {
        double acc = 0;
        for (long j = 0; j < n3; ++j) acc += inv[i * n3 + j] * src[c * n3 + j];
        dst[c * n3 + i] = acc;
      }
    }
  }
}
void orc_assembled_apply(void* h, const double* src, double* dst) { assembled_apply(*((Problem*)h)->opd, src, dst); }

void orc_rhs(void* h, int fn_kind, double omega, int with_f, double* b) {
  Fn fn{fn_kind, omega};
  ((Problem*)h)->opd->rhs(fn, with_f != 0, b);
}

double orc_error(void* h, const double* x, int fn_kind, double omega) {
  Problem* p = (Problem*)h;
  Fn fn{fn_kind, omega};
  return relative_l2_error(p->mesh, p->degree, x, fn);
}

// interpolation of the manufactured solution at the DoF nodes (used for tests)
void orc_interpolate(void* h, int fn_kind, double omega, double* x) {
  Problem* p = (Problem*)h;
  Fn fn{fn_kind, omega};
  int n = p->degree + 1;
  std::vector<double> z = gauss_lobatto_points(n);
  long n3 = (long)n * n * n;
  for (long c = 0; c < p->mesh.n_cells(); ++c) {
    MappingEval me;
    me.init(p->mesh, c);
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double xi[3] = {z[i], z[j], z[k]}, xx[3], J[3][3];
          me.eval(xi, xx, J);
          x[c * n3 + (k * n + j) * n + i] = fn.u(xx);
        }
  }
}

void orc_default_solver_desc(orc_solver_desc* d) {
  d->precond = 2;
  d->rel_tol = 1e-10;
  d->abs_tol = 1e-20;
  d->max_iter = 10000;
  d->mg_float = 1;
  d->cheb_degree = 5;
  d->smoothing_range = 20;
  d->eig_iters = 20;
  d->coarse_rel_tol = 1e-3;
  d->coarse_abs_tol = 1e-12;
  d->coarse_max_iter = 10000;
  d->coarse_double = 0;
  d->min_coarse_cells = 2;
  d->singular = 0;
  d->mg_type = 0;
  d->smoother_block = 0;
}

// multigrid handle (templated on the V-cycle precision)
struct MGHandle {
  int is_float;
  std::unique_ptr<Multigrid<float>> mf;
  std::unique_ptr<Multigrid<double>> md;
  void vmult(const double* s, double* d) const {
    if (is_float)
      mf->vmult(s, d);
    else
      md->vmult(s, d);
  }
};

void* orc_mg_create(void* h, const orc_solver_desc* d) {
  Problem* p = (Problem*)h;
  auto* mg = new MGHandle();
  mg->is_float = d->mg_float;
  if (d->mg_float) {
    mg->mf.reset(new Multigrid<float>());
    mg->mf->setup(p->mesh.d, p->degree, p->ip, *d);
  } else {
    mg->md.reset(new Multigrid<double>());
    mg->md->setup(p->mesh.d, p->degree, p->ip, *d);
  }
  return mg;
}
void orc_mg_destroy(void* mg) { delete (MGHandle*)mg; }
void orc_mg_vmult(void* mg, const double* src, double* dst) { ((MGHandle*)mg)->vmult(src, dst); }
int orc_mg_n_levels(void* mg) {
  auto* m = (MGHandle*)mg;
  return m->is_float ? (int)m->mf->info.size() : (int)m->md->info.size();
}
// level info: N[3], degree, lambda_max (raw CG estimate), eig iterations
void orc_mg_level(void* mg, int l, int* N, int* degree, double* lambda_max, int* eig_its) {
  auto* m = (MGHandle*)mg;
  const LevelInfo& li = m->is_float ? m->mf->info[l] : m->md->info[l];
  for (int e = 0; e < 3; ++e) N[e] = li.N[e];
  *degree = li.degree;
  *lambda_max = 0;
  *eig_its = 0;
  if (l > 0) {
    if (m->is_float) {
      *lambda_max = m->mf->smoothers[l]->lambda_max;
      *eig_its = m->mf->smoothers[l]->eig_its;
    } else {
      *lambda_max = m->md->smoothers[l]->lambda_max;
      *eig_its = m->md->smoothers[l]->eig_its;
    }
  }
}
long orc_mg_coarse_iterations(void* mg) {
  auto* m = (MGHandle*)mg;
  return m->is_float ? m->mf->coarse_its : m->md->coarse_its;
}

// outer CG (Krylov::KrylovSolver::solve -> SolverCG with ReductionControl)
void orc_block_jacobi(void* h, const double* src, double* dst);

int orc_solve(void* h, const orc_solver_desc* d, const double* b, double* x, orc_solver_result* res) {
  Problem* p = (Problem*)h;
  long N = p->opd->n_dofs();
  std::vector<double> bv(b, b + N), xv(x, x + N);
  auto Aop = [&](const std::vector<double>& in, std::vector<double>& out) { p->opd->apply(in.data(), out.data()); };
  CGResult r;
  if (d->precond == 0) {
    auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) { out = in; };
    r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
  } else if (d->precond == 3) {  // block Jacobi
    auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) { orc_block_jacobi(h, in.data(), out.data()); };
    r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
  } else if (d->precond == 1) {
    std::vector<double> dg(N);
    p->opd->diagonal(dg.data());
    for (long i = 0; i < N; ++i) dg[i] = std::fabs(dg[i]) > 1e-10 ? 1.0 / dg[i] : 1.0;
    auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) {
      for (long i = 0; i < N; ++i) out[i] = dg[i] * in[i];
    };
    r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
  } else {
    MGHandle* mg = (MGHandle*)orc_mg_create(h, d);
    auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) { mg->vmult(in.data(), out.data()); };
    r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
    delete mg;
  }
  std::copy(xv.begin(), xv.end(), x);
  if (res) {
    res->iterations = r.its;
    res->converged = r.converged;
    res->r0 = r.r0;
    res->rn = r.rn;
    // performance metrics, iterative_solvers_dealii_wrapper.h:63-78
    if (r.its > 0) {
      res->rho = std::pow(r.rn / r.r0, 1.0 / r.its);
      res->n10 = -10.0 * std::log(10.0) / std::log(res->rho);
    } else {
      res->rho = 0;
      res->n10 = 0;
    }
  }
  return r.converged ? 0 : 1;
}

// CG with an external preconditioner given by the MG handle (for mixed-precision parity)
int orc_solve_with_mg(void* h, void* mg, const orc_solver_desc* d, const double* b, double* x, orc_solver_result* res) {
  Problem* p = (Problem*)h;
  long N = p->opd->n_dofs();
  std::vector<double> bv(b, b + N), xv(x, x + N);
  auto Aop = [&](const std::vector<double>& in, std::vector<double>& out) { p->opd->apply(in.data(), out.data()); };
  auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) { ((MGHandle*)mg)->vmult(in.data(), out.data()); };
  CGResult r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
  std::copy(xv.begin(), xv.end(), x);
  if (res) {
    res->iterations = r.its;
    res->converged = r.converged;
    res->r0 = r.r0;
    res->rn = r.rn;
    res->rho = r.its > 0 ? std::pow(r.rn / r.r0, 1.0 / r.its) : 0;
    res->n10 = r.its > 0 ? -10.0 * std::log(10.0) / std::log(res->rho) : 0;
  }
  return r.converged ? 0 : 1;
}

// Chebyshev smoother on the fine operator alone (double), for smoother parity tests
// mode 0: vmult (zero start), mode 1: step
void orc_chebyshev(void* h, int degree, double range, int eig_iters, int mode, const double* b, double* x, double* lambda_max) {
  Problem* p = (Problem*)h;
  Chebyshev<double> ch;
  ch.setup(p->opd.get(), degree, range, eig_iters);
  long N = p->opd->n_dofs();
  std::vector<double> xv(x, x + N), bv(b, b + N);
  ch.iterate(xv, bv, mode == 0);
  std::copy(xv.begin(), xv.end(), x);
  if (lambda_max) *lambda_max = ch.lambda_max;
}

// transfers between two levels (coarse degree/cells -> fine)
void orc_transfer(int kc, int kf, const int* Nc, const int* Nf, int restrict_mode, const double* src, double* dst) {
  LevelInfo c{{Nc[0], Nc[1], Nc[2]}, kc, 1}, f{{Nf[0], Nf[1], Nf[2]}, kf, 1};
  Transfer<double> t;
  t.setup(c, f);
  if (restrict_mode)
    t.restrict_add(dst, src);
  else
    t.prolongate_add(dst, src);
}

// continuous levels: the lattice operator (cphMG) and its transfers
struct CGHandle {
  ContinuousLaplace<double> d;
  ContinuousLaplace<float> f;
  orc_mesh_desc mesh;
  int degree;
};
void* orc_cg_create(const orc_mesh_desc* m, int degree, int singular) {
  auto* h = new CGHandle();
  h->d.init(*m, degree, singular != 0);
  h->f.init(*m, degree, singular != 0);
  h->mesh = *m;
  h->degree = degree;
  return h;
}
// multigrid for the continuous discretization (levels: continuous p- then h-coarsening)
void* orc_cg_mg_create(void* h, const orc_solver_desc* d) {
  CGHandle* c = (CGHandle*)h;
  auto* mg = new MGHandle();
  mg->is_float = d->mg_float;
  if (d->mg_float) {
    mg->mf.reset(new Multigrid<float>());
    mg->mf->setup(c->mesh, c->degree, 1.0, *d, true);
  } else {
    mg->md.reset(new Multigrid<double>());
    mg->md->setup(c->mesh, c->degree, 1.0, *d, true);
  }
  return mg;
}
// CG on the continuous operator, preconditioned by such a multigrid (mg may be null: no
// preconditioner)
int orc_cg_solve(void* h, void* mg, const orc_solver_desc* d, const double* b, double* x, orc_solver_result* res) {
  CGHandle* c = (CGHandle*)h;
  long N = c->d.n_dofs();
  std::vector<double> bv(b, b + N), xv(x, x + N);
  auto Aop = [&](const std::vector<double>& in, std::vector<double>& out) { c->d.apply(in.data(), out.data()); };
  CGResult r;
  if (mg) {
    auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) { ((MGHandle*)mg)->vmult(in.data(), out.data()); };
    r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
  } else {
    auto Pop = [&](const std::vector<double>& in, std::vector<double>& out) { out = in; };
    r = pcg(Aop, Pop, bv, xv, d->rel_tol, d->abs_tol, d->max_iter, false);
  }
  std::copy(xv.begin(), xv.end(), x);
  if (res) {
    res->iterations = r.its;
    res->converged = r.converged;
    res->r0 = r.r0;
    res->rn = r.rn;
    res->rho = r.its > 0 ? std::pow(r.rn / r.r0, 1.0 / r.its) : 0;
    res->n10 = r.its > 0 ? -10.0 * std::log(10.0) / std::log(res->rho) : 0;
  }
  return r.converged ? 0 : 1;
}
void orc_cg_destroy(void* h) { delete (CGHandle*)h; }
long orc_cg_n_dofs(void* h) { return ((CGHandle*)h)->d.n_dofs(); }
void orc_cg_apply_f64(void* h, const double* src, double* dst) { ((CGHandle*)h)->d.apply(src, dst); }
void orc_cg_apply_f32(void* h, const float* src, float* dst) { ((CGHandle*)h)->f.apply(src, dst); }
void orc_cg_diagonal_f64(void* h, double* d) { ((CGHandle*)h)->d.diagonal(d); }
void orc_cg_constrained(void* h, unsigned char* mask) {
  const Lattice& L = ((CGHandle*)h)->d.L;
  for (long i = 0; i < L.size(); ++i) mask[i] = L.constrained(i) ? 1 : 0;
}
void orc_cg_dg_map(void* h, long* map) {
  std::vector<long> m;
  ((CGHandle*)h)->d.dg_map(m);
  std::copy(m.begin(), m.end(), map);
}
// transfer from the continuous level (Nc cells, degree kc) to the level of mesh m (degree kf,
// discontinuous when fine_dg, then with Nc = m's cells and kc = kf)
void orc_lattice_transfer(const orc_mesh_desc* m, const int* Nc, int kc, int kf, int fine_dg, int singular,
                          int restrict_mode, const double* src, double* dst) {
  orc_mesh_desc mc = *m;
  for (int e = 0; e < 3; ++e) mc.n_cells[e] = Nc[e];
  Lattice lc = make_lattice(mc, kc, singular != 0);
  LatticeTransfer<double> t;
  ContinuousLaplace<double> same;
  if (fine_dg) {
    same.init(mc, kc, singular != 0);
    t.setup(lc, nullptr, &same);
  } else {
    Lattice lf = make_lattice(*m, kf, singular != 0);
    t.setup(lc, &lf, nullptr);
  }
  if (restrict_mode)
    t.restrict_add(dst, src);
  else
    t.prolongate_add(dst, src);
}
int orc_mg_level_dg(void* mg, int l) {
  auto* m = (MGHandle*)mg;
  return m->is_float ? m->mf->info[l].dg : m->md->info[l].dg;
}

// 1D finite element data, so the tests can check the product's tables
void orc_fe1d(int n, double* gl_nodes, double* gauss_pts, double* gauss_wts) {
  std::vector<double> z = gauss_lobatto_points(n), x, w;
  gauss_rule(n, x, w);
  for (int i = 0; i < n; ++i) {
    gl_nodes[i] = z[i];
    gauss_pts[i] = x[i];
    gauss_wts[i] = w[i];
  }
}

// Chebyshev eigen estimate helper exposed for tests: eigenvalues of a tridiagonal matrix
void orc_tridiag_eigs(int n, const double* d, const double* e, double* out) {
  std::vector<double> dv(d, d + n), ev(e, e + (n > 0 ? n - 1 : 0));
  auto r = tridiag_eigenvalues(dv, ev);
  for (int i = 0; i < n; ++i) out[i] = r[i];
}

}  // extern "C"
