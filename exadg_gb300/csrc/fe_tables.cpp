// 1D finite-element tables for FE_DGQ(k) on Gauss-Lobatto support points with QGauss(n_q)
// (operators/finite_element.h:60, operators/quadrature.h:45), and the Cartesian coefficient set
// of the SIPG operator (poisson/spatial_discretization/laplace_operator.cpp:129-265).
#include <cmath>
#include <cstring>

#include "internal.h"

namespace exg {

static double legendre_p(int n, double x, double* dp) {
  if (n == 0) {
    *dp = 0;
    return 1;
  }
  double p0 = 1, p1 = x, d0 = 0, d1 = 1;
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    double d2 = d0 + (2 * k - 1) * p1;
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  *dp = d1;
  return p1;
}

void gauss(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0);
  w.assign(n, 0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p = legendre_p(n, z, &dp);
      double dz = p / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    legendre_p(n, z, &dp);
    double wi = 1.0 / ((1 - z * z) * dp * dp);
    x[i] = 0.5 - 0.5 * z;
    x[n - 1 - i] = 0.5 + 0.5 * z;
    w[i] = w[n - 1 - i] = wi;
  }
}

std::vector<double> gauss_lobatto(int n) {
  std::vector<double> x(n);
  x[0] = 0;
  x[n - 1] = 1;
  int k = n - 1;
  for (int i = 1; i <= (n - 1) / 2; ++i) {
    double z = std::cos(M_PI * i / k), dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p = legendre_p(k, z, &dp);
      double ddp = (2 * z * dp - k * (k + 1.0) * p) / (1 - z * z);
      double dz = dp / ddp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = 0.5 - 0.5 * z;
    x[n - 1 - i] = 0.5 + 0.5 * z;
  }
  if (n % 2 == 1 && n > 2) x[n / 2] = 0.5;
  return x;
}

double lagrange(const std::vector<double>& z, int i, double x) {
  double v = 1;
  for (int j = 0; j < (int)z.size(); ++j)
    if (j != i) v *= (x - z[j]) / (z[i] - z[j]);
  return v;
}

double lagrange_d(const std::vector<double>& z, int i, double x) {
  double s = 0;
  for (int m = 0; m < (int)z.size(); ++m) {
    if (m == i) continue;
    double t = 1 / (z[i] - z[m]);
    for (int j = 0; j < (int)z.size(); ++j)
      if (j != i && j != m) t *= (x - z[j]) / (z[i] - z[j]);
    s += t;
  }
  return s;
}

void FE1D::init(int degree, int n_q) {
  k = degree;
  n = degree + 1;
  nq = n_q;
  gl = gauss_lobatto(n);
  gauss(nq, gq, gw);
  S.resize(nq * n);
  D.resize(nq * n);
  for (int q = 0; q < nq; ++q)
    for (int i = 0; i < n; ++i) {
      S[q * n + i] = lagrange(gl, i, gq[q]);
      D[q * n + i] = lagrange_d(gl, i, gq[q]);
    }
  M.assign(n * n, 0);
  K.assign(n * n, 0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int q = 0; q < nq; ++q) {
        M[i * n + j] += gw[q] * S[q * n + i] * S[q * n + j];
        K[i * n + j] += gw[q] * D[q * n + i] * D[q * n + j];
      }
  dL.resize(n);
  dR.resize(n);
  for (int i = 0; i < n; ++i) {
    dL[i] = lagrange_d(gl, i, 0.0);
    dR[i] = lagrange_d(gl, i, 1.0);
  }
}

// On an affine box cell the SIPG operator with QGauss(k+1) factorises exactly:
//   A = sum_d (A_d * L_d) (x) M (x) M,
// L_d = line operator of direction d (stiffness / h_d plus the face terms of
// laplace_operator.cpp:139-163, 221-265), M = reference mass, A_d = face area normal to d.
// B holds the interior-cell line operator (times h_d): K + 1/2 (dL e0^T + e0 dL^T)
//   - 1/2 (dR e_{n-1}^T + e_{n-1} dR^T); penalty and boundary variants are added in the kernel.
void build_cart_host(const MeshInfo& m, const FE1D& fe, double ip, CartHost& out) {
  std::memset(&out, 0, sizeof(out));
  int n = fe.n;
  out.n = n;
  for (int i = 0; i < n * n; ++i) out.M[i] = fe.M[i];
  for (int d = 0; d < 3; ++d) {
    double A = 1.0;
    for (int e = 0; e < 3; ++e)
      if (e != d) A *= m.h[e];
    double s = A / m.h[d];
    out.A[d] = A;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double b = fe.K[i * n + j];
        if (j == 0) b += 0.5 * fe.dL[i];
        if (i == 0) b += 0.5 * fe.dL[j];
        if (j == n - 1) b -= 0.5 * fe.dR[i];
        if (i == n - 1) b -= 0.5 * fe.dR[j];
        out.B[d][i * n + j] = s * b;
      }
    for (int i = 0; i < n; ++i) {
      out.sdL[d][i] = 0.5 * s * fe.dL[i];
      out.sdR[d][i] = 0.5 * s * fe.dR[i];
    }
  }
  for (int e = 0; e < 3; ++e) out.pen.inv_h[e] = 1.0 / m.h[e];
  out.pen.factor = ip * (fe.k + 1.0) * (fe.k + 1.0);
  // IP::calculate_penalty_parameter on a box cell: tau_c = surface / volume with weight 1 on
  // non-periodic boundary faces and 0.5 elsewhere = sum_e (w_low + w_high) / h_e.  The class of a
  // cell encodes per direction bit 0 = at the low boundary, bit 1 = at the high boundary.
  for (int cls = 0; cls < 64; ++cls) {
    double t = 0;
    for (int e = 0; e < 3; ++e) {
      int code = (cls >> (2 * e)) & 3;
      double wl = (code & 1) ? 1.0 : 0.5, wr = (code & 2) ? 1.0 : 0.5;
      t += (wl + wr) / m.h[e];
    }
    for (int d = 0; d < 3; ++d) out.tauA[d][cls] = out.A[d] * t * out.pen.factor;
  }
  for (int e = 0; e < 3; ++e) {
    out.mesh.N[e] = m.N[e];
    out.mesh.periodic[e] = m.d.periodic[e];
  }
  for (int f = 0; f < 6; ++f) out.mesh.bc[f] = m.d.bc[f];
  out.mesh.n_cells = m.n_cells();
  out.mesh.n_dofs = m.n_cells() * n * n * n;
  out.mesh.cell_begin = 0;
  out.mesh.cell_end = out.mesh.n_cells;
}

}  // namespace exg
