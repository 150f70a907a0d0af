// Host orchestration: operator set-up and dispatch, the multigrid hierarchy (phMG, Bisect,
// Chebyshev-Jacobi, coarse CG, V-cycle as a CUDA graph) and the outer PCG.
#include "host.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>

namespace exg {

MeshInfo make_mesh_info(const exg_mesh_desc& d) {
  MeshInfo m;
  m.d = d;
  for (int e = 0; e < 3; ++e) {
    EXG_CHECK(d.n_cells[e] >= 1, EXG_ERR_INVALID, "n_cells must be >= 1");
    EXG_CHECK(d.hi[e] > d.lo[e], EXG_ERR_INVALID, "box must have positive extent");
    m.N[e] = d.n_cells[e];
    m.h[e] = (d.hi[e] - d.lo[e]) / d.n_cells[e];
    if (d.deform_amp != 0.0)
      EXG_CHECK(!d.periodic[e], EXG_ERR_UNSUPPORTED, "periodic directions need an affine mesh");
  }
  for (int f = 0; f < 6; ++f)
    EXG_CHECK(d.bc[f] == EXG_BC_DIRICHLET || d.bc[f] == EXG_BC_NEUMANN, EXG_ERR_INVALID, "bad boundary type");
  return m;
}

// --------------------------------------------------------------------------------------------
// deterministic scalar readback
// --------------------------------------------------------------------------------------------
static double read_slot(Reduction& red, int slot, cudaStream_t s) {
  double v;
  EXG_CUDA(cudaMemcpyAsync(&v, red.out + slot, sizeof(double), cudaMemcpyDeviceToHost, s));
  EXG_CUDA(cudaStreamSynchronize(s));
  return v;
}

static size_t psize(int prec) { return prec == EXG_PREC_F32 ? sizeof(float) : sizeof(double); }

static void* dalloc(size_t bytes) {
  void* p = nullptr;
  EXG_CUDA(cudaMalloc(&p, bytes));
  return p;
}

}  // namespace exg

using namespace exg;

// ============================================================================================
// operator
// ============================================================================================
exg_op::exg_op(const MeshInfo& m, int deg, double ip_factor, int prec)
    : mesh(m), degree(deg), n(deg + 1), ip(ip_factor), precision(prec) {
  EXG_CHECK(deg >= 1 && deg <= 8, EXG_ERR_UNSUPPORTED, "degree must be 1..8");
  EXG_CHECK(prec == EXG_PREC_F64 || prec == EXG_PREC_F32 || prec == EXG_PREC_F64E, EXG_ERR_INVALID,
            "unknown precision");
  EXG_CHECK(m.n_cells() * n * n * n < (1LL << 40), EXG_ERR_INVALID, "mesh too large");
  fe.init(deg, deg + 1);
  cartesian = m.affine();
  build_cart_host(m, fe, ip, cart);
  if (!cartesian) {
    geo.reset(new GeneralGeom());
    geo->build(m, fe, ip, prec, false, nullptr);
    EXG_CUDA(cudaDeviceSynchronize());
  }
}

std::unique_ptr<exg_op> exg_op::continuous_level(const MeshInfo& m, int deg, int prec, bool singular) {
  EXG_CHECK(prec == EXG_PREC_F32 || prec == EXG_PREC_F64, EXG_ERR_UNSUPPORTED,
            "continuous levels compute in FP32 or FP64");
  std::unique_ptr<exg_op> op(new exg_op(m, deg, 1.0, prec));
  op->continuous = true;
  op->lat.reset(new LatticeHost());
  make_lattice(m, deg, singular, *op->lat);
  lattice_prepare(*op->lat, prec);
  if (!op->cartesian) {
    // curved: the DG geometry with every face read as Neumann is the cell term alone
    std::vector<long long> neumann((size_t)m.n_cells() * 6, -2);
    EXG_CUDA(cudaMemcpy(op->geo->fnb, neumann.data(), neumann.size() * sizeof(long long), cudaMemcpyHostToDevice));
    op->geo->cell_only = true;
    op->cdg.reset(new DgScratch());
    const size_t bytes = (size_t)m.n_cells() * op->n * op->n * op->n * psize(prec);
    for (void*& p : op->cdg->v) p = dalloc(bytes);
  }
  return op;
}

const BlockJacobi& exg_op::block_jacobi(int prec) {
  EXG_CHECK(!continuous, EXG_ERR_UNSUPPORTED, "block Jacobi is built for the DG operator");
  const int slot = prec == EXG_PREC_F32 ? 0 : 1;
  if (!bj[slot]) {
    std::unique_ptr<BlockJacobi> b(new BlockJacobi());
    b->setup(mesh, fe, ip, prec == EXG_PREC_F32 ? EXG_PREC_F32 : EXG_PREC_F64);
    bj[slot] = std::move(b);
  }
  return *bj[slot];
}

void exg_op::apply(const void* src, void* dst, int n_rhs, cudaStream_t s, const exg::PointEpilogue& ep,
                   long long cell_begin, long long cell_end) const {
  if (continuous) {
    EXG_CHECK(cell_begin == 0 && cell_end < 0, EXG_ERR_INVALID, "continuous levels apply on the whole lattice");
    EXG_CHECK(n_rhs == 1 || ep.mode < 0, EXG_ERR_INVALID, "fused store needs a single right-hand side");
    const size_t stride = (size_t)lat->size() * (precision == EXG_PREC_F32 ? 4 : 8);
    for (int r = 0; r < n_rhs; ++r) {
      const void* sr = (const char*)src + r * stride;
      void* dr = dst ? (char*)dst + r * stride : nullptr;
      if (cartesian) {
        lattice_apply(*lat, precision, sr, dr, s, ep);
      } else {
        lattice_to_dg(*lat, precision, sr, cdg->v[0], s);
        general_apply(*geo, fe, cdg->v[0], cdg->v[1], 1, s);
        dg_to_lattice_apply(*lat, precision, cdg->v[1], sr, dr, ep, s);
      }
    }
    return;
  }
  const long long nc = mesh.n_cells();
  if (cell_end < 0) cell_end = nc;
  EXG_CHECK(cell_begin >= 0 && cell_begin < cell_end && cell_end <= nc, EXG_ERR_INVALID, "bad cell range");
  if (cartesian) {
    if (cell_begin == 0 && cell_end == nc) {
      cart_apply(cart, precision, src, dst, n_rhs, cpb, s, ep);
    } else {
      CartHost part = cart;
      part.mesh.cell_begin = cell_begin;
      part.mesh.cell_end = cell_end;
      cart_apply(part, precision, src, dst, n_rhs, cpb, s, ep);
    }
  } else {
    general_apply(*geo, fe, src, dst, n_rhs, s, ep, cell_begin, cell_end);
  }
}

HostPipe::~HostPipe() {
  for (cudaEvent_t e : loaded) cudaEventDestroy(e);
  for (cudaEvent_t e : done) cudaEventDestroy(e);
  for (cudaEvent_t e : {start, end})
    if (e) cudaEventDestroy(e);
  for (cudaStream_t t : {in, comp, out})
    if (t) cudaStreamDestroy(t);
  for (double* p : {src, dst})
    if (p) cudaFree(p);
}

// The mesh is cut into K slabs of z-planes (contiguous cell and DoF ranges).  Slab j is copied in
// on one stream, applied on a second once the slabs it touches through faces are resident, and
// copied out on a third, so the host-to-device copy of slab j+1, the apply of slab j and the copy
// back of slab j-1 overlap.  With periodicity in z, slab 0 needs slab K-1 and is applied last.
void exg_op::apply_host(const double* src_host, double* dst_host, int n_slabs, cudaStream_t s) {
  EXG_CHECK(!continuous, EXG_ERR_UNSUPPORTED, "not available for a continuous operator");
  EXG_CHECK(precision != EXG_PREC_F32, EXG_ERR_INVALID, "host apply needs an FP64-storage operator");
  const int Nz = mesh.N[2];
  const int K = std::max(1, std::min(n_slabs, Nz));
  const long long plane_dofs = (long long)mesh.N[0] * mesh.N[1] * n * n * n;
  const long long plane_cells = (long long)mesh.N[0] * mesh.N[1];
  if (!pipe) {
    pipe.reset(new HostPipe());
    pipe->src = (double*)dalloc(n_dofs() * 8);
    pipe->dst = (double*)dalloc(n_dofs() * 8);
    EXG_CUDA(cudaStreamCreateWithFlags(&pipe->in, cudaStreamNonBlocking));
    EXG_CUDA(cudaStreamCreateWithFlags(&pipe->comp, cudaStreamNonBlocking));
    EXG_CUDA(cudaStreamCreateWithFlags(&pipe->out, cudaStreamNonBlocking));
    EXG_CUDA(cudaEventCreateWithFlags(&pipe->start, cudaEventDisableTiming));
    EXG_CUDA(cudaEventCreateWithFlags(&pipe->end, cudaEventDisableTiming));
  }
  HostPipe& P = *pipe;
  while ((int)P.loaded.size() < K) {
    cudaEvent_t a, b;
    EXG_CUDA(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
    EXG_CUDA(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
    P.loaded.push_back(a);
    P.done.push_back(b);
  }
  auto zb = [&](int j) { return (int)((long long)Nz * j / K); };  // first plane of slab j
  EXG_CUDA(cudaEventRecord(P.start, s));
  EXG_CUDA(cudaStreamWaitEvent(P.in, P.start, 0));
  EXG_CUDA(cudaStreamWaitEvent(P.out, P.start, 0));
  for (int j = 0; j < K; ++j) {
    const long long off = zb(j) * plane_dofs, len = (long long)(zb(j + 1) - zb(j)) * plane_dofs;
    EXG_CUDA(cudaMemcpyAsync(P.src + off, src_host + off, len * 8, cudaMemcpyHostToDevice, P.in));
    EXG_CUDA(cudaEventRecord(P.loaded[j], P.in));
  }
  const bool zper = mesh.d.periodic[2] != 0 && K > 1;
  std::vector<int> order;
  for (int j = zper ? 1 : 0; j < K; ++j) order.push_back(j);
  if (zper) order.push_back(0);
  for (int j : order) {
    const int need = (zper && j == 0) ? K - 1 : std::min(j + 1, K - 1);
    EXG_CUDA(cudaStreamWaitEvent(P.comp, P.loaded[need], 0));
    apply(P.src, P.dst, 1, P.comp, PointEpilogue(), zb(j) * plane_cells, zb(j + 1) * plane_cells);
    EXG_CUDA(cudaEventRecord(P.done[j], P.comp));
    const long long off = zb(j) * plane_dofs, len = (long long)(zb(j + 1) - zb(j)) * plane_dofs;
    EXG_CUDA(cudaStreamWaitEvent(P.out, P.done[j], 0));
    EXG_CUDA(cudaMemcpyAsync(dst_host + off, P.dst + off, len * 8, cudaMemcpyDeviceToHost, P.out));
  }
  // the caller's stream continues after the last copy back (and after the apply stream, so the
  // next call's copies into the device buffers follow this call's reads)
  EXG_CUDA(cudaEventRecord(P.end, P.out));
  EXG_CUDA(cudaStreamWaitEvent(s, P.end, 0));
  EXG_CUDA(cudaEventRecord(P.end, P.comp));
  EXG_CUDA(cudaStreamWaitEvent(s, P.end, 0));
}

void exg_op::diagonal(void* d, bool invert, cudaStream_t s) const {
  if (continuous && cartesian) {
    lattice_diagonal(*lat, precision, d, invert, s);
  } else if (continuous) {
    general_diagonal(*geo, fe, cdg->v[1], false, s);
    dg_to_lattice_diagonal(*lat, precision, cdg->v[1], d, invert, s);
  }
  else if (cartesian)
    cart_diagonal(cart, precision, d, invert, s);
  else
    general_diagonal(*geo, fe, d, invert, s);
}

// Autotuner: time every cells-per-block variant of the affine kernel on this operator's mesh,
// degree and precision (CUDA events, median of 5 launches after 2 warm-up launches) and keep the
// fastest.  Curved meshes have a single variant.
int exg_op::tune(int n_rhs, cudaStream_t s, std::vector<std::pair<int, float>>* timings) {
  if (!cartesian || continuous) return 0;
  std::vector<int> opts = cart_cpb_options(n, precision);
  size_t bytes = (size_t)n_dofs() * n_rhs * (precision == EXG_PREC_F32 ? 4 : 8);
  void* x = dalloc(bytes);
  void* y = dalloc(bytes);
  vec_fill(x, precision, 1.0, n_dofs() * n_rhs, s);
  cudaEvent_t e0, e1;
  EXG_CUDA(cudaEventCreate(&e0));
  EXG_CUDA(cudaEventCreate(&e1));
  int best = opts.empty() ? 0 : opts[0];
  float best_ms = 1e30f;
  for (int c : opts) {
    cpb = c;
    for (int w = 0; w < 2; ++w) apply(x, y, n_rhs, s);
    std::vector<float> t;
    for (int r = 0; r < 5; ++r) {
      EXG_CUDA(cudaEventRecord(e0, s));
      apply(x, y, n_rhs, s);
      EXG_CUDA(cudaEventRecord(e1, s));
      EXG_CUDA(cudaEventSynchronize(e1));
      float ms;
      EXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      t.push_back(ms);
    }
    std::sort(t.begin(), t.end());
    if (timings) timings->push_back({c, t[2]});
    if (t[2] < best_ms) {
      best_ms = t[2];
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(y);
  cpb = best;
  return best;
}

CGWorkspace& exg_op::workspace() {
  if (!ws) {
    ws.reset(new CGWorkspace());
    long long n = n_dofs();
    ws->r = (double*)dalloc(n * 8);
    ws->z = (double*)dalloc(n * 8);
    ws->p = (double*)dalloc(n * 8);
    ws->v = (double*)dalloc(n * 8);
    ws->dinv = (double*)dalloc(n * 8);
    ws->red = Reduction::create();
  }
  return *ws;
}

CGWorkspace::~CGWorkspace() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cap) cudaStreamDestroy(cap);
  if (st_host) cudaFreeHost(st_host);
  if (st) cudaFree(st);
  for (double* ptr : {r, z, p, v, dinv, xw, bw})
    if (ptr) cudaFree(ptr);
  red.destroy();
}

void exg_op::ensure_rhs_geometry(cudaStream_t s) {
  EXG_CHECK(!continuous, EXG_ERR_UNSUPPORTED, "not available for a continuous operator");
  if (rhs_geo) return;
  rhs_geo.reset(new GeneralGeom());
  rhs_geo->build(mesh, fe, ip, EXG_PREC_F64, true, s);
  EXG_CUDA(cudaStreamSynchronize(s));
}

void exg_op::quadrature_points(double* cx, double* fx, long long* ncp, long long* nfp, cudaStream_t s) {
  ensure_rhs_geometry(s);
  const GeneralGeom& g = (rhs_geo ? *rhs_geo : *geo);
  general_points(g, cx, fx, ncp, nfp, s);
}

void exg_op::rhs(const double* f, const double* g, const double* h, double* b, cudaStream_t s) {
  ensure_rhs_geometry(s);
  const GeneralGeom& gg = (rhs_geo ? *rhs_geo : *geo);
  general_rhs(gg, fe, f, g, h, b, s);
}

// ============================================================================================
// PCG driver (deal.II SolverCG + ReductionControl / IterationNumberControl semantics,
// solvers/iterative_solvers_dealii_wrapper.h:136-221)
// ============================================================================================
namespace exg {
struct CGStats {
  int its = 0;
  int status = 0;  // 0 converged, 1 max_iter, 2 non-finite
  double r0 = 0, rn = 0;
  std::vector<double> diag, offdiag;
};

template <class T, class AOp, class POp>
static CGStats pcg_run(AOp&& A, POp&& P, const T* b, T* x, long long n, double rel, double abs, int max_iter,
                       bool fixed, bool track, T* r, T* z, T* p, T* v, Reduction& red, cudaStream_t s) {
  CGStats st;
  dot<T>(x, x, n, red, 0, s);
  bool xzero = read_slot(red, 0, s) == 0.0;
  if (xzero)
    residual<T>(b, nullptr, r, n, red, 1, s);
  else {
    A(x, v);
    residual<T>(b, v, r, n, red, 1, s);
  }
  double rn = std::sqrt(read_slot(red, 1, s));
  st.r0 = rn;
  double tol = fixed ? abs : std::max(abs, rel * rn);
  auto check = [&](int it, double val) -> int {
    if (!std::isfinite(val)) return 2;
    if (fixed) return (it >= max_iter || val <= tol) ? 0 : -1;
    if (val <= tol) return 0;
    if (it >= max_iter) return 1;
    return -1;
  };
  int c = check(0, rn);
  int it = 0;
  double rho_old = 0, alpha_old = 0;
  while (c < 0) {
    ++it;
    double rho = P(r, z);
    double beta = it == 1 ? 0.0 : rho / rho_old;
    p_update<T>(z, p, beta, it == 1, n, s);
    A(p, v);
    dot<T>(p, v, n, red, 2, s);
    double pv = read_slot(red, 2, s);
    double alpha = rho / pv;
    xr_update<T>(x, r, p, v, alpha, n, red, 3, s);
    rn = std::sqrt(read_slot(red, 3, s));
    if (track) {
      if (it == 1)
        st.diag.push_back(1.0 / alpha);
      else {
        st.diag.push_back(1.0 / alpha + beta / alpha_old);
        st.offdiag.push_back(std::sqrt(beta) / alpha_old);
      }
    }
    alpha_old = alpha;
    rho_old = rho;
    c = check(it, rn);
  }
  st.its = it;
  st.rn = rn;
  st.status = c;
  return st;
}

// eigenvalues of a symmetric tridiagonal matrix: implicit QL iteration with Wilkinson shifts
static std::vector<double> tridiag_eigs(std::vector<double> d, std::vector<double> e) {
  const int n = (int)d.size();
  e.resize(n, 0.0);
  for (int l = 0; l < n; ++l) {
    for (int iter = 0; iter < 100; ++iter) {
      int m = l;
      for (; m < n - 1; ++m)
        if (std::fabs(e[m]) <= 1e-15 * (std::fabs(d[m]) + std::fabs(d[m + 1]))) break;
      if (m == l) break;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
      double sn = 1, cs = 1, p = 0;
      bool deflated = false;
      for (int i = m - 1; i >= l; --i) {
        double f = sn * e[i], bb = cs * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= p;
          e[m] = 0.0;
          deflated = true;
          break;
        }
        sn = f / r;
        cs = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * sn + 2.0 * cs * bb;
        p = sn * r;
        d[i + 1] = g + p;
        g = cs * r - bb;
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  std::sort(d.begin(), d.end());
  return d;
}

// MGLevelInfo list for phMG with the Bisect p-sequence (multigrid_preconditioner_base.cpp:97-323)
struct LevelSpec {
  std::array<int, 3> N;
  int degree;
  int dg;
};

// multigrid_preconditioner_base.cpp:137-307 with PSequenceType::Bisect: h-levels at the coarsest
// p-level, then the p-levels on the finest mesh.  cphMG (c_transfer) inserts a continuous level of
// the finest degree below the DG level (:188-199); every level below it is continuous.
static std::vector<LevelSpec> mg_level_list(const int Nf[3], int degree, int min_coarse, bool c_transfer) {
  std::vector<std::array<int, 3>> h;
  std::array<int, 3> Nc = {Nf[0], Nf[1], Nf[2]};
  h.push_back(Nc);
  while (Nc[0] % 2 == 0 && Nc[1] % 2 == 0 && Nc[2] % 2 == 0 && Nc[0] / 2 >= min_coarse && Nc[1] / 2 >= min_coarse &&
         Nc[2] / 2 >= min_coarse) {
    for (int e = 0; e < 3; ++e) Nc[e] /= 2;
    h.push_back(Nc);
  }
  std::reverse(h.begin(), h.end());
  std::vector<std::pair<int, int>> p;  // (degree, dg), fine to coarse
  int pp = degree, dg = 1;
  if (c_transfer) {
    p.push_back({pp, 1});
    dg = 0;
  }
  do {
    p.push_back({pp, dg});
    pp = std::max(pp / 2, 1);
  } while (pp != p.back().first);
  std::reverse(p.begin(), p.end());
  std::vector<LevelSpec> out;
  for (size_t i = 0; i + 1 < h.size(); ++i) out.push_back({h[i], p.front().first, p.front().second});
  for (auto q : p) out.push_back({h.back(), q.first, q.second});
  return out;
}
}  // namespace exg

// ============================================================================================
// multigrid
// ============================================================================================
template <class T>
static void level_eigen(MGLevel& L, const exg_mg_desc& d, cudaStream_t s) {
  // Lanczos estimate of lambda_max(D^-1 A) from CG on A x = b, b_i = (i mod 11) - mean
  // (deal.II PreconditionChebyshev::estimate_eigenvalues, chebyshev_smoother.h:149-210)
  long long n = L.n;
  std::vector<T> hb(n);
  double mean = 0;
  for (long long i = 0; i < n; ++i) {
    hb[i] = (T)(i % 11);
    mean += (double)hb[i];
  }
  mean /= (double)n;
  for (long long i = 0; i < n; ++i) hb[i] = hb[i] - (T)mean;
  T* b = (T*)dalloc(n * sizeof(T));
  T* x = (T*)dalloc(n * sizeof(T));
  T* r = (T*)dalloc(n * sizeof(T));
  T* z = (T*)dalloc(n * sizeof(T));
  T* p = (T*)dalloc(n * sizeof(T));
  T* v = (T*)dalloc(n * sizeof(T));
  EXG_CUDA(cudaMemcpyAsync(b, hb.data(), n * sizeof(T), cudaMemcpyHostToDevice, s));
  EXG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(T), s));
  Reduction red = Reduction::create();
  const T* dinv = (const T*)L.invd;
  auto A = [&](const T* in, T* out) { L.op->apply(in, out, 1, s); };
  auto P = [&](const T* in, T* out) -> double {
    if (L.bj) {
      L.bj->apply(in, out, s);
      dot<T>(in, out, n, red, 4, s);
    } else {
      precond_dot<T>(dinv, in, out, n, red, 4, s);
    }
    return read_slot(red, 4, s);
  };
  CGStats st = pcg_run<T>(A, P, b, x, n, 0.0, 1e-10, d.eig_iters, true, true, r, z, p, v, red, s);
  EXG_CUDA(cudaStreamSynchronize(s));
  red.destroy();
  for (T* ptr : {b, x, r, z, p, v}) cudaFree(ptr);
  std::vector<double> ev = tridiag_eigs(st.diag, st.offdiag);
  L.eig_its = st.its;
  L.lambda_max = ev.empty() ? 1.0 : ev.back();
  L.lambda_min = ev.empty() ? 1.0 : ev.front();
  double lmax = 1.2 * L.lambda_max;
  double alpha = d.smoothing_range > 1.0 ? lmax / d.smoothing_range : std::min(0.9 * lmax, L.lambda_min);
  L.delta = (lmax - alpha) * 0.5;
  L.theta = (lmax + alpha) * 0.5;
}

static TransferParams make_transfer(const MGLevel& c, const MGLevel& f) {
  TransferParams P{};
  P.is_h = c.N[0] != f.N[0];
  P.nf = f.degree + 1;
  P.nc = c.degree + 1;
  for (int e = 0; e < 3; ++e) {
    P.Nf[e] = f.N[e];
    P.Nc[e] = c.N[e];
  }
  // degree pairs with a compiled transfer kernel: h at k = 1, p from k to max(k / 2, 1)
  EXG_CHECK((P.nf == 2 && P.nc == 2) || (P.nf >= 3 && P.nf <= 9 && P.nc == (P.nf + 1) / 2), EXG_ERR_UNSUPPORTED,
            "unsupported multigrid transfer");
  std::vector<double> zc = gauss_lobatto(P.nc), zf = gauss_lobatto(P.nf);
  if (P.is_h) {
    for (int ch = 0; ch < 2; ++ch)
      for (int i = 0; i < P.nf; ++i)
        for (int j = 0; j < P.nc; ++j) P.P[ch][i * P.nc + j] = lagrange(zc, j, 0.5 * (ch + zf[i]));
  } else {
    for (int i = 0; i < P.nf; ++i)
      for (int j = 0; j < P.nc; ++j) P.P[0][i * P.nc + j] = P.P[1][i * P.nc + j] = lagrange(zc, j, zf[i]);
  }
  return P;
}

exg_mg::exg_mg(const exg_op& fine, const exg_mg_desc& d) : desc(d) {
  EXG_CHECK(d.mg_precision == EXG_PREC_F32 || d.mg_precision == EXG_PREC_F64, EXG_ERR_INVALID,
            "mg_precision must be EXG_PREC_F32 or EXG_PREC_F64");
  EXG_CHECK(d.cheb_degree >= 1 && d.eig_iters >= 1, EXG_ERR_INVALID, "bad smoother parameters");
  prec = d.mg_precision;
  coarse_prec = d.coarse_double ? EXG_PREC_F64 : prec;
  EXG_CHECK(d.mg_type == EXG_MG_PH || d.mg_type == EXG_MG_CPH, EXG_ERR_INVALID, "mg_type must be EXG_MG_PH or EXG_MG_CPH");
  // a continuous fine operator (the continuous discretization): the cphMG list without its DG top
  auto list = mg_level_list(fine.mesh.N, fine.degree, std::max(1, d.min_coarse_cells),
                            d.mg_type == EXG_MG_CPH || fine.continuous);
  if (fine.continuous) {
    list.pop_back();
    EXG_CHECK(fine.lat->mask.pin_first == (d.singular ? 1 : 0), EXG_ERR_INVALID,
              "the multigrid's singular flag must match the continuous operator's");
  }
  EXG_CHECK(list.size() <= 32, EXG_ERR_UNSUPPORTED, "too many levels");
  cudaStream_t s = nullptr;
  lv.resize(list.size());
  for (size_t l = 0; l < list.size(); ++l) {
    MGLevel& L = lv[l];
    for (int e = 0; e < 3; ++e) L.N[e] = list[l].N[e];
    L.degree = list[l].degree;
    L.dg = list[l].dg;
    MeshInfo m = fine.mesh;
    for (int e = 0; e < 3; ++e) {
      m.d.n_cells[e] = L.N[e];
      m.N[e] = L.N[e];
      m.h[e] = (m.d.hi[e] - m.d.lo[e]) / L.N[e];
    }
    if (L.dg)
      L.op.reset(new exg_op(m, L.degree, fine.ip, prec));
    else
      L.op = exg_op::continuous_level(m, L.degree, prec, d.singular != 0);
    L.n = L.op->n_dofs();
    if (L.op->cartesian && l > 0) L.op->tune(1, s, nullptr);  // autotuned launch variant per level
    size_t bytes = L.n * psize(prec);
    L.sol = dalloc(bytes);
    L.def = dalloc(bytes);
    L.t = dalloc(bytes);
    EXG_CUDA(cudaMemset(L.sol, 0, bytes));
    EXG_CUDA(cudaMemset(L.def, 0, bytes));
    if (l > 0) {
      L.tmp = dalloc(bytes);
      L.old = dalloc(bytes);
      L.invd = dalloc(bytes);
      L.op->diagonal(L.invd, true, s);
      if (d.smoother_preconditioner == 1) {
        EXG_CHECK(L.dg && L.op->cartesian, EXG_ERR_UNSUPPORTED,
                  "block-Jacobi smoothing is built for DG levels of Cartesian meshes (phMG)");
        L.bj = &L.op->block_jacobi(prec);
        L.ones = dalloc(bytes);
        L.zeros = dalloc(bytes);
        vec_fill(L.ones, prec, 1.0, L.n, s);
        EXG_CUDA(cudaMemsetAsync(L.zeros, 0, bytes, s));
      }
      if (prec == EXG_PREC_F32)
        level_eigen<float>(L, d, s);
      else
        level_eigen<double>(L, d, s);
      MGLevel& C = lv[l - 1];
      if (C.dg) {
        L.tr = make_transfer(C, L);
      } else {
        L.ltr.reset(new LatticeTransfer());
        if (L.dg)
          L.ltr->setup_dg(*C.op->lat, prec);
        else
          L.ltr->setup(*C.op->lat, *L.op->lat, prec);
      }
    } else {
      n_coarse = (int)L.n;
      EXG_CHECK(L.n <= 4096, EXG_ERR_UNSUPPORTED, "coarse level too large for the single-CTA coarse solver");
      MeshInfo mc = m;
      if (L.dg)
        coarse_op.reset(new exg_op(mc, L.degree, fine.ip, coarse_prec));
      else
        coarse_op = exg_op::continuous_level(mc, L.degree, coarse_prec, d.singular != 0);
      size_t cb = psize(coarse_prec);
      coarseA = dalloc((size_t)L.n * L.n * cb);
      void* eye = dalloc((size_t)L.n * L.n * cb);
      if (coarse_prec == EXG_PREC_F32)
        identity<float>((float*)eye, (int)L.n, s);
      else
        identity<double>((double*)eye, (int)L.n, s);
      coarse_op->apply(eye, coarseA, (int)L.n, s);
      EXG_CUDA(cudaDeviceSynchronize());
      cudaFree(eye);
      coarse_invd = dalloc(L.n * cb);
      coarse_op->diagonal(coarse_invd, true, s);
      coarse_x = dalloc(L.n * cb);
      EXG_CUDA(cudaMemset(coarse_x, 0, L.n * cb));
      its_dev = (long long*)dalloc(sizeof(long long));
      EXG_CUDA(cudaMemset(its_dev, 0, sizeof(long long)));
      if (prec == EXG_PREC_F32 && coarse_prec == EXG_PREC_F32)
        coarse_cg_prepare<float, float>(n_coarse);
      else if (prec == EXG_PREC_F32)
        coarse_cg_prepare<float, double>(n_coarse);
      else
        coarse_cg_prepare<double, double>(n_coarse);
    }
  }
  EXG_CUDA(cudaDeviceSynchronize());
  EXG_CUDA(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
}

exg_mg::~exg_mg() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  if (cap_stream) cudaStreamDestroy(cap_stream);
  for (auto& L : lv)
    for (void* p : {L.invd, L.sol, L.def, L.t, L.tmp, L.old, L.ones, L.zeros})
      if (p) cudaFree(p);
  for (void* p : {coarseA, coarse_invd, coarse_x, (void*)its_dev})
    if (p) cudaFree(p);
}

void exg_mg::smooth(int l, bool zero_start, cudaStream_t s) {
  MGLevel& L = lv[l];
  const int deg = desc.cheb_degree;
  auto upd = [&](int mode, double f1, double f2) {
    if (prec == EXG_PREC_F32)
      chebyshev_update<float>(mode, (float*)L.sol, (float*)L.old, (const float*)L.def, (const float*)L.tmp,
                              (const float*)L.invd, f1, f2, L.n, s);
    else
      chebyshev_update<double>(mode, (double*)L.sol, (double*)L.old, (const double*)L.def, (const double*)L.tmp,
                               (const double*)L.invd, f1, f2, L.n, s);
  };
  // fused: the operator kernel writes the new iterate into L.old, then the two buffers swap roles
  // (the previous iterate becomes 'old' without a copy).  The swaps are host bookkeeping, so a
  // captured graph replays the same buffer sequence every time.
  auto step = [&](int mode, double f1, double f2) {
    if (!desc.fuse_smoother) {
      L.op->apply(L.sol, L.tmp, 1, s);
      upd(mode, f1, f2);
      return;
    }
    PointEpilogue ep;
    ep.mode = mode;
    ep.old = L.old;
    ep.b = L.def;
    ep.d = L.invd;
    ep.out = L.old;
    ep.f1 = f1;
    ep.f2 = f2;
    L.op->apply(L.sol, nullptr, 1, s, ep);
    std::swap(L.sol, L.old);
  };
  if (L.bj) {
    // Chebyshev on block Jacobi: every step z = P^-1 (def - A sol) and the update with d = 1,
    // t = 0 in the shared point formula (pr = d (b - t) = z)
    auto bupd = [&](int mode, double f1, double f2) {
      if (prec == EXG_PREC_F32)
        chebyshev_update<float>(mode, (float*)L.sol, (float*)L.old, (const float*)L.t, (const float*)L.zeros,
                                (const float*)L.ones, f1, f2, L.n, s);
      else
        chebyshev_update<double>(mode, (double*)L.sol, (double*)L.old, (const double*)L.t, (const double*)L.zeros,
                                 (const double*)L.ones, f1, f2, L.n, s);
    };
    auto bstep = [&](int mode, double f1, double f2) {
      L.op->apply(L.sol, L.tmp, 1, s);
      if (prec == EXG_PREC_F32)
        rsub<float>((const float*)L.def, (float*)L.tmp, L.n, s);
      else
        rsub<double>((const double*)L.def, (double*)L.tmp, L.n, s);
      L.bj->apply(L.tmp, L.t, s);
      bupd(mode, f1, f2);
    };
    int bfirst;
    if (zero_start) {
      L.bj->apply(L.def, L.t, s);
      bupd(0, 0.0, 1.0 / L.theta);
      bfirst = 0;
    } else {
      bstep(1, 0.0, 1.0 / L.theta);
      bfirst = 1;
    }
    if (deg < 2 || std::fabs(L.delta) < 1e-40) return;
    double rk = L.delta / L.theta, sg = L.theta / L.delta;
    for (int k = 0; k < deg - 1; ++k) {
      double rkp = 1.0 / (2.0 * sg - rk);
      double f1 = rkp * rk, f2 = 2.0 * rkp / L.delta;
      rk = rkp;
      int idx = k + 1 + bfirst;
      bstep(idx == 1 ? 2 : 3, f1, f2);
    }
    return;
  }
  int first;
  if (zero_start) {
    upd(0, 0.0, 1.0 / L.theta);
    first = 0;
  } else {
    step(1, 0.0, 1.0 / L.theta);
    first = 1;
  }
  if (deg < 2 || std::fabs(L.delta) < 1e-40) return;
  double rhok = L.delta / L.theta, sigma = L.theta / L.delta;
  for (int k = 0; k < deg - 1; ++k) {
    double rhokp = 1.0 / (2.0 * sigma - rhok);
    double f1 = rhokp * rhok, f2 = 2.0 * rhokp / L.delta;
    rhok = rhokp;
    int idx = k + 1 + first;
    step(idx == 1 ? 2 : 3, f1, f2);
  }
}

void exg_mg::coarse_solve(cudaStream_t s) {
  MGLevel& L = lv[0];
  if (prec == EXG_PREC_F32 && coarse_prec == EXG_PREC_F32)
      coarse_cg<float, float>((const float*)coarseA, (const float*)coarse_invd, (const float*)L.def, (float*)L.sol,
                              (float*)coarse_x, n_coarse, desc.coarse_rel_tol, desc.coarse_abs_tol,
                              desc.coarse_max_iter, desc.singular, its_dev, s);
    else if (prec == EXG_PREC_F32)
      coarse_cg<float, double>((const double*)coarseA, (const double*)coarse_invd, (const float*)L.def,
                               (float*)L.sol, (double*)coarse_x, n_coarse, desc.coarse_rel_tol, desc.coarse_abs_tol,
                               desc.coarse_max_iter, desc.singular, its_dev, s);
    else
      coarse_cg<double, double>((const double*)coarseA, (const double*)coarse_invd, (const double*)L.def,
                                (double*)L.sol, (double*)coarse_x, n_coarse, desc.coarse_rel_tol,
                                desc.coarse_abs_tol, desc.coarse_max_iter, desc.singular, its_dev, s);
}

void exg_mg::v_cycle(int l, cudaStream_t s) {
  MGLevel& L = lv[l];
  auto mark = [&](int k) {
    if (tev) EXG_CUDA(cudaEventRecord((*tev)[4 * l + k], s));
  };
  mark(0);
  if (l == 0) {
    coarse_solve(s);
    mark(1);
    return;
  }
  MGLevel& C = lv[l - 1];
  smooth(l, true, s);
  if (desc.fuse_smoother) {  // t = def - A sol in the operator's store
    PointEpilogue ep;
    ep.mode = 4;
    ep.b = L.def;
    ep.out = L.t;
    L.op->apply(L.sol, nullptr, 1, s, ep);
  } else {
    L.op->apply(L.sol, L.t, 1, s);
    if (prec == EXG_PREC_F32)
      rsub<float>((const float*)L.def, (float*)L.t, L.n, s);
    else
      rsub<double>((const double*)L.def, (double*)L.t, L.n, s);
  }
  if (L.ltr)
    L.ltr->restrict_add(L.t, C.def, s);
  else if (prec == EXG_PREC_F32)
    restrict_add<float>(L.tr, (const float*)L.t, (float*)C.def, s);
  else
    restrict_add<double>(L.tr, (const double*)L.t, (double*)C.def, s);
  mark(1);
  v_cycle(l - 1, s);
  mark(2);
  if (L.ltr)
    L.ltr->prolongate_add(C.sol, L.sol, s);
  else if (prec == EXG_PREC_F32)
    prolongate_add<float>(L.tr, (const float*)C.sol, (float*)L.sol, s);
  else
    prolongate_add<double>(L.tr, (const double*)C.sol, (double*)L.sol, s);
  smooth(l, false, s);
  mark(3);
}

void exg_mg::run_vcycle(cudaStream_t s) {
  int top = (int)lv.size() - 1;
  for (int l = 0; l < top; ++l) EXG_CUDA(cudaMemsetAsync(lv[l].def, 0, lv[l].n * psize(prec), s));
  v_cycle(top, s);
}

void exg_mg::vmult(const double* src, double* dst, cudaStream_t s) {
  MGLevel& F = lv.back();
  vec_copy_convert(src, EXG_PREC_F64, F.def, prec, F.n, s);
  if (desc.use_graph) {
    if (!graph_exec) {
      // capture once on an internal stream (capture is not allowed on the legacy default stream)
      cudaEvent_t ev;
      EXG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      EXG_CUDA(cudaEventRecord(ev, s));
      EXG_CUDA(cudaStreamWaitEvent(cap_stream, ev, 0));
      EXG_CUDA(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
      run_vcycle(cap_stream);
      EXG_CUDA(cudaStreamEndCapture(cap_stream, &graph));
      EXG_CUDA(cudaGraphInstantiate(&graph_exec, graph, 0));
      EXG_CUDA(cudaEventDestroy(ev));
      graph_result = F.sol;  // every replay ends in the buffer the capture ended in
    }
    EXG_CUDA(cudaGraphLaunch(graph_exec, s));
    vec_copy_convert(graph_result, prec, dst, EXG_PREC_F64, F.n, s);
  } else {
    run_vcycle(s);
    vec_copy_convert(F.sol, prec, dst, EXG_PREC_F64, F.n, s);
  }
  ++vcycles;
}

void exg_mg::enqueue_vmult(const double* src, double* dst, cudaStream_t s) {
  MGLevel& F = lv.back();
  vec_copy_convert(src, EXG_PREC_F64, F.def, prec, F.n, s);
  run_vcycle(s);
  vec_copy_convert(F.sol, prec, dst, EXG_PREC_F64, F.n, s);
}

void exg_mg::timed_vmult(const double* src, double* dst, std::vector<float>& ms, cudaStream_t s) {
  const int nl = (int)lv.size();
  std::vector<cudaEvent_t> ev(4 * nl);
  for (auto& e : ev) EXG_CUDA(cudaEventCreate(&e));
  MGLevel& F = lv.back();
  vec_copy_convert(src, EXG_PREC_F64, F.def, prec, F.n, s);
  tev = &ev;
  try {
    run_vcycle(s);
  } catch (...) {
    tev = nullptr;
    for (auto& e : ev) cudaEventDestroy(e);
    throw;
  }
  tev = nullptr;
  vec_copy_convert(F.sol, prec, dst, EXG_PREC_F64, F.n, s);
  EXG_CUDA(cudaStreamSynchronize(s));
  ms.assign(nl, 0.0f);
  for (int l = 0; l < nl; ++l) {
    float a = 0, b = 0;
    EXG_CUDA(cudaEventElapsedTime(&a, ev[4 * l], ev[4 * l + 1]));
    if (l > 0) EXG_CUDA(cudaEventElapsedTime(&b, ev[4 * l + 2], ev[4 * l + 3]));
    ms[l] = a + b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  ++vcycles;
}

void exg_mg::level_apply(int l, const void* src, void* dst, cudaStream_t s) {
  EXG_CHECK(l >= 0 && l < (int)lv.size(), EXG_ERR_INVALID, "level out of range");
  lv[l].op->apply(src, dst, 1, s);
}

// SmootherBase::vmult (zero_start) / step on level l >= 1: the level's own work vectors are used
// and their roles restored afterwards, so a captured V-cycle graph stays valid
void exg_mg::level_smooth(int l, const void* rhs, void* x, bool zero_start, cudaStream_t s) {
  EXG_CHECK(l >= 1 && l < (int)lv.size(), EXG_ERR_INVALID, "smoothing levels are 1..n_levels-1");
  MGLevel& L = lv[l];
  const size_t bytes = (size_t)L.n * psize(prec);
  void* sol0 = L.sol;
  void* old0 = L.old;
  EXG_CUDA(cudaMemcpyAsync(L.def, rhs, bytes, cudaMemcpyDeviceToDevice, s));
  if (!zero_start) EXG_CUDA(cudaMemcpyAsync(L.sol, x, bytes, cudaMemcpyDeviceToDevice, s));
  smooth(l, zero_start, s);
  EXG_CUDA(cudaMemcpyAsync(x, L.sol, bytes, cudaMemcpyDeviceToDevice, s));
  L.sol = sol0;
  L.old = old0;
}

void exg_mg::level_restrict_add(int l, const void* fine, void* coarse, cudaStream_t s) {
  EXG_CHECK(l >= 1 && l < (int)lv.size(), EXG_ERR_INVALID, "transfers are between levels l-1 and l >= 1");
  MGLevel& L = lv[l];
  if (L.ltr)
    L.ltr->restrict_add(fine, coarse, s);
  else if (prec == EXG_PREC_F32)
    restrict_add<float>(L.tr, (const float*)fine, (float*)coarse, s);
  else
    restrict_add<double>(L.tr, (const double*)fine, (double*)coarse, s);
}

void exg_mg::level_prolongate_add(int l, const void* coarse, void* fine, cudaStream_t s) {
  EXG_CHECK(l >= 1 && l < (int)lv.size(), EXG_ERR_INVALID, "transfers are between levels l-1 and l >= 1");
  MGLevel& L = lv[l];
  if (L.ltr)
    L.ltr->prolongate_add(coarse, fine, s);
  else if (prec == EXG_PREC_F32)
    prolongate_add<float>(L.tr, (const float*)coarse, (float*)fine, s);
  else
    prolongate_add<double>(L.tr, (const double*)coarse, (double*)fine, s);
}

void exg_mg::coarse_solve_into(const void* src, void* dst, cudaStream_t s) {
  MGLevel& L = lv[0];
  const size_t bytes = (size_t)L.n * psize(prec);
  EXG_CUDA(cudaMemcpyAsync(L.def, src, bytes, cudaMemcpyDeviceToDevice, s));
  coarse_solve(s);
  EXG_CUDA(cudaMemcpyAsync(dst, L.sol, bytes, cudaMemcpyDeviceToDevice, s));
}

void exg_mg::info(exg_mg_info& out) const {
  std::memset(&out, 0, sizeof(out));
  out.n_levels = (int)lv.size();
  for (size_t l = 0; l < lv.size(); ++l) {
    out.degree[l] = lv[l].degree;
    for (int e = 0; e < 3; ++e) out.n_cells[l][e] = lv[l].N[e];
    out.lambda_max[l] = lv[l].lambda_max;
    out.eig_iters[l] = lv[l].eig_its;
    out.dg[l] = lv[l].dg;
  }
  long long its = 0;
  if (its_dev) cudaMemcpy(&its, its_dev, sizeof(long long), cudaMemcpyDeviceToHost);
  out.coarse_iterations = its;
  out.vcycles = vcycles;
}

// ============================================================================================
// outer CG
// ============================================================================================
// Graph-driven PCG: x and b are copied into fixed work vectors, the initial residual is checked
// on the host (as the host loop does), then one launch of a graph whose WHILE node repeats the
// captured iteration until cg_check_kernel reports convergence, the iteration cap or a
// non-finite residual.  The graph is captured on the first call with a given preconditioner.
static exg_status cg_solve_device(exg_op& op, exg_mg* mg, const exg_cg_desc& d, const double* b, double* x,
                                  exg_cg_result& res, cudaStream_t s) {
  const long long n = op.n_dofs();
  CGWorkspace& w = op.workspace();
  Reduction& red = w.red;
  if (!w.xw) {
    w.xw = (double*)dalloc(n * 8);
    w.bw = (double*)dalloc(n * 8);
    w.st = (CGDevState*)dalloc(sizeof(CGDevState));
    EXG_CUDA(cudaMallocHost(&w.st_host, sizeof(CGDevState)));
    EXG_CUDA(cudaStreamCreateWithFlags(&w.cap, cudaStreamNonBlocking));
  }
  const void* want_mg = d.precond == 2 ? (const void*)mg : nullptr;
  if (w.exec && (w.graph_mg != want_mg || w.graph_precond != d.precond)) {
    cudaGraphExecDestroy(w.exec);
    cudaGraphDestroy(w.graph);
    w.exec = nullptr;
    w.graph = nullptr;
  }
  const double* dinv = d.precond == 1 ? w.dinv : nullptr;
  if (!w.exec) {
    op.apply(w.r, w.v, 1, s);  // first launches (kernel attributes) happen outside the capture
    EXG_CUDA(cudaStreamSynchronize(s));
    EXG_CUDA(cudaGraphCreate(&w.graph, 0));
    cudaGraphConditionalHandle h;
    EXG_CUDA(cudaGraphConditionalHandleCreate(&h, w.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    EXG_CUDA(cudaGraphAddNode(&node, w.graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    EXG_CUDA(cudaStreamBeginCaptureToGraph(w.cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    double *r = w.r, *z = w.z, *p = w.p, *v = w.v;
    const double* out = red.out;
    if (d.precond == 2) {
      mg->enqueue_vmult(r, z, w.cap);
      dot<double>(r, z, n, red, 4, w.cap);
    } else if (d.precond == 3) {
      op.bj[1]->apply(r, z, w.cap);
      dot<double>(r, z, n, red, 4, w.cap);
    } else {
      precond_dot<double>(dinv, r, z, n, red, 4, w.cap);
    }
    cg_rho(w.st, out + 4, w.cap);
    cg_p_update(z, p, w.st, n, w.cap);
    op.apply(p, v, 1, w.cap);
    dot<double>(p, v, n, red, 2, w.cap);
    cg_alpha(w.st, out + 2, w.cap);
    xr_update_dev(w.xw, r, p, v, &w.st->alpha, n, red, 3, w.cap);
    cg_check(w.st, out + 3, h, w.cap);
    cudaGraph_t captured;
    EXG_CUDA(cudaStreamEndCapture(w.cap, &captured));
    EXG_CUDA(cudaGraphInstantiate(&w.exec, w.graph, 0));
    w.graph_mg = want_mg;
    w.graph_precond = d.precond;
  }
  EXG_CUDA(cudaStreamSynchronize(s));
  auto t0 = std::chrono::steady_clock::now();
  EXG_CUDA(cudaMemcpyAsync(w.xw, x, n * 8, cudaMemcpyDeviceToDevice, s));
  EXG_CUDA(cudaMemcpyAsync(w.bw, b, n * 8, cudaMemcpyDeviceToDevice, s));
  // initial residual, as pcg_run
  dot<double>(w.xw, w.xw, n, red, 0, s);
  const bool xzero = read_slot(red, 0, s) == 0.0;
  if (xzero) {
    residual<double>(w.bw, nullptr, w.r, n, red, 1, s);
  } else {
    op.apply(w.xw, w.v, 1, s);
    residual<double>(w.bw, w.v, w.r, n, red, 1, s);
  }
  const double r0 = std::sqrt(read_slot(red, 1, s));
  const double tol = std::max(d.abs_tol, d.rel_tol * r0);
  CGDevState& h = *w.st_host;
  h = CGDevState{};
  h.rn = r0;
  h.tol = tol;
  h.max_iter = d.max_iter;
  h.status = !std::isfinite(r0) ? 2 : (r0 <= tol ? 0 : (d.max_iter <= 0 ? 1 : -1));
  if (h.status < 0) {
    EXG_CUDA(cudaMemcpyAsync(w.st, &h, sizeof(CGDevState), cudaMemcpyHostToDevice, s));
    EXG_CUDA(cudaGraphLaunch(w.exec, s));
    EXG_CUDA(cudaMemcpyAsync(&h, w.st, sizeof(CGDevState), cudaMemcpyDeviceToHost, s));
  }
  EXG_CUDA(cudaMemcpyAsync(x, w.xw, n * 8, cudaMemcpyDeviceToDevice, s));
  EXG_CUDA(cudaStreamSynchronize(s));
  auto t1 = std::chrono::steady_clock::now();
  if (mg && d.precond == 2) mg->vcycles += h.it;
  res.iterations = h.it;
  res.converged = h.status == 0;
  res.r0 = r0;
  res.rn = h.rn;
  res.rho = h.it > 0 && r0 > 0 ? std::pow(h.rn / r0, 1.0 / h.it) : 0.0;
  res.n10 = (res.rho > 0 && res.rho < 1) ? -10.0 * std::log(10.0) / std::log(res.rho) : 0.0;
  res.seconds = std::chrono::duration<double>(t1 - t0).count();
  if (h.status == 2) return EXG_ERR_NONFINITE;
  if (h.status == 1) return EXG_ERR_NOT_CONVERGED;
  return EXG_OK;
}

exg_status exg::cg_solve(exg_op& op, exg_mg* mg, const exg_cg_desc& d, const double* b, double* x, exg_cg_result& res,
                         cudaStream_t s) {
  long long n = op.n_dofs();
  // work vectors live with the operator and are reused by later solves
  CGWorkspace& w = op.workspace();
  double *r = w.r, *z = w.z, *p = w.p, *v = w.v;
  Reduction& red = w.red;
  double* dinv = nullptr;
  if (d.precond == 1) {
    if (!w.dinv_valid) {
      op.diagonal(w.dinv, true, s);
      w.dinv_valid = true;
    }
    dinv = w.dinv;
  }
  if (d.precond == 3) op.block_jacobi(EXG_PREC_F64);  // FP64 work vectors; set up before any capture
  if (d.device_loop) return cg_solve_device(op, mg, d, b, x, res, s);
  EXG_CUDA(cudaStreamSynchronize(s));
  auto t0 = std::chrono::steady_clock::now();
  auto A = [&](const double* in, double* out) { op.apply(in, out, 1, s); };
  auto P = [&](const double* in, double* out) -> double {
    if (d.precond == 2) {
      mg->vmult(in, out, s);
      dot<double>(in, out, n, red, 4, s);
    } else if (d.precond == 3) {
      op.bj[1]->apply(in, out, s);
      dot<double>(in, out, n, red, 4, s);
    } else {
      precond_dot<double>(d.precond == 1 ? dinv : nullptr, in, out, n, red, 4, s);
    }
    return read_slot(red, 4, s);
  };
  CGStats st = pcg_run<double>(A, P, b, x, n, d.rel_tol, d.abs_tol, d.max_iter, false, false, r, z, p, v, red, s);
  EXG_CUDA(cudaStreamSynchronize(s));
  auto t1 = std::chrono::steady_clock::now();
  res.iterations = st.its;
  res.converged = st.status == 0;
  res.r0 = st.r0;
  res.rn = st.rn;
  res.rho = st.its > 0 && st.r0 > 0 ? std::pow(st.rn / st.r0, 1.0 / st.its) : 0.0;
  res.n10 = (res.rho > 0 && res.rho < 1) ? -10.0 * std::log(10.0) / std::log(res.rho) : 0.0;
  res.seconds = std::chrono::duration<double>(t1 - t0).count();
  if (st.status == 2) return EXG_ERR_NONFINITE;
  if (st.status == 1) return EXG_ERR_NOT_CONVERGED;
  return EXG_OK;
}
