// Host-side objects behind the C ABI handles.
#pragma once

#include <memory>
#include <vector>

#include "cg_device.h"
#include "general.h"
#include "internal.h"
#include "block_jacobi.h"
#include "lattice.h"
#include "solver_kernels.h"

struct exg_mesh {
  exg::MeshInfo info;
  explicit exg_mesh(const exg::MeshInfo& m) : info(m) {}
};

namespace exg {
MeshInfo make_mesh_info(const exg_mesh_desc& d);
}

namespace exg {
// CG work vectors kept with an operator between solves
struct CGWorkspace {
  double *r = nullptr, *z = nullptr, *p = nullptr, *v = nullptr, *dinv = nullptr;
  bool dinv_valid = false;
  Reduction red;
  // graph-driven loop: the iteration body captured under a WHILE node on fixed vectors
  double *xw = nullptr, *bw = nullptr;
  CGDevState* st = nullptr;
  CGDevState* st_host = nullptr;  // pinned
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* graph_mg = nullptr;  // preconditioner the graph was captured with
  int graph_precond = -1;
  ~CGWorkspace();
};

// device buffers, streams and events of the host-vector apply (exg_sipg_apply_host_f64)
struct HostPipe {
  double* src = nullptr;
  double* dst = nullptr;
  cudaStream_t in = nullptr, comp = nullptr, out = nullptr;
  std::vector<cudaEvent_t> loaded, done;
  cudaEvent_t start = nullptr, end = nullptr;
  ~HostPipe();
};
}  // namespace exg

// SIPG Laplace operator (Poisson::LaplaceOperator)
struct exg_op {
  exg::MeshInfo mesh;
  int degree, n;
  double ip;
  int precision;
  bool cartesian;
  exg::FE1D fe;
  exg::CartHost cart;
  int cpb = 0;  // Cartesian cells per block (0 = tuned default)
  std::unique_ptr<exg::GeneralGeom> geo;      // curved meshes
  std::unique_ptr<exg::GeneralGeom> rhs_geo;  // FP64 geometry with points (rhs / quadrature points)

  exg_op(const exg::MeshInfo& m, int degree, double ip, int precision);
  // continuous FE_Q(degree) Laplacian on the node lattice (a cphMG level; Cartesian meshes)
  static std::unique_ptr<exg_op> continuous_level(const exg::MeshInfo& m, int degree, int precision, bool singular);
  bool continuous = false;
  std::unique_ptr<exg::LatticeHost> lat;
  // curved continuous levels: two DG-layout work vectors around the cell-term apply
  struct DgScratch {
    void* v[2] = {nullptr, nullptr};
    ~DgScratch() {
      for (void* p : v)
        if (p) cudaFree(p);
    }
  };
  std::unique_ptr<DgScratch> cdg;
  // block Jacobi (Cartesian), one instance per precision (FP32, FP64) built on first use
  // (synchronous) and kept: captured graphs hold their device pointers
  std::unique_ptr<exg::BlockJacobi> bj[2];
  const exg::BlockJacobi& block_jacobi(int precision);
  long long n_dofs() const { return continuous ? lat->size() : mesh.n_cells() * n * n * n; }
  // dst = A src on the cells [cell_begin, cell_end) (cell_end < 0: all cells)
  void apply(const void* src, void* dst, int n_rhs, cudaStream_t s,
             const exg::PointEpilogue& ep = exg::PointEpilogue(), long long cell_begin = 0,
             long long cell_end = -1) const;
  // dst_host = A src_host for FP64 host vectors, copies pipelined against the apply by z-slabs
  void apply_host(const double* src_host, double* dst_host, int n_slabs, cudaStream_t s);
  void diagonal(void* d, bool invert, cudaStream_t s) const;
  void quadrature_points(double* cx, double* fx, long long* ncp, long long* nfp, cudaStream_t s);
  void rhs(const double* f, const double* g, const double* h, double* b, cudaStream_t s);
  void ensure_rhs_geometry(cudaStream_t s);
  int tune(int n_rhs, cudaStream_t s, std::vector<std::pair<int, float>>* timings);
  exg::CGWorkspace& workspace();
  std::unique_ptr<exg::CGWorkspace> ws;
  std::unique_ptr<exg::HostPipe> pipe;
};

namespace exg {
struct MGLevel {
  int N[3];
  int degree;
  int dg = 1;  // 0: continuous level (cphMG)
  std::unique_ptr<exg_op> op;
  long long n = 0;
  void* invd = nullptr;
  void* sol = nullptr;
  void* def = nullptr;
  void* t = nullptr;
  void* tmp = nullptr;
  void* old = nullptr;
  double theta = 1, delta = 0, lambda_max = 0, lambda_min = 0;
  int eig_its = 0;
  TransferParams tr{};  // transfer from level l-1 to l (l-1 discontinuous)
  std::unique_ptr<LatticeTransfer> ltr;  // transfer from a continuous level l-1
  const BlockJacobi* bj = nullptr;       // block-Jacobi smoothing: the level's block inverse
  void* ones = nullptr;                  // block-Jacobi smoothing: unit "diagonal" for the update
  void* zeros = nullptr;
};
}  // namespace exg

// multigrid preconditioner (MultigridPreconditionerBase + MultigridAlgorithm)
struct exg_mg {
  exg_mg_desc desc;
  int prec;  // level precision
  std::vector<exg::MGLevel> lv;
  int coarse_prec;
  std::unique_ptr<exg_op> coarse_op;
  void* coarseA = nullptr;
  void* coarse_invd = nullptr;
  void* coarse_x = nullptr;
  long long* its_dev = nullptr;
  int n_coarse = 0;
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  void* graph_result = nullptr;  // finest-level solution buffer the captured V-cycle ends in
  long long vcycles = 0;

  exg_mg(const exg_op& fine, const exg_mg_desc& d);
  ~exg_mg();
  void vmult(const double* src, double* dst, cudaStream_t s);
  // dst = V-cycle(src) enqueued without a graph launch, for capture into a larger graph
  void enqueue_vmult(const double* src, double* dst, cudaStream_t s);
  // one eager V-cycle with CUDA events around every level's work (smoothing, residual and
  // transfers on the way down and up; the coarse solve); ms[l] for l = 0 (coarse) .. n_levels-1
  void timed_vmult(const double* src, double* dst, std::vector<float>& ms, cudaStream_t s);
  void info(exg_mg_info& out) const;

  // the level objects behind the reference's component interfaces (level vectors in the
  // multigrid precision; level 0 = coarsest)
  void level_apply(int l, const void* src, void* dst, cudaStream_t s);
  void level_smooth(int l, const void* rhs, void* x, bool zero_start, cudaStream_t s);
  void level_restrict_add(int l, const void* fine, void* coarse, cudaStream_t s);
  void level_prolongate_add(int l, const void* coarse, void* fine, cudaStream_t s);
  void coarse_solve_into(const void* src, void* dst, cudaStream_t s);

 private:
  void coarse_solve(cudaStream_t s);  // lv[0].sol = coarse CG(lv[0].def)
  void v_cycle(int l, cudaStream_t s);
  std::vector<cudaEvent_t>* tev = nullptr;  // 4 events per level while timed_vmult runs
  void smooth(int l, bool zero_start, cudaStream_t s);
  void run_vcycle(cudaStream_t s);
};

namespace exg {
exg_status cg_solve(exg_op& op, exg_mg* mg, const exg_cg_desc& d, const double* b, double* x, exg_cg_result& r,
                    cudaStream_t s);
}
