// C ABI of the library (include/exadg_gb300.h).  Every entry point catches all exceptions and
// returns a status; the message of the last failure is kept per host thread.
#include <algorithm>
#include <cstring>
#include <string>

#include "internal.h"
#include "host.h"

namespace exg {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace exg

using namespace exg;

#define EXG_API_BEGIN try {
#define EXG_API_END                        \
  }                                        \
  catch (const exg::Error& e) {            \
    set_error(e.msg);                      \
    return e.status;                       \
  }                                        \
  catch (const std::exception& e) {        \
    set_error(e.what());                   \
    return EXG_ERR_INVALID;                \
  }                                        \
  catch (...) {                            \
    set_error("unknown error");            \
    return EXG_ERR_INVALID;                \
  }                                        \
  return EXG_OK;

extern "C" {

const char* exg_status_string(exg_status s) {
  switch (s) {
    case EXG_OK: return "ok";
    case EXG_ERR_INVALID: return "invalid argument";
    case EXG_ERR_CUDA: return "CUDA error";
    case EXG_ERR_NOT_CONVERGED: return "solver did not converge";
    case EXG_ERR_NONFINITE: return "non-finite residual";
    case EXG_ERR_UNSUPPORTED: return "unsupported configuration";
    case EXG_ERR_NEEDS_UPDATE: return "preconditioner needs update";
  }
  return "unknown status";
}

const char* exg_last_error(void) { return g_last_error.c_str(); }

exg_status exg_device_fma_peaks(double* f64_tflops, double* f32_tflops, void* stream) {
  EXG_API_BEGIN
  device_fma_peaks(f64_tflops, f32_tflops, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mesh_create(const exg_mesh_desc* desc, exg_mesh** mesh) {
  EXG_API_BEGIN
  EXG_CHECK(desc && mesh, EXG_ERR_INVALID, "null argument");
  *mesh = new exg_mesh(make_mesh_info(*desc));
  EXG_API_END
}

exg_status exg_mesh_destroy(exg_mesh* mesh) {
  EXG_API_BEGIN
  delete mesh;
  EXG_API_END
}

exg_status exg_sipg_create(const exg_mesh* mesh, int degree, double ip_factor, int precision, exg_op** op) {
  EXG_API_BEGIN
  EXG_CHECK(mesh && op, EXG_ERR_INVALID, "null argument");
  *op = new exg_op(mesh->info, degree, ip_factor, precision);
  EXG_API_END
}

exg_status exg_continuous_create(const exg_mesh* mesh, int degree, int precision, int singular, exg_op** op) {
  EXG_API_BEGIN
  EXG_CHECK(mesh && op, EXG_ERR_INVALID, "null argument");
  *op = exg_op::continuous_level(mesh->info, degree, precision, singular != 0).release();
  EXG_API_END
}

exg_status exg_sipg_destroy(exg_op* op) {
  EXG_API_BEGIN
  delete op;
  EXG_API_END
}

exg_status exg_sipg_n_dofs(const exg_op* op, long long* n) {
  EXG_API_BEGIN
  EXG_CHECK(op && n, EXG_ERR_INVALID, "null argument");
  *n = op->n_dofs();
  EXG_API_END
}

exg_status exg_sipg_info(const exg_op* op, int* degree, int* precision, int* cartesian) {
  EXG_API_BEGIN
  EXG_CHECK(op, EXG_ERR_INVALID, "null argument");
  if (degree) *degree = op->degree;
  if (precision) *precision = op->precision;
  if (cartesian) *cartesian = op->cartesian ? 1 : 0;
  EXG_API_END
}

exg_status exg_sipg_apply_f64(exg_op* op, const double* src, double* dst, int n_rhs, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && src && dst, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision != EXG_PREC_F32, EXG_ERR_INVALID, "operator precision is FP32: use exg_sipg_apply_f32");
  EXG_CHECK(src != dst, EXG_ERR_INVALID, "src and dst must not alias");
  op->apply(src, dst, n_rhs, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_sipg_apply_f32(exg_op* op, const float* src, float* dst, int n_rhs, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && src && dst, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision == EXG_PREC_F32, EXG_ERR_INVALID, "operator precision is FP64: use exg_sipg_apply_f64");
  EXG_CHECK(src != dst, EXG_ERR_INVALID, "src and dst must not alias");
  op->apply(src, dst, n_rhs, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_sipg_apply_host_f64(exg_op* op, const double* src_host, double* dst_host, int n_slabs,
                                   void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && src_host && dst_host, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(src_host != dst_host, EXG_ERR_INVALID, "src and dst must not alias");
  EXG_CHECK(n_slabs >= 1, EXG_ERR_INVALID, "n_slabs must be >= 1");
  op->apply_host(src_host, dst_host, n_slabs, (cudaStream_t)stream);
  EXG_API_END
}

static exg_status block_jacobi_apply(exg_op* op, const void* src, void* dst, int prec, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && src && dst && src != dst, EXG_ERR_INVALID, "null or aliased argument");
  op->block_jacobi(prec).apply(src, dst, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_sipg_apply_inverse_block_diagonal_f64(exg_op* op, const double* src, double* dst, void* stream) {
  return block_jacobi_apply(op, src, dst, EXG_PREC_F64, stream);
}

exg_status exg_sipg_apply_inverse_block_diagonal_f32(exg_op* op, const float* src, float* dst, void* stream) {
  return block_jacobi_apply(op, src, dst, EXG_PREC_F32, stream);
}

exg_status exg_sipg_residual_f64(exg_op* op, const double* b, const double* x, double* r, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && b && x && r, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision != EXG_PREC_F32, EXG_ERR_INVALID, "operator precision is FP32");
  EXG_CHECK(x != r, EXG_ERR_INVALID, "x and r must not alias");
  exg::PointEpilogue ep;
  ep.mode = 4;
  ep.b = b;
  ep.out = r;
  op->apply(x, nullptr, 1, (cudaStream_t)stream, ep);
  EXG_API_END
}

exg_status exg_sipg_tune(exg_op* op, int n_rhs, int* launch_config, float* timings_ms, int* n_timings,
                         void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(n_rhs >= 1 && n_rhs <= 65535, EXG_ERR_INVALID, "n_rhs out of range");
  std::vector<std::pair<int, float>> t;
  int best = op->tune(n_rhs, (cudaStream_t)stream, &t);
  if (launch_config) *launch_config = best;
  if (n_timings) {
    int cap = *n_timings;
    *n_timings = (int)t.size();
    for (int i = 0; i < (int)t.size() && i < cap && timings_ms; ++i) {
      timings_ms[2 * i] = (float)t[i].first;
      timings_ms[2 * i + 1] = t[i].second;
    }
  }
  EXG_API_END
}

exg_status exg_sipg_set_launch_config(exg_op* op, int launch_config) {
  EXG_API_BEGIN
  EXG_CHECK(op, EXG_ERR_INVALID, "null argument");
  std::vector<int> o = cart_cpb_options(op->n, op->precision);
  EXG_CHECK(launch_config == 0 || std::find(o.begin(), o.end(), launch_config) != o.end(), EXG_ERR_INVALID,
            "launch_config is not one of the tuned cells-per-block values");
  op->cpb = launch_config;
  EXG_API_END
}

exg_status exg_sipg_inverse_diagonal_f64(exg_op* op, double* d, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && d, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision != EXG_PREC_F32, EXG_ERR_INVALID, "operator precision is FP32");
  op->diagonal(d, true, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_sipg_inverse_diagonal_f32(exg_op* op, float* d, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && d, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision == EXG_PREC_F32, EXG_ERR_INVALID, "operator precision is FP64");
  op->diagonal(d, true, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_sipg_quadrature_points(exg_op* op, double* cell_xyz, double* face_xyz, long long* n_cell_pts,
                                      long long* n_face_pts, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op, EXG_ERR_INVALID, "null argument");
  op->quadrature_points(cell_xyz, face_xyz, n_cell_pts, n_face_pts, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_sipg_rhs(exg_op* op, const double* f_cell, const double* g_face, const double* h_face, double* b,
                        void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(op && b, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision != EXG_PREC_F32, EXG_ERR_INVALID, "rhs is assembled by FP64 operators");
  op->rhs(f_cell, g_face, h_face, b, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_default_desc(exg_mg_desc* d) {
  EXG_API_BEGIN
  EXG_CHECK(d, EXG_ERR_INVALID, "null argument");
  std::memset(d, 0, sizeof(*d));
  d->mg_precision = EXG_PREC_F32;
  d->cheb_degree = 5;
  d->smoothing_range = 20.0;
  d->eig_iters = 20;
  d->coarse_rel_tol = 1e-3;
  d->coarse_abs_tol = 1e-12;
  d->coarse_max_iter = 10000;
  d->coarse_double = 0;
  d->min_coarse_cells = 2;
  d->singular = 0;
  d->use_graph = 1;
  d->fuse_smoother = 1;
  d->mg_type = EXG_MG_PH;
  d->smoother_preconditioner = 0;
  EXG_API_END
}

exg_status exg_mg_create(const exg_op* fine, const exg_mg_desc* desc, exg_mg** mg) {
  EXG_API_BEGIN
  EXG_CHECK(fine && desc && mg, EXG_ERR_INVALID, "null argument");
  *mg = new exg_mg(*fine, *desc);
  EXG_API_END
}

exg_status exg_mg_destroy(exg_mg* mg) {
  EXG_API_BEGIN
  delete mg;
  EXG_API_END
}

exg_status exg_mg_vmult(exg_mg* mg, const double* src, double* dst, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && src && dst, EXG_ERR_INVALID, "null argument");
  mg->vmult(src, dst, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_level_timings(exg_mg* mg, const double* src, double* dst, float* ms, int capacity,
                                int* n_levels, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && src && dst && n_levels, EXG_ERR_INVALID, "null argument");
  std::vector<float> t;
  mg->timed_vmult(src, dst, t, (cudaStream_t)stream);
  *n_levels = (int)t.size();
  for (int l = 0; l < (int)t.size() && l < capacity && ms; ++l) ms[l] = t[l];
  EXG_API_END
}

exg_status exg_mg_level_n_dofs(const exg_mg* mg, int level, long long* n_dofs, int* is_dg) {
  EXG_API_BEGIN
  EXG_CHECK(mg && n_dofs, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(level >= 0 && level < (int)mg->lv.size(), EXG_ERR_INVALID, "level out of range");
  *n_dofs = mg->lv[level].n;
  if (is_dg) *is_dg = mg->lv[level].dg;
  EXG_API_END
}

exg_status exg_mg_level_apply(exg_mg* mg, int level, const void* src, void* dst, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && src && dst && src != dst, EXG_ERR_INVALID, "null or aliased argument");
  mg->level_apply(level, src, dst, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_smooth(exg_mg* mg, int level, const void* rhs, void* x, int zero_start, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && rhs && x && rhs != x, EXG_ERR_INVALID, "null or aliased argument");
  mg->level_smooth(level, rhs, x, zero_start != 0, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_restrict_add(exg_mg* mg, int level, const void* fine, void* coarse, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && fine && coarse, EXG_ERR_INVALID, "null argument");
  mg->level_restrict_add(level, fine, coarse, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_prolongate_add(exg_mg* mg, int level, const void* coarse, void* fine, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && fine && coarse, EXG_ERR_INVALID, "null argument");
  mg->level_prolongate_add(level, coarse, fine, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_coarse_solve(exg_mg* mg, const void* src, void* dst, void* stream) {
  EXG_API_BEGIN
  EXG_CHECK(mg && src && dst && src != dst, EXG_ERR_INVALID, "null or aliased argument");
  mg->coarse_solve_into(src, dst, (cudaStream_t)stream);
  EXG_API_END
}

exg_status exg_mg_info_get(const exg_mg* mg, exg_mg_info* info) {
  EXG_API_BEGIN
  EXG_CHECK(mg && info, EXG_ERR_INVALID, "null argument");
  mg->info(*info);
  EXG_API_END
}

exg_status exg_cg_default_desc(exg_cg_desc* d) {
  EXG_API_BEGIN
  EXG_CHECK(d, EXG_ERR_INVALID, "null argument");
  d->max_iter = 10000;
  d->abs_tol = 1e-20;
  d->rel_tol = 1e-10;
  d->precond = 2;
  d->device_loop = 1;
  EXG_API_END
}

exg_status exg_cg_solve(exg_op* op, exg_mg* mg, const exg_cg_desc* desc, const double* b, double* x,
                        exg_cg_result* result, void* stream) {
  exg_status st = EXG_OK;
  EXG_API_BEGIN
  EXG_CHECK(op && desc && b && x, EXG_ERR_INVALID, "null argument");
  EXG_CHECK(op->precision != EXG_PREC_F32, EXG_ERR_INVALID, "outer CG runs on an FP64 operator");
  EXG_CHECK(desc->precond != 2 || mg, EXG_ERR_INVALID, "multigrid preconditioner requested but mg is NULL");
  EXG_CHECK(desc->precond >= 0 && desc->precond <= 3, EXG_ERR_INVALID, "unknown preconditioner");
  exg_cg_result r{};
  st = cg_solve(*op, desc->precond == 2 ? mg : nullptr, *desc, b, x, r, (cudaStream_t)stream);
  if (result) *result = r;
  if (st != EXG_OK) set_error(exg_status_string(st));
  return st;
  EXG_API_END
}

}  // extern "C"
