// Dispatch, launch-variant list and diagonal of the affine SIPG operator (kernels in
// sipg_cartesian.cuh, instantiated per arithmetic in sipg_cart_{f64,f32,df64}.cu).
#include "sipg_cartesian.cuh"

namespace exg {

void cart_apply_f64(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                    const PointEpilogue& ep);
void cart_apply_f32(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                    const PointEpilogue& ep);
void cart_apply_df64(const CartHost& h, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                    const PointEpilogue& ep);

void cart_apply(const CartHost& h, int precision, const void* src, void* dst, int n_rhs, int cpb, cudaStream_t s,
                const PointEpilogue& ep) {
  EXG_CHECK(ep.mode < 0 || n_rhs == 1, EXG_ERR_INVALID, "fused point update needs a single right-hand side");
  if (precision == EXG_PREC_F64)
    cart_apply_f64(h, src, dst, n_rhs, cpb, s, ep);
  else if (precision == EXG_PREC_F32)
    cart_apply_f32(h, src, dst, n_rhs, cpb, s, ep);
  else if (precision == EXG_PREC_F64E)
    cart_apply_df64(h, src, dst, n_rhs, cpb, s, ep);
  else
    throw Error{EXG_ERR_INVALID, "unknown precision"};
}

// launch variants: > 0 cells per block in a row (neighbour lines from L1/L2), < 0 brick shapes
// with the halo staged in shared memory
template <int N>
static std::vector<int> cpb_list() {
  return {CpbChoice<N>::a, CpbChoice<N>::b, CpbChoice<N>::c, -1, -2};
}

std::vector<int> cart_cpb_options(int n, int) {
  switch (n) {
    case 2: return cpb_list<2>();
    case 3: return cpb_list<3>();
    case 4: return cpb_list<4>();
    case 5: return cpb_list<5>();
    case 6: return cpb_list<6>();
    case 7: return cpb_list<7>();
    case 8: return cpb_list<8>();
    case 9: return cpb_list<9>();
  }
  return {};
}

template <int N, class T, class C>
static void diag_n(const CartHost& h, void* diag, bool invert, cudaStream_t s) {
  CartCoef<N, C> P = make_coef<N, C>(h);
  long long blocks = (h.mesh.n_dofs + 255) / 256;
  cart_diag_kernel<N, T, C><<<(unsigned)blocks, 256, 0, s>>>((T*)diag, P, h.mesh, invert);
  EXG_CUDA(cudaGetLastError());
}

template <class T, class C>
static void diag_prec(const CartHost& h, void* diag, bool invert, cudaStream_t s) {
  switch (h.n) {
    case 2: diag_n<2, T, C>(h, diag, invert, s); break;
    case 3: diag_n<3, T, C>(h, diag, invert, s); break;
    case 4: diag_n<4, T, C>(h, diag, invert, s); break;
    case 5: diag_n<5, T, C>(h, diag, invert, s); break;
    case 6: diag_n<6, T, C>(h, diag, invert, s); break;
    case 7: diag_n<7, T, C>(h, diag, invert, s); break;
    case 8: diag_n<8, T, C>(h, diag, invert, s); break;
    case 9: diag_n<9, T, C>(h, diag, invert, s); break;
    default: throw Error{EXG_ERR_UNSUPPORTED, "degree must be 1..8"};
  }
}

void cart_diagonal(const CartHost& h, int precision, void* diag, bool invert, cudaStream_t s) {
  // the diagonal is computed in double and rounded once to the storage type
  if (precision == EXG_PREC_F32)
    diag_prec<float, double>(h, diag, invert, s);
  else
    diag_prec<double, double>(h, diag, invert, s);
}

}  // namespace exg
