// Davidson preconditioners (A12).
//
// The reference builds the diagonal preconditioner 1 / (theta - H_II) with one
// expectation value per determinant (algorithm/davidson.py:159-180, 273-280).
// Here the diagonal comes from fqegpu_diagonal (one Slater-Condon pass) and
// the preconditioned residual is formed in one streaming kernel:
//   t_I = m_I * r_I / (theta - H_II),   |theta - H_II| floored at `floor`,
// with m_I = 1 (diagonal preconditioner) or the output of a small MLP on the
// determinant's features (learned correction, mlp.cu).
#include "ham.cuh"

namespace fqegpu {

__global__ void k_precond_diag(int64_t n, const double2* __restrict__ r,
                               const double* __restrict__ diag, double theta,
                               double floor_, double2* __restrict__ t) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double den = theta - diag[i];
    if (fabs(den) < floor_) den = den < 0.0 ? -floor_ : floor_;
    const double inv = 1.0 / den;
    const double2 v = r[i];
    t[i] = make_double2(v.x * inv, v.y * inv);
  }
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_precondition(int64_t n, const double* d_r, const double* d_diag,
                                   double theta, double floor_, double* d_t, void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && d_r && d_diag && d_t, "NULL argument");
  FQE_CHECK_ARG(floor_ > 0.0, "floor must be positive");
  if (n == 0) return FQEGPU_OK;
  int64_t blocks = (n + 255) / 256;
  if (blocks > (int64_t)kNumSMs * 16) blocks = (int64_t)kNumSMs * 16;
  k_precond_diag<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      n, (const double2*)d_r, d_diag, theta, floor_, (double2*)d_t);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}
