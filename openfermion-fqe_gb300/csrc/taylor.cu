// Taylor propagator (A10): psi <- sum_k (-i t H)^k / k! psi.
//
// Reference: Wavefunction.apply_generated_unitary, 'taylor' branch
// (wavefunction.py:553-568): work = H' work; result += work / k!; stop when
// ||work|| / k! < accuracy; RuntimeError when `expansion` - 1 orders do not
// reach it; then the e_0 phase (wavefunction.py:605-606).  Here the work
// vectors, the axpy and the FP64 norm stay on the device; one 16-byte read per
// order brings the norm back for the stopping test.
#include <cmath>

#include "ham.cuh"

using namespace fqegpu;

extern "C" int fqegpu_taylor(fqegpu_ham h, double* d_psi, double time,
                             double e0_re, double e0_im, double accuracy,
                             int expansion, int precision, int* h_terms,
                             void* stream) {
  clear_error();
  FQE_CHECK_ARG(h && d_psi, "NULL argument");
  FQE_CHECK_ARG(expansion >= 1, "expansion must be >= 1");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = h->g->a.len * h->g->b.len;
  if (!h->d_vec) FQE_CUDA(cudaMalloc(&h->d_vec, sizeof(double2) * 2 * (size_t)N));
  if (!h->d_red) FQE_CUDA(cudaMalloc(&h->d_red, (size_t)dot_scratch_bytes()));
  double2* psi = (double2*)d_psi;
  double2* work = h->d_vec;
  double2* next = h->d_vec + N;
  FQE_CUDA(cudaMemcpyAsync(work, psi, sizeof(double2) * N, cudaMemcpyDeviceToDevice, st));
  const double2 alpha = make_double2(0.0, -time);
  const double2 zero = make_double2(0.0, 0.0);
  double inv_fact = 1.0;
  int order = 1;
  bool converged = false;
  double2* d_nrm = h->d_red + (dot_scratch_bytes() / (int)sizeof(double2) - 1);
  for (; order < expansion; ++order) {
    int s = fqegpu_apply(h, (const double*)work, (double*)next, alpha.x, alpha.y,
                         zero.x, zero.y, precision, stream);
    if (s != FQEGPU_OK) return s;
    double2* t = work;
    work = next;
    next = t;
    inv_fact /= (double)order;
    FQE_TRY(axpy_async(N, make_double2(inv_fact, 0.0), work, psi, st));
    FQE_TRY(dot_async(N, work, nullptr, h->d_red, d_nrm, st));
    double2 nrm2;
    FQE_CUDA(cudaMemcpyAsync(&nrm2, d_nrm, sizeof(double2), cudaMemcpyDeviceToHost, st));
    FQE_CUDA(cudaStreamSynchronize(st));
    if (!std::isfinite(nrm2.x)) {
      set_error("taylor: non-finite norm at order %d", order);
      return FQEGPU_ERR_NUMERIC;
    }
    if (std::sqrt(nrm2.x) * inv_fact < accuracy) {
      converged = true;
      break;
    }
  }
  if (h_terms) *h_terms = order;
  if (!converged) {
    set_error("maximum taylor expansion limit reached");
    return FQEGPU_ERR_NUMERIC;
  }
  if (std::hypot(e0_re * time, e0_im * time) > 1.0e-15) {
    // exp(-i t e0)
    const double re = e0_im * time, im = -e0_re * time;  // -i t e0
    const double m = std::exp(re);
    FQE_TRY(scale_async(N, make_double2(m * std::cos(im), m * std::sin(im)), psi, st));
  }
  return FQEGPU_OK;
}
