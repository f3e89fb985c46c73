// Many sectors' applies recorded into one CUDA graph.
//
// The reference applies sectors one after another from Python
// (Wavefunction._apply_array loops over the sectors, wavefunction.py:366-399),
// each call a separate native invocation.  For many small wavefunctions the
// launch and synchronisation overhead of one apply at a time dominates, so
// fqegpu_batch_create runs every (Hamiltonian, psi, sigma) apply once (which
// allocates workspaces and tensor-core plans), then records all of them, in
// order, on one stream into a CUDA graph; fqegpu_batch_launch replays the
// whole batch with one launch.  Buffers are fixed at creation (update their
// contents between launches).  The tensor-core path's end-of-apply error
// readback is deferred to fqegpu_batch_check.
#include <algorithm>
#include <vector>

#include "ham.cuh"

struct fqegpu_batch_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<fqegpu_ham> hams;
  int precision = 0;
};

using namespace fqegpu;

namespace {

int apply_one(fqegpu_ham h, const double* psi, double* sigma, double2 al, double2 be,
              int precision, cudaStream_t st) {
  if (precision == FQEGPU_PREC_FP64)
    return apply_fp64(h, (const double2*)psi, (double2*)sigma, al, be, st);
  return apply_ozaki(h, (const double2*)psi, (double2*)sigma, al, be, st);
}

}  // namespace

extern "C" int fqegpu_batch_destroy(fqegpu_batch b) {
  if (!b) return FQEGPU_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  delete b;
  return FQEGPU_OK;
}

extern "C" int fqegpu_batch_create(int n, const fqegpu_ham* hams, const double* const* d_psis,
                                   double* const* d_sigmas, double alpha_re, double alpha_im,
                                   double beta_re, double beta_im, int precision, void* stream,
                                   fqegpu_batch* out) {
  clear_error();
  FQE_CHECK_ARG(out && n > 0 && hams && d_psis && d_sigmas, "bad batch arguments");
  FQE_CHECK_ARG(precision == FQEGPU_PREC_FP64 || precision == FQEGPU_PREC_OZAKI,
                "unknown precision");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    FQE_CHECK_ARG(hams[i] && d_psis[i] && d_sigmas[i], "NULL entry in the batch");
    FQE_CHECK_ARG((const void*)d_psis[i] != (const void*)d_sigmas[i],
                  "psi and sigma must not alias");
  }
  const double2 al = make_double2(alpha_re, alpha_im), be = make_double2(beta_re, beta_im);
  cudaStream_t st = (cudaStream_t)stream;
  // one uncaptured pass: workspaces, plans and tables exist afterwards
  for (int i = 0; i < n; ++i) FQE_TRY(apply_one(hams[i], d_psis[i], d_sigmas[i], al, be, precision, st));
  FQE_CUDA(cudaStreamSynchronize(st));
  auto* b = new fqegpu_batch_s();
  b->precision = precision;
  b->hams.assign(hams, hams + n);
  cudaStream_t cs = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  int s = FQEGPU_OK;
  if (e == cudaSuccess) {
    for (int i = 0; i < n; ++i) hams[i]->defer_check = true;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      for (int i = 0; i < n && s == FQEGPU_OK; ++i)
        s = apply_one(hams[i], d_psis[i], d_sigmas[i], al, be, precision, cs);
      cudaGraph_t g = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
      b->graph = g;
      if (e2 != cudaSuccess && s == FQEGPU_OK) e = e2;
    }
    for (int i = 0; i < n; ++i) hams[i]->defer_check = false;
    if (e == cudaSuccess && s == FQEGPU_OK) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    cudaStreamDestroy(cs);
  }
  if (s != FQEGPU_OK || e != cudaSuccess) {
    if (s == FQEGPU_OK) {
      set_error("batch capture: %s", cudaGetErrorString(e));
      s = FQEGPU_ERR_CUDA;
    }
    fqegpu_batch_destroy(b);
    return s;
  }
  *out = b;
  return FQEGPU_OK;
}

extern "C" int fqegpu_batch_launch(fqegpu_batch b, void* stream) {
  clear_error();
  FQE_CHECK_ARG(b && b->exec, "NULL batch");
  FQE_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return FQEGPU_OK;
}

extern "C" int fqegpu_batch_check(fqegpu_batch b, void* stream) {
  clear_error();
  FQE_CHECK_ARG(b, "NULL batch");
  FQE_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (b->precision != FQEGPU_PREC_OZAKI) return FQEGPU_OK;
  std::vector<fqegpu_ham> seen;
  for (fqegpu_ham h : b->hams) {
    if (std::find(seen.begin(), seen.end(), h) != seen.end()) continue;
    seen.push_back(h);
    int32_t flag = 0;
    FQE_TRY(ozaki_error_flag(h, &flag));
    if (flag != 0) {
      set_error("tensor-core contraction in a batch: a bounded wait gave up (role %d)", flag);
      return FQEGPU_ERR_TIMEOUT;
    }
  }
  return FQEGPU_OK;
}
