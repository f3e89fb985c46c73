// H·psi without any device allocation: fqegpu_apply_noalloc.
//
// Some callers cannot allocate device memory while they run: a host program
// whose device memory is owned by another allocator (a framework's caching
// allocator, a fixed arena sized up front) must not have a library reserve
// gigabytes behind its back, and cudaMalloc/cudaFree synchronise the device,
// which a latency-sensitive loop cannot afford.  For them this entry point
// computes the same FP64 apply as fqegpu_apply (gather -> pair contraction ->
// scatter, same kernels, same results) with every piece of device working
// memory — string tables, pair matrix, D and G blocks — carved out of one
// file-scope __device__ array of kNoAllocScratchBytes (64 MiB).  Every GPU that
// loads the library holds that array until the process exits.  The beta-column
// block width shrinks until D and G fit; sectors whose tables plus one column
// do not fit are rejected with FQEGPU_ERR_UNSUPPORTED.
//
// The array's device address is taken with cudaGetSymbolAddress at the first
// call on each device (with that device current); that first call should come
// before any stream capture.  All calls share the array and leave the last
// call's contents in it: calls that overlap on the GPU (different streams or
// host threads without ordering) race on it and must be serialised by the
// caller.
#include <complex>
#include <cfloat>
#include <mutex>
#include <vector>

#include "ham.cuh"

namespace fqegpu {

int64_t build_spin_into(int norb, int nele, void* mem, size_t bytes, cudaStream_t st,
                        SpinTables& t);
int launch_pairgemm(int P, int64_t ncol, const double* Vr, const double2* Vc,
                    const double2* D, double2* G, cudaStream_t st);
int launch_axpby(int64_t n, double2 beta, const double2* x, double2* y, cudaStream_t st);

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

int scratch_address(unsigned char** out) {
  int dev = 0;
  FQE_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device index %d out of range", dev);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    FQE_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return FQEGPU_OK;
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_apply_noalloc(int norb, int nalpha, int nbeta, const double* h_h1,
                                    const double* h_h2, const double* d_psi, double* d_sigma,
                                    double alpha_re, double alpha_im, double beta_re,
                                    double beta_im, void* stream) {
  clear_error();
  FQE_CHECK_ARG(norb >= 0 && norb <= 63, "norb must be in [0, 63]");
  FQE_CHECK_ARG(nalpha >= 0 && nalpha <= norb && nbeta >= 0 && nbeta <= norb,
                "electron counts must be in [0, norb]");
  FQE_CHECK_ARG(h_h2 != nullptr, "h2 is required (two-body operator)");
  FQE_CHECK_ARG(d_psi && d_sigma && d_psi != d_sigma, "psi and sigma must be distinct buffers");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t lena = binom_host(norb, nalpha), lenb = binom_host(norb, nbeta);
  const int64_t N = lena * lenb;
  const double2 alpha = make_double2(alpha_re, alpha_im), beta = make_double2(beta_re, beta_im);
  const double2* psi = reinterpret_cast<const double2*>(d_psi);
  double2* sigma = reinterpret_cast<double2*>(d_sigma);
  if (lena > 65535) {
    set_error("alpha string space of %lld exceeds the 65535 rows one launch covers",
              (long long)lena);
    return FQEGPU_ERR_UNSUPPORTED;
  }

  // the same pair matrix fqegpu_ham_create prepares (ham.cuh: prepare_pairs)
  PairMatrix hp;
  prepare_pairs(norb, nalpha + nbeta, reinterpret_cast<const zd*>(h_h1),
                reinterpret_cast<const zd*>(h_h2), hp);
  if (hp.zero) {
    FQE_TRY(launch_axpby(N, beta, psi, sigma, st));
    FQE_CUDA(cudaStreamSynchronize(st));  // synchronous on every path
    return FQEGPU_OK;
  }

  unsigned char* base = nullptr;
  FQE_TRY(scratch_address(&base));
  size_t used = 0;
  fqegpu_graph_s g;
  g.norb = norb;
  g.nalpha = nalpha;
  g.nbeta = nbeta;
  const int64_t ua = build_spin_into(norb, nalpha, base, kNoAllocScratchBytes, st, g.a);
  if (ua < 0) {
    set_error("sector (norb=%d, %d alpha, %d beta) needs more than the %zu-byte static scratch "
              "for its string tables", norb, nalpha, nbeta, kNoAllocScratchBytes);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  used = up256((size_t)ua);
  const int64_t ub = build_spin_into(norb, nbeta, base + used, kNoAllocScratchBytes - used, st, g.b);
  if (ub < 0) {
    set_error("sector (norb=%d, %d alpha, %d beta) needs more than the %zu-byte static scratch "
              "for its string tables", norb, nalpha, nbeta, kNoAllocScratchBytes);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  used += up256((size_t)ub);
  const int P = hp.P;
  const size_t vbytes = hp.real ? sizeof(double) * P * P : sizeof(double2) * P * P;
  const size_t per_col = 2 * (size_t)P * (size_t)lena * sizeof(double2);
  if (used + up256(vbytes) + per_col > kNoAllocScratchBytes) {
    set_error("sector (norb=%d, %d alpha, %d beta) needs %zu bytes for its tables and one "
              "beta column; the static scratch holds %zu", norb, nalpha, nbeta,
              used + up256(vbytes) + per_col, kNoAllocScratchBytes);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  void* dV = base + used;
  used += up256(vbytes);
  FQE_CUDA(cudaMemcpyAsync(dV, hp.real ? (const void*)hp.vr.data() : (const void*)hp.vc.data(),
                           vbytes, cudaMemcpyHostToDevice, st));
  int64_t w = (int64_t)((kNoAllocScratchBytes - used) / per_col);
  w = std::min<int64_t>(std::max<int64_t>(w, 1), lenb);
  double2* D = reinterpret_cast<double2*>(base + used);
  double2* G = D + (size_t)P * lena * w;
  const double2 al = make_double2(alpha.x * hp.phase.x - alpha.y * hp.phase.y,
                                  alpha.x * hp.phase.y + alpha.y * hp.phase.x);
  const bool single = w >= lenb;
  if (!single) FQE_TRY(launch_axpby(N, beta, psi, sigma, st));
  for (int64_t c0 = 0; c0 < lenb; c0 += w) {
    const int64_t wb = std::min<int64_t>(w, lenb - c0);
    const int32_t* ta = hp.compressed ? g.a.tab_tri : g.a.tab_full;
    const int32_t* tb = hp.compressed ? g.b.tab_tri : g.b.tab_full;
    FQE_TRY(launch_gather(&g, ta, tb, P, c0, wb, psi, D, st));
    FQE_TRY(launch_pairgemm(P, lena * wb, hp.real ? static_cast<const double*>(dV) : nullptr,
                            hp.real ? nullptr : static_cast<const double2*>(dV), D, G, st));
    FQE_TRY(launch_scatter(&g, ta, tb, P, c0, wb, G, psi, al, beta, single, sigma, st));
  }
  // hp's host buffers are read by the copy above; keep them alive until then
  FQE_CUDA(cudaStreamSynchronize(st));
  return FQEGPU_OK;
}
