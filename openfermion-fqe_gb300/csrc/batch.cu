// Many sectors' applies recorded into one CUDA graph.
//
// The reference applies sectors one after another from Python
// (Wavefunction._apply_array loops over the sectors, wavefunction.py:366-399),
// each call a separate native invocation.  For many small wavefunctions the
// launch and synchronisation overhead of one apply at a time dominates, so
// fqegpu_batch_create runs every (Hamiltonian, psi, sigma) apply once (which
// allocates workspaces and tensor-core plans), then records all of them into
// a CUDA graph of up to eight parallel branches (the applies of one handle in
// order on one branch); fqegpu_batch_launch replays the whole batch with one
// launch.  Buffers are fixed at creation (update their
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
  // Taylor batches: one device loop state per sector, their host copies
  // (pinned) and the series' expansion limit
  std::vector<void*> states;
  unsigned char* h_states = nullptr;
  int expansion = 0;
};

using namespace fqegpu;

namespace {

constexpr int kLanes = 8;  // parallel branches of a batch graph

int apply_one(fqegpu_ham h, const double* psi, double* sigma, double2 al, double2 be,
              int precision, cudaStream_t st) {
  if (precision == FQEGPU_PREC_FP64)
    return apply_fp64(h, (const double2*)psi, (double2*)sigma, al, be, st);
  return apply_ozaki(h, (const double2*)psi, (double2*)sigma, al, be, st);
}

}  // namespace

// Distinct handles of a batch (a handle may appear several times).
static std::vector<fqegpu_ham> distinct(const std::vector<fqegpu_ham>& hams) {
  std::vector<fqegpu_ham> seen;
  for (fqegpu_ham h : hams)
    if (std::find(seen.begin(), seen.end(), h) == seen.end()) seen.push_back(h);
  return seen;
}

extern "C" int fqegpu_batch_destroy(fqegpu_batch b) {
  if (!b) return FQEGPU_OK;
  if (b->exec) {
    // the graph may still run: it reads the handles' workspaces
    cudaGraphExecDestroy(b->exec);
    for (fqegpu_ham h : distinct(b->hams)) --h->live_graphs;
  }
  if (b->graph) cudaGraphDestroy(b->graph);
  for (void* p : b->states) cudaFree(p);
  if (b->h_states) cudaFreeHost(b->h_states);
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
  // entries may run concurrently: a sigma must not overlap another entry's
  // psi or sigma
  {
    auto span = [&](int i, const void* p) {
      const int64_t N = hams[i]->g->a.len * hams[i]->g->b.len;
      const char* c = static_cast<const char*>(p);
      return std::make_pair(c, c + sizeof(double2) * (size_t)N);
    };
    for (int i = 0; i < n; ++i) {
      const auto si = span(i, d_sigmas[i]);
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        const auto pj = span(j, d_psis[j]), sj = span(j, d_sigmas[j]);
        FQE_CHECK_ARG(si.second <= pj.first || pj.second <= si.first,
                      "a sigma of the batch overlaps another entry's psi");
        FQE_CHECK_ARG(si.second <= sj.first || sj.second <= si.first,
                      "two sigmas of the batch overlap");
      }
    }
  }
  const double2 al = make_double2(alpha_re, alpha_im), be = make_double2(beta_re, beta_im);
  cudaStream_t st = (cudaStream_t)stream;
  // one uncaptured pass: workspaces, plans and tables exist afterwards
  for (int i = 0; i < n; ++i) FQE_TRY(apply_one(hams[i], d_psis[i], d_sigmas[i], al, be, precision, st));
  FQE_CUDA(cudaStreamSynchronize(st));
  auto* b = new fqegpu_batch_s();
  b->precision = precision;
  b->hams.assign(hams, hams + n);
  // Parallel branches: every handle is given one of up to kLanes lanes (its
  // first appearance, round robin), and its applies run in order on that
  // lane — a handle's workspace is never used by two branches at once —
  // while small sectors of different handles run side by side.
  const std::vector<fqegpu_ham> hs = distinct(b->hams);
  const int lanes = std::min<int>(kLanes, (int)hs.size());
  std::vector<int> lane_of(n);
  for (int i = 0; i < n; ++i)
    lane_of[i] = (int)(std::find(hs.begin(), hs.end(), hams[i]) - hs.begin()) % lanes;
  cudaStream_t cs[kLanes] = {};
  cudaEvent_t fork = nullptr, joins[kLanes] = {};
  cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  for (int l = 0; l < lanes && e == cudaSuccess; ++l) {
    e = cudaStreamCreateWithFlags(&cs[l], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&joins[l], cudaEventDisableTiming);
  }
  int s = FQEGPU_OK;
  if (e == cudaSuccess) {
    std::vector<bool> timing(n);
    for (int i = 0; i < n; ++i) {
      timing[i] = hams[i]->timing;
      hams[i]->timing = false;
      hams[i]->defer_check = true;
    }
    e = cudaStreamBeginCapture(cs[0], cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      e = cudaEventRecord(fork, cs[0]);
      for (int l = 1; l < lanes && e == cudaSuccess; ++l) e = cudaStreamWaitEvent(cs[l], fork, 0);
      for (int i = 0; i < n && s == FQEGPU_OK && e == cudaSuccess; ++i)
        s = apply_one(hams[i], d_psis[i], d_sigmas[i], al, be, precision, cs[lane_of[i]]);
      for (int l = 1; l < lanes && e == cudaSuccess && s == FQEGPU_OK; ++l) {
        e = cudaEventRecord(joins[l], cs[l]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs[0], joins[l], 0);
      }
      cudaGraph_t g = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(cs[0], &g);
      b->graph = g;
      if (e2 != cudaSuccess && s == FQEGPU_OK && e == cudaSuccess) e = e2;
    }
    for (int i = 0; i < n; ++i) {
      hams[i]->defer_check = false;
      hams[i]->timing = timing[i];
    }
    if (e == cudaSuccess && s == FQEGPU_OK) {
      e = cudaGraphInstantiate(&b->exec, b->graph, 0);
      if (e != cudaSuccess) b->exec = nullptr;
    }
    if (b->exec)
      for (fqegpu_ham h : hs) ++h->live_graphs;
  }
  for (int l = 0; l < kLanes; ++l) {
    if (cs[l]) cudaStreamDestroy(cs[l]);
    if (joins[l]) cudaEventDestroy(joins[l]);
  }
  if (fork) cudaEventDestroy(fork);
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
  for (fqegpu_ham h : distinct(b->hams)) FQE_TRY(ozaki_check(h, (cudaStream_t)stream));
  return FQEGPU_OK;
}

// ---- Taylor series of many sectors in one graph ------------------------------
// Each sector's series is the device-resident loop of fqegpu_taylor (a WHILE
// conditional node whose body is one order); the sectors are spread over
// kLanes parallel branches of the graph, so small sectors overlap on the GPU.
// The handles must be distinct (each series uses its handle's work vectors).

extern "C" int fqegpu_batch_taylor_create(int n, const fqegpu_ham* hams, double* const* d_psis,
                                          double time, double accuracy, int expansion,
                                          int precision, void* stream, fqegpu_batch* out) {
  clear_error();
  FQE_CHECK_ARG(out && n > 0 && hams && d_psis, "bad batch arguments");
  FQE_CHECK_ARG(precision == FQEGPU_PREC_FP64 || precision == FQEGPU_PREC_OZAKI,
                "unknown precision");
  FQE_CHECK_ARG(expansion >= 1, "expansion must be >= 1");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    FQE_CHECK_ARG(hams[i] && d_psis[i], "NULL entry in the batch");
    for (int j = 0; j < i; ++j)
      FQE_CHECK_ARG(hams[j] != hams[i], "a Taylor batch needs one handle per sector");
  }
  auto* b = new (std::nothrow) fqegpu_batch_s();
  if (!b) {
    set_error("host allocation failed");
    return FQEGPU_ERR_NOMEM;
  }
  b->precision = precision;
  b->expansion = expansion;
  b->hams.assign(hams, hams + n);
  int s = FQEGPU_OK;
  // workspaces, plans, work vectors and loop states exist before the capture
  for (int i = 0; i < n && s == FQEGPU_OK; ++i) {
    fqegpu_ham h = hams[i];
    const int64_t N = h->g->a.len * h->g->b.len;
    if (!h->d_vec && dev_alloc(&h->d_vec, sizeof(double2) * 2 * (size_t)N) != cudaSuccess) {
      set_error("device allocation of %lld bytes failed", (long long)(32 * N));
      s = FQEGPU_ERR_NOMEM;
      break;
    }
    s = apply_prepare(h, precision);
    void* st = nullptr;
    if (s == FQEGPU_OK && dev_alloc(&st, taylor_state_bytes()) != cudaSuccess) {
      set_error("device allocation failed");
      s = FQEGPU_ERR_NOMEM;
    }
    if (st) b->states.push_back(st);
  }
  if (s == FQEGPU_OK &&
      cudaHostAlloc(&b->h_states, kTaylorStateHostBytes * (size_t)n, cudaHostAllocDefault) !=
          cudaSuccess) {
    set_error("pinned host allocation failed");
    s = FQEGPU_ERR_NOMEM;
  }
  if (s != FQEGPU_OK) {
    fqegpu_batch_destroy(b);
    return s;
  }
  cudaStream_t cs[kLanes] = {};
  cudaStream_t bs = nullptr;  // loop bodies are captured here, one after another
  cudaEvent_t fork = nullptr, joins[kLanes] = {};
  cudaError_t e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
  for (int l = 0; l < kLanes && e == cudaSuccess; ++l) {
    e = cudaStreamCreateWithFlags(&cs[l], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&joins[l], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  std::vector<bool> timing(n);
  for (int i = 0; i < n; ++i) {
    timing[i] = hams[i]->timing;
    hams[i]->timing = false;
    hams[i]->defer_check = true;
  }
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs[0], cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const int lanes = std::min(kLanes, n);
    e = cudaEventRecord(fork, cs[0]);
    for (int l = 1; l < lanes && e == cudaSuccess; ++l) e = cudaStreamWaitEvent(cs[l], fork, 0);
    for (int i = 0; i < n && s == FQEGPU_OK && e == cudaSuccess; ++i)
      s = taylor_record(hams[i], (double2*)d_psis[i], time, accuracy, expansion, precision,
                        b->states[i], cs[i % lanes], bs);
    for (int l = 1; l < lanes && e == cudaSuccess && s == FQEGPU_OK; ++l) {
      e = cudaEventRecord(joins[l], cs[l]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(cs[0], joins[l], 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs[0], &g);
    b->graph = g;
    if (e == cudaSuccess) e = e2;
  }
  for (int i = 0; i < n; ++i) {
    hams[i]->timing = timing[i];
    hams[i]->defer_check = false;
  }
  if (e == cudaSuccess && s == FQEGPU_OK) {
    e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) b->exec = nullptr;
  }
  if (b->exec)
    for (fqegpu_ham h : distinct(b->hams)) ++h->live_graphs;
  for (int l = 0; l < kLanes; ++l) {
    if (cs[l]) cudaStreamDestroy(cs[l]);
    if (joins[l]) cudaEventDestroy(joins[l]);
  }
  if (fork) cudaEventDestroy(fork);
  if (bs) cudaStreamDestroy(bs);
  if (s != FQEGPU_OK || e != cudaSuccess) {
    if (s == FQEGPU_OK) {
      set_error("Taylor batch capture: %s", cudaGetErrorString(e));
      s = FQEGPU_ERR_CUDA;
    }
    fqegpu_batch_destroy(b);
    return s;
  }
  (void)stream;
  *out = b;
  return FQEGPU_OK;
}

extern "C" int fqegpu_batch_taylor_terms(fqegpu_batch b, int* h_terms, void* stream) {
  clear_error();
  FQE_CHECK_ARG(b && !b->states.empty(), "not a Taylor batch");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = b->states.size();
  for (size_t i = 0; i < n; ++i)
    FQE_CUDA(cudaMemcpyAsync(b->h_states + kTaylorStateHostBytes * i, b->states[i],
                             kTaylorStateHostBytes, cudaMemcpyDeviceToHost, st));
  FQE_CUDA(cudaStreamSynchronize(st));
  if (b->precision == FQEGPU_PREC_OZAKI)
    for (fqegpu_ham h : distinct(b->hams)) FQE_TRY(ozaki_check(h, st));
  int status = FQEGPU_OK;
  for (size_t i = 0; i < n; ++i) {
    int terms = 0;
    const int r = taylor_result(b->h_states + kTaylorStateHostBytes * i, b->expansion, &terms);
    if (h_terms) h_terms[i] = terms;
    if (r != FQEGPU_OK && status == FQEGPU_OK) status = r;
  }
  return status;
}
