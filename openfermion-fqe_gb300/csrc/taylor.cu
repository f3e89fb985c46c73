// Taylor propagator (A10): psi <- sum_k (-i t H)^k / k! psi, on the device.
//
// Reference: Wavefunction.apply_generated_unitary, 'taylor' branch
// (wavefunction.py:553-568): work = H' work; result += work / k!; stop when
// ||work|| / k! < accuracy; RuntimeError when `expansion` - 1 orders do not
// reach it; then the e_0 phase (wavefunction.py:605-606).
//
// The whole series is one CUDA graph: a WHILE conditional node whose body is
// one order — the apply work -> next (every kernel of the FP64 or tensor-core
// apply), k_taylor_term (psi += next / k!, work = next, partial sums of
// |next|^2 over a fixed grid) and k_taylor_decide (the norm in a fixed
// summation order, the reference's stopping test, the loop condition via
// cudaGraphSetConditional).  The host launches the graph and reads the
// 32-byte loop state once at the end: no host round trip per order, no
// extra order computed after the stopping test.  The graph of a handle is
// kept and relaunched while its arguments (buffers, t, accuracy, expansion,
// precision, workspace) stay the same.
#include <cmath>
#include <vector>

#include "ham.cuh"

namespace fqegpu {

namespace {
constexpr int kTermBlocks = 4 * kNumSMs;  // fixed grid: deterministic partial sums
constexpr int kTermThreads = 256;
}  // namespace

struct TaylorState {
  double inv_fact;  // 1/k! of the last order added
  double nrm2;      // |(-i t H)^k psi|^2 of that order
  int order;        // last order added (0 before the first)
  int stop;         // 1 once converged, non-finite or out of orders
  int converged;
  int nonfinite;
};

// psi += (inv_fact / (order + 1)) next; work = next; partial[block] =
// sum of |next|^2 over the block's grid-stride elements.
__global__ void __launch_bounds__(kTermThreads) k_taylor_term(
    int64_t n, const TaylorState* __restrict__ st, const double2* __restrict__ next,
    double2* __restrict__ work, double2* __restrict__ psi, double* __restrict__ partial) {
  __shared__ double red[kTermThreads / 32];
  const double c = st->inv_fact / (double)(st->order + 1);
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = next[i];
    double2 p = psi[i];
    p.x += c * v.x;
    p.y += c * v.y;
    psi[i] = p;
    work[i] = v;
    acc += v.x * v.x + v.y * v.y;
  }
  for (int m = 16; m > 0; m >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, m);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kTermThreads / 32; ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

// One block of 256 threads: the norm of the order (fixed summation tree),
// the stopping rule of wavefunction.py:561-568, and the loop condition.
__global__ void __launch_bounds__(256) k_taylor_decide(TaylorState* st,
                                                       const double* __restrict__ partial,
                                                       int nparts, double accuracy, int expansion,
                                                       cudaGraphConditionalHandle cond) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partial[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int k = st->order + 1;
    const double inv = st->inv_fact / (double)k;
    const double nrm2 = red[0];
    st->order = k;
    st->inv_fact = inv;
    st->nrm2 = nrm2;
    int stop = 0;
    if (!isfinite(nrm2)) {
      st->nonfinite = 1;
      stop = 1;
    } else if (sqrt(nrm2) * inv < accuracy) {
      st->converged = 1;
      stop = 1;
    } else if (k + 1 >= expansion) {
      stop = 1;
    }
    st->stop = stop;
    cudaGraphSetConditional(cond, stop ? 0u : 1u);
  }
}

__global__ void k_taylor_init(TaylorState* st) {
  st->inv_fact = 1.0;
  st->nrm2 = 0.0;
  st->order = 0;
  st->stop = 0;
  st->converged = 0;
  st->nonfinite = 0;
}

static_assert(sizeof(TaylorState) == kTaylorStateHostBytes, "state size");

size_t taylor_state_bytes() { return sizeof(TaylorState) + sizeof(double) * kTermBlocks; }

// Records into the graph being captured on `cs`: psi -> work, the state's
// reset, and the WHILE node of the series (its body captured on `bs`, a
// stream that is not capturing, created by the caller before the capture).
// work and next are the handle's two-vector buffer; `state` holds a
// TaylorState followed by kTermBlocks partial sums.
int taylor_record(fqegpu_ham h, double2* psi, double time, double accuracy, int expansion,
                  int precision, void* state, cudaStream_t cs, cudaStream_t bs) {
  const int64_t N = h->g->a.len * h->g->b.len;
  double2* work = h->d_vec;
  double2* next = h->d_vec + N;
  TaylorState* ts = reinterpret_cast<TaylorState*>(state);
  double* partial = reinterpret_cast<double*>(ts + 1);
  FQE_CUDA(cudaMemcpyAsync(work, psi, sizeof(double2) * N, cudaMemcpyDeviceToDevice, cs));
  k_taylor_init<<<1, 1, 0, cs>>>(ts);
  FQE_CUDA(cudaGetLastError());
  if (expansion <= 1) return FQEGPU_OK;  // no order is computed
  cudaStreamCaptureStatus cst;
  cudaGraph_t capg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  FQE_CUDA(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &capg, &deps, nullptr, &ndeps));
  if (cst != cudaStreamCaptureStatusActive) {
    set_error("taylor_record: the stream is not capturing");
    return FQEGPU_ERR_CUDA;
  }
  cudaGraphConditionalHandle cond;
  FQE_CUDA(cudaGraphConditionalHandleCreate(&cond, capg, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = cond;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  std::vector<cudaGraphNode_t> dv(deps, deps + ndeps);
  FQE_CUDA(cudaGraphAddNode(&node, capg, dv.data(), nullptr, dv.size(), &p));
  FQE_CUDA(cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1,
                                               cudaStreamSetCaptureDependencies));
  cudaGraph_t body = p.conditional.phGraph_out[0];
  int s = FQEGPU_OK;
  cudaError_t e = cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const double2 alpha = make_double2(0.0, -time), zero = make_double2(0.0, 0.0);
    s = precision == FQEGPU_PREC_OZAKI ? apply_ozaki(h, work, next, alpha, zero, bs)
                                       : apply_fp64(h, work, next, alpha, zero, bs);
    if (s == FQEGPU_OK) {
      k_taylor_term<<<kTermBlocks, kTermThreads, 0, bs>>>(N, ts, next, work, psi, partial);
      k_taylor_decide<<<1, 256, 0, bs>>>(ts, partial, kTermBlocks, accuracy, expansion, cond);
      e = cudaGetLastError();
    }
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(bs, &out);
    if (e == cudaSuccess) e = e2;
  }
  if (s != FQEGPU_OK) return s;
  if (e != cudaSuccess) {
    set_error("taylor graph body: %s", cudaGetErrorString(e));
    return FQEGPU_ERR_CUDA;
  }
  return FQEGPU_OK;
}

// Reads a finished series' state: terms, and the reference's errors.
int taylor_result(const void* h_state, int expansion, int* h_terms) {
  const TaylorState* ts = reinterpret_cast<const TaylorState*>(h_state);
  if (h_terms) *h_terms = ts->converged ? ts->order : expansion;
  if (ts->nonfinite) {
    set_error("taylor: non-finite norm at order %d", ts->order);
    return FQEGPU_ERR_NUMERIC;
  }
  if (!ts->converged) {
    set_error("maximum taylor expansion limit reached");
    return FQEGPU_ERR_NUMERIC;
  }
  return FQEGPU_OK;
}

// The e_0 phase exp(-i t e0) of wavefunction.py:605-606.
int taylor_phase(double2* psi, int64_t N, double time, double e0_re, double e0_im,
                 cudaStream_t st) {
  if (std::hypot(e0_re * time, e0_im * time) <= 1.0e-15) return FQEGPU_OK;
  const double re = e0_im * time, im = -e0_re * time;  // -i t e0
  const double m = std::exp(re);
  return scale_async(N, make_double2(m * std::cos(im), m * std::sin(im)), psi, st);
}

struct TaylorGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void* d_state = nullptr;
  TaylorState* h_state = nullptr;  // pinned
  // arguments the recorded graph depends on
  double2* psi = nullptr;
  double time = 0.0, accuracy = 0.0;
  int expansion = 0, precision = -1;
  void* ws = nullptr;
  const void* plan = nullptr;
  int64_t block_w = 0;
  int tuning = -1;
};

void taylor_destroy(fqegpu_ham h) {
  TaylorGraph* tg = h->taylor;
  if (!tg) return;
  if (tg->exec) cudaGraphExecDestroy(tg->exec);
  if (tg->graph) cudaGraphDestroy(tg->graph);
  cudaFree(tg->d_state);
  if (tg->h_state) cudaFreeHost(tg->h_state);
  delete tg;
  h->taylor = nullptr;
}

static void drop_graph(TaylorGraph* tg) {
  if (tg->exec) cudaGraphExecDestroy(tg->exec);
  if (tg->graph) cudaGraphDestroy(tg->graph);
  tg->exec = nullptr;
  tg->graph = nullptr;
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_taylor(fqegpu_ham h, double* d_psi, double time,
                             double e0_re, double e0_im, double accuracy,
                             int expansion, int precision, int* h_terms,
                             void* stream) {
  clear_error();
  FQE_CHECK_ARG(h && d_psi, "NULL argument");
  FQE_CHECK_ARG(expansion >= 1, "expansion must be >= 1");
  FQE_CHECK_ARG(precision == FQEGPU_PREC_FP64 || precision == FQEGPU_PREC_OZAKI,
                "unknown precision");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = h->g->a.len * h->g->b.len;
  if (!h->d_vec) FQE_CUDA(dev_alloc(&h->d_vec, sizeof(double2) * 2 * (size_t)N));
  FQE_TRY(apply_prepare(h, precision));
  if (!h->taylor) {
    auto* tg = new (std::nothrow) TaylorGraph();
    if (!tg) {
      set_error("host allocation failed");
      return FQEGPU_ERR_NOMEM;
    }
    h->taylor = tg;
    FQE_CUDA(dev_alloc(&tg->d_state, taylor_state_bytes()));
    FQE_CUDA(cudaHostAlloc(&tg->h_state, sizeof(TaylorState), cudaHostAllocDefault));
  }
  TaylorGraph* tg = h->taylor;
  double2* psi = (double2*)d_psi;
  const bool same = tg->exec && tg->psi == psi && tg->time == time &&
                    tg->accuracy == accuracy && tg->expansion == expansion &&
                    tg->precision == precision && tg->ws == h->d_ws &&
                    tg->plan == (const void*)h->oz && tg->block_w == h->block_w &&
                    tg->tuning == ozaki_tuning_key(h);
  if (!same) {
    drop_graph(tg);
    cudaStream_t cs = nullptr, bs = nullptr;
    FQE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess) {
      cudaStreamDestroy(cs);
      set_error("stream creation failed");
      return FQEGPU_ERR_CUDA;
    }
    const bool timing = h->timing;
    h->timing = false;      // no event records inside a graph
    h->defer_check = true;  // the tensor-core error word is read after the graph
    int s = FQEGPU_OK;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      s = taylor_record(h, psi, time, accuracy, expansion, precision, tg->d_state, cs, bs);
      cudaGraph_t g = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
      tg->graph = g;
      if (e == cudaSuccess) e = e2;
    }
    h->timing = timing;
    h->defer_check = false;
    cudaStreamDestroy(cs);
    cudaStreamDestroy(bs);
    if (s == FQEGPU_OK && e == cudaSuccess) e = cudaGraphInstantiate(&tg->exec, tg->graph, 0);
    if (s != FQEGPU_OK || e != cudaSuccess) {
      if (tg->exec == nullptr && tg->graph) {
        cudaGraphDestroy(tg->graph);
        tg->graph = nullptr;
      }
      if (s != FQEGPU_OK) return s;
      set_error("taylor graph: %s", cudaGetErrorString(e));
      return FQEGPU_ERR_CUDA;
    }
    tg->psi = psi;
    tg->time = time;
    tg->accuracy = accuracy;
    tg->expansion = expansion;
    tg->precision = precision;
    tg->ws = h->d_ws;
    tg->plan = h->oz;
    tg->block_w = h->block_w;
    tg->tuning = ozaki_tuning_key(h);
  }
  FQE_CUDA(cudaGraphLaunch(tg->exec, st));
  FQE_CUDA(cudaMemcpyAsync(tg->h_state, tg->d_state, sizeof(TaylorState),
                           cudaMemcpyDeviceToHost, st));
  FQE_CUDA(cudaStreamSynchronize(st));
  if (h->oz) FQE_TRY(ozaki_check(h, st));
  FQE_TRY(taylor_result(tg->h_state, expansion, h_terms));
  return taylor_phase(psi, N, time, e0_re, e0_im, st);
}
