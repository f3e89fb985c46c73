// Prepared restricted Hamiltonian of one sector, and the apply pipeline's
// internal entry points shared by the FP64 and the tensor-core paths.
#pragma once

#include <complex>
#include <vector>

#include "common.cuh"

namespace fqegpu {

using zd = std::complex<double>;

struct OzakiPlan;    // tensor-core contraction state (ozaki.cu)
struct TaylorGraph;  // recorded Taylor series of a handle (taylor.cu)

// Host preparation of (h1, h2) for one sector (fqe_data.py:691-693 and the
// compressed branch's symmetry assumption, fqe_data.py:658-681):
//   V[ij][kl] = h2'[i,j,k,l] = -h2[i,k,j,l],  h1' = h1 + sum_k h2[i,k,k,j],
// with the one-body part folded in as h1'[ij] delta_kl / N_e (two-body) or
// kept as the weight vector h1' (one-body, h2 == NULL).  A global phase is
// factored out when what remains is real (to 64 ulp of the largest entry);
// the pair space is compressed to p = tri(i, j) when the tensors have the
// real-orbital pair symmetries.  Used by fqegpu_ham_create and
// fqegpu_apply_noalloc, so both apply the same operator.
struct PairMatrix {
  bool zero = false;        // identically zero on this sector
  bool onebody = false;     // h2 == NULL
  bool real = false;        // phase * (real tensor)
  bool compressed = false;  // pair space p = tri(i, j)
  double2 phase{1.0, 0.0};
  int P = 0;
  std::vector<zd> h1p;        // [norb][norb] prepared one-body h1'
  std::vector<zd> v2;         // [norb^2][norb^2] prepared two-body V' (two-body only)
  std::vector<double> vr;     // [P][P] (two-body) or [P] (one-body), real case
  std::vector<double2> vc;    // same, complex case
};
void prepare_pairs(int norb, int nele, const zd* H1, const zd* H2, PairMatrix& out);
// The spin-orbital form (h1 [2 norb][2 norb], h2 [2 norb]^4, alpha orbitals
// first; h2 may be NULL): pair space of alpha pairs then beta pairs, P =
// 2 norb^2 (or 2 norb(norb+1)/2 compressed); h1p and v2 are left empty.
void prepare_pairs_spin(int norb, int nalpha, int nbeta, const zd* H1, const zd* H2,
                        PairMatrix& out);

int axpy_async(int64_t n, double2 a, const double2* x, double2* y, cudaStream_t st);
int scale_async(int64_t n, double2 a, double2* x, cudaStream_t st);
int dot_async(int64_t n, const double2* x, const double2* y, double2* scratch,
              double2* d_out, cudaStream_t st);
int dot_scratch_bytes();

}  // namespace fqegpu

struct fqegpu_ham_s {
  fqegpu_graph g = nullptr;
  int norb = 0;
  int nele = 0;
  bool zero = false;        // operator is identically zero on this sector
  bool onebody = false;     // no two-body tensor: sigma = sum_p h1_p E_p psi
  bool compressed = false;  // pair space p = tri(i, j)
  bool real = false;        // tensors are phase * (real tensor)
  bool spin = false;        // spin-orbital operator: alpha pairs, then beta pairs
  double2 phase{1.0, 0.0};
  int P = 0;                // pair count
  // Pair tables [P][len] of a spin-orbital operator (alpha rows zero in the
  // beta table and vice versa), owned; NULL for a restricted operator, which
  // reads the graph's tables.
  int32_t* d_tabA = nullptr;
  int32_t* d_tabB = nullptr;
  // Device copies, already divided by `phase` when real.
  double* d_Vr = nullptr;   // [P][P] real pair matrix (two-body, real)
  double2* d_Vc = nullptr;  // [P][P] complex pair matrix (two-body, complex)
  double* d_h1r = nullptr;  // [P] one-body weights (one-body mode, real)
  double2* d_h1c = nullptr; // [P] one-body weights (one-body mode, complex)
  // Host copies used by the diagonal (Davidson) and the tensor-core planner.
  std::vector<fqegpu::zd> h1p;   // [norb][norb] prepared one-body h1'
  std::vector<fqegpu::zd> v2;    // [norb^2][norb^2] prepared two-body V'
  std::vector<double> vpair;     // [P][P] real pair matrix incl. h1'/N_e (real)
  // Apply workspace (beta-column blocks of D and G).
  int64_t scratch_limit = 0;
  int64_t block_w = 0;
  size_t ws_bytes = 0;
  void* d_ws = nullptr;
  // Taylor / reduction workspace.
  double2* d_vec = nullptr;  // 2 * N complex
  double2* d_red = nullptr;
  fqegpu::OzakiPlan* oz = nullptr;
  fqegpu::TaylorGraph* taylor = nullptr;
  // Optional per-stage timing: 4 events per beta block (start, after gather,
  // after contraction, after scatter), recorded on the launching stream.
  bool timing = false;
  std::vector<cudaEvent_t> events;
  int events_used = 0;
  // Set while an apply is recorded into a CUDA graph: the tensor-core path
  // then skips its end-of-apply error readback (fqegpu_batch_check reads it).
  bool defer_check = false;
  // Number of live CUDA graphs (batches, Taylor graphs) that hold this
  // handle's workspace and plan pointers; while nonzero the handle refuses to
  // reallocate them (scratch-limit changes) and to be destroyed.
  int live_graphs = 0;
  // fqegpu_apply_host: a copy stream and one event per row chunk, so sigma's
  // finished rows travel to the host while the scatter of later rows runs.
  cudaStream_t out_stream = nullptr;
  cudaEvent_t out_ev[8] = {};
};

namespace fqegpu {
// The pair tables an apply of `h` reads: tab[p][string] = sign * (source + 1).
inline const int32_t* ham_tabA(const fqegpu_ham_s* h) {
  return h->d_tabA ? h->d_tabA : (h->compressed ? h->g->a.tab_tri : h->g->a.tab_full);
}
inline const int32_t* ham_tabB(const fqegpu_ham_s* h) {
  return h->d_tabB ? h->d_tabB : (h->compressed ? h->g->b.tab_tri : h->g->b.tab_full);
}
inline double2 zmul_host(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Records event k of block `blk` when timing is on (no-op otherwise).
int stage_mark(fqegpu_ham h, int blk, int k, cudaStream_t st);
int apply_fp64(fqegpu_ham h, const double2* psi, double2* sigma, double2 alpha,
               double2 beta, cudaStream_t st);
// Host output of an apply (fqegpu_apply_host): when `h_sigma` is set, the
// tensor-core path scatters its last beta-column block in row chunks and
// copies each chunk of sigma to h_sigma on `copy` as soon as it is final
// (`issued` reports that it did; the caller then waits for `copy`).
struct HostOut {
  double2* h_sigma = nullptr;
  cudaStream_t copy = nullptr;
  cudaEvent_t* ev = nullptr;  // kOutChunks events
  bool issued = false;
};
constexpr int kOutChunks = 8;
int apply_ozaki(fqegpu_ham h, const double2* psi, double2* sigma, double2 alpha,
                double2 beta, cudaStream_t st, HostOut* out = nullptr);
void ozaki_destroy(fqegpu_ham h);
// Creates the tensor-core plan if the operator fits it (FQEGPU_ERR_UNSUPPORTED
// otherwise: the apply then runs the FP64 kernels).
int ozaki_prepare(fqegpu_ham h);
// Waits for `st` and reports (and clears) the tensor-core path's sticky
// error word: FQEGPU_ERR_TIMEOUT when a bounded wait gave up since the last
// check.
int ozaki_check(fqegpu_ham h, cudaStream_t st);
// Tuning of the tensor-core path: tiles per column super-block (> 0; else
// unchanged) and whether the operator runs the FP64 kernels instead.
int ozaki_set_tuning(fqegpu_ham h, int super_tiles, int use_fp64);
// Whether the tuned tensor-core path runs the FP64 kernels; a key of the
// current tuning (recorded graphs are re-recorded when it changes).
bool ozaki_runs_fp64(fqegpu_ham h);
int ozaki_tuning_key(fqegpu_ham h);
// Test-only: wait limit of the tensor-core kernel (cycles; <= 0: default) and
// a ring slot of CTA 0's first tile pair left unfilled (-1: none).
int ozaki_set_test_injection(fqegpu_ham h, long long wait_cycles, int skip_slot);
// Allocates what an apply of `precision` needs (plan, workspace) without
// running it, so that the apply can be recorded into a CUDA graph.
int apply_prepare(fqegpu_ham h, int precision);
// Device-resident Taylor series (taylor.cu): bytes of one series' device
// state; recording of one series of `h` on `psi` into the graph being
// captured on `cs`, its loop body captured on `bs` (a stream that is not
// capturing; uses h->d_vec, which must hold 2 N elements); reading of
// a finished series' state (copied to the host) into the reference's
// errors; the e_0 phase.
size_t taylor_state_bytes();
int taylor_record(fqegpu_ham h, double2* psi, double time, double accuracy, int expansion,
                  int precision, void* state, cudaStream_t cs, cudaStream_t bs);
int taylor_result(const void* h_state, int expansion, int* h_terms);
int taylor_phase(double2* psi, int64_t N, double time, double e0_re, double e0_im,
                 cudaStream_t st);
void taylor_destroy(fqegpu_ham h);
constexpr size_t kTaylorStateHostBytes = 32;  // sizeof(TaylorState)
// Gather / scatter building blocks (apply.cu) over the pair tables
// tabA [P][lena], tabB [P][lenb] of the graph's sector.
int launch_gather(const fqegpu_graph_s* g, const int32_t* tabA, const int32_t* tabB, int P,
                  int64_t c0, int64_t w, const double2* psi, double2* D, cudaStream_t st);
int launch_scatter(const fqegpu_graph_s* g, const int32_t* tabA, const int32_t* tabB, int P,
                   int64_t c0, int64_t w, const double2* G, const double2* psi,
                   double2 alpha, double2 beta, bool init, double2* sigma,
                   cudaStream_t st);
}  // namespace fqegpu
