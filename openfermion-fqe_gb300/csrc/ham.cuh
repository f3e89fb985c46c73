// Prepared restricted Hamiltonian of one sector, and the apply pipeline's
// internal entry points shared by the FP64 and the tensor-core paths.
#pragma once

#include <complex>
#include <vector>

#include "common.cuh"

namespace fqegpu {

using zd = std::complex<double>;

struct OzakiPlan;  // tensor-core contraction state (ozaki.cu)

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
  double2 phase{1.0, 0.0};
  int P = 0;                // pair count
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
  // Optional per-stage timing: 4 events per beta block (start, after gather,
  // after contraction, after scatter), recorded on the launching stream.
  bool timing = false;
  std::vector<cudaEvent_t> events;
  int events_used = 0;
  // Set while an apply is recorded into a CUDA graph: the tensor-core path
  // then skips its end-of-apply error readback (fqegpu_batch_check reads it).
  bool defer_check = false;
};

namespace fqegpu {
inline double2 zmul_host(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Records event k of block `blk` when timing is on (no-op otherwise).
int stage_mark(fqegpu_ham h, int blk, int k, cudaStream_t st);
int apply_fp64(fqegpu_ham h, const double2* psi, double2* sigma, double2 alpha,
               double2 beta, cudaStream_t st);
int apply_ozaki(fqegpu_ham h, const double2* psi, double2* sigma, double2 alpha,
                double2 beta, cudaStream_t st);
void ozaki_destroy(fqegpu_ham h);
// Error word of the tensor-core path's last apply (0 when none ran or OK).
int ozaki_error_flag(fqegpu_ham h, int32_t* out);
// Gather / scatter building blocks (apply.cu).
int launch_gather(const fqegpu_graph_s* g, bool tri, int P, int64_t c0,
                  int64_t w, const double2* psi, double2* D, cudaStream_t st);
int launch_scatter(const fqegpu_graph_s* g, bool tri, int P, int64_t c0,
                   int64_t w, const double2* G, const double2* psi,
                   double2 alpha, double2 beta, bool init, double2* sigma,
                   cudaStream_t st);
}  // namespace fqegpu
