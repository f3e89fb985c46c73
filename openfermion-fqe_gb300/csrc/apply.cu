// H·psi for the restricted Hamiltonian of one sector (A2-A7 of the path).
//
// The reference applies sigma = sum h1' E + sum h2' E E through three native
// loops (lm_apply_array12_same_spin_opt for alpha and beta, and
// lm_apply_array12_diff_spin_opt; lib/fqe_data.c:668-720, 879-996).  Here the
// same operator is applied in the Knowles-Handy dvec form the reference's own
// Python path uses (fqe_data.py:647-681, 2209-2234, 2309-2334):
//
//   D[q][I] = <I| E_q |psi>                         (K2 gather)
//   G[p][I] = sum_q V[p][q] D[q][I]                  (K3 pair contraction)
//   sigma[I] = beta psi[I] + alpha sum_p <I|E_p|J> G[p][J]   (K4 scatter)
//
// with E = E^alpha + E^beta summed over spin and V the pair matrix
// V[ij][kl] = h2'[i,j,k,l] + h1'[ij] delta_kl / N_e (the one-body part rides
// along in the contraction because sum_k E_kk = N_e on the sector).  When the
// integrals have the real-orbital pair symmetries the pair space is the
// compressed p = tri(i, j) space (E_p = E_ij + E_ji), as fqe_data.py:658-681.
//
// Layout in HBM: psi, sigma [lena][lenb] complex128; D and G [P][lena][w]
// complex128 for a beta-column block [c0, c0 + w).  Every target string has at
// most one source under each E_p, so both gather and scatter are target-owned
// reads through the per-pair tables tab[p][string] = sign * (source + 1); no
// atomics.  The alpha half of the scatter stays inside the block; the beta
// half reads G at source columns, so with several blocks each block adds its
// share to every column (a fixed block order keeps the result deterministic).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "ham.cuh"

namespace fqegpu {

__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ---------------------------------------------------------------------------
// K2: D[p][a][c] for columns b = c0 + c of the block.  One CTA per (p, a) row.
__global__ void __launch_bounds__(256) k_gather_f64(
    int P, int64_t lena, int64_t lenb, int64_t c0, int64_t w,
    const int32_t* __restrict__ tabA, const int32_t* __restrict__ tabB,
    const double2* __restrict__ psi, double2* __restrict__ D) {
  const int64_t row = blockIdx.x;
  const int64_t p = row / lena, a = row - p * lena;
  const int32_t ca = tabA[p * lena + a];
  const double2* srcA = nullptr;
  double sA = 0.0;
  if (ca) {
    srcA = psi + (int64_t)(abs(ca) - 1) * lenb;
    sA = ca > 0 ? 1.0 : -1.0;
  }
  const double2* rowa = psi + a * lenb;
  const int32_t* tb = tabB + p * lenb;
  double2* out = D + row * w;
  for (int64_t c = threadIdx.x; c < w; c += blockDim.x) {
    const int64_t b = c0 + c;
    double2 v = make_double2(0.0, 0.0);
    if (srcA) {
      const double2 x = srcA[b];
      v.x = sA * x.x;
      v.y = sA * x.y;
    }
    const int32_t cb = tb[b];
    if (cb) {
      const double2 x = rowa[abs(cb) - 1];
      const double s = cb > 0 ? 1.0 : -1.0;
      v.x += s * x.x;
      v.y += s * x.y;
    }
    out[c] = v;
  }
}

// ---------------------------------------------------------------------------
// K3 (FP64): G[p][n] = sum_q V[p][q] D[q][n] over n in [0, ncol) complex
// columns.  64x64 tile, 16-deep K steps, 256 threads with 4x4 outputs each.
// The FP64 pipe of GB300 (~1.1 TFLOP/s) bounds this kernel.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_pairgemm_f64(
    int P, int64_t ncol, const double* __restrict__ Vr,
    const double2* __restrict__ Vc, const double2* __restrict__ D,
    double2* __restrict__ G) {
  constexpr int BM = 64, BN = 64, BK = 16;
  using AT = typename std::conditional<CPLX, double2, double>::type;
  __shared__ AT As[BK][BM];
  __shared__ double2 Bs[BK][BN];
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const int m0 = blockIdx.y * BM;
  const int64_t n0 = (int64_t)blockIdx.x * BN;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);

  for (int k0 = 0; k0 < P; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + 256 * r;
      const int m = idx / BK, k = idx % BK;
      const int gm = m0 + m, gk = k0 + k;
      if constexpr (CPLX) {
        As[k][m] = (gm < P && gk < P) ? Vc[(int64_t)gm * P + gk]
                                      : make_double2(0.0, 0.0);
      } else {
        As[k][m] = (gm < P && gk < P) ? Vr[(int64_t)gm * P + gk] : 0.0;
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + 256 * r;
      const int k = idx / BN, n = idx % BN;
      const int gk = k0 + k;
      const int64_t gn = n0 + n;
      Bs[k][n] = (gk < P && gn < ncol) ? D[(int64_t)gk * ncol + gn]
                                       : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      AT a[4];
      double2 b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if constexpr (CPLX) {
            acc[i][j].x = fma(a[i].x, b[j].x, fma(-a[i].y, b[j].y, acc[i][j].x));
            acc[i][j].y = fma(a[i].x, b[j].y, fma(a[i].y, b[j].x, acc[i][j].y));
          } else {
            acc[i][j].x = fma(a[i], b[j].x, acc[i][j].x);
            acc[i][j].y = fma(a[i], b[j].y, acc[i][j].y);
          }
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= P) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gn = n0 + tx + 16 * j;
      if (gn < ncol) G[(int64_t)gm * ncol + gn] = acc[i][j];
    }
  }
}

// ---------------------------------------------------------------------------
// K4: sigma[a][b] (=|+=) beta psi + alpha sum_p [alpha-half + beta-half].
// One thread per determinant, CTA = 256 columns of one alpha row.
// ONEBODY: the contracted value at source J is h1[p] * psi[J] (no G buffer).
template <int MODE>  // 0: G buffer, 1: one-body real weights, 2: one-body complex
__global__ void __launch_bounds__(256) k_scatter(
    int P, int64_t lena, int64_t lenb, int64_t c0, int64_t w,
    const int32_t* __restrict__ tabA, const int32_t* __restrict__ tabB,
    const double2* __restrict__ G, const double2* __restrict__ psi,
    const double* __restrict__ h1r, const double2* __restrict__ h1c,
    double2 alpha, double2 beta, int init, double2* __restrict__ sigma) {
  const int64_t a = blockIdx.y;
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= lenb) return;
  const bool inblk = (b >= c0) && (b < c0 + w);
  double2 acc = make_double2(0.0, 0.0);
  for (int p = 0; p < P; ++p) {
    double2 t = make_double2(0.0, 0.0);
    const int32_t ca = tabA[(int64_t)p * lena + a];
    if (ca && inblk) {
      const int64_t J = abs(ca) - 1;
      const double s = ca > 0 ? 1.0 : -1.0;
      const double2 x = (MODE == 0) ? G[((int64_t)p * lena + J) * w + (b - c0)]
                                    : psi[J * lenb + b];
      t.x += s * x.x;
      t.y += s * x.y;
    }
    const int32_t cb = tabB[(int64_t)p * lenb + b];
    if (cb) {
      const int64_t J = abs(cb) - 1;
      if (J >= c0 && J < c0 + w) {
        const double s = cb > 0 ? 1.0 : -1.0;
        const double2 x = (MODE == 0) ? G[((int64_t)p * lena + a) * w + (J - c0)]
                                      : psi[a * lenb + J];
        t.x += s * x.x;
        t.y += s * x.y;
      }
    }
    if (MODE == 0) {
      acc.x += t.x;
      acc.y += t.y;
    } else if (MODE == 1) {
      acc.x += h1r[p] * t.x;
      acc.y += h1r[p] * t.y;
    } else {
      const double2 m = cmul(h1c[p], t);
      acc.x += m.x;
      acc.y += m.y;
    }
  }
  const int64_t I = a * lenb + b;
  double2 out;
  if (init) {
    out = (beta.x == 0.0 && beta.y == 0.0) ? make_double2(0.0, 0.0)
                                           : cmul(beta, psi[I]);
  } else {
    out = sigma[I];
  }
  const double2 r = cmul(alpha, acc);
  out.x += r.x;
  out.y += r.y;
  sigma[I] = out;
}

__global__ void k_axpby(int64_t n, double2 beta, const double2* __restrict__ x,
                        double2* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (beta.x == 0.0 && beta.y == 0.0) ? make_double2(0.0, 0.0)
                                            : cmul(beta, x[i]);
}

int launch_gather(const fqegpu_graph_s* g, const int32_t* tabA, const int32_t* tabB, int P,
                  int64_t c0, int64_t w, const double2* psi, double2* D, cudaStream_t st) {
  const int64_t lena = g->a.len, lenb = g->b.len;
  const int64_t rows = (int64_t)P * lena;
  if (rows == 0 || w == 0) return FQEGPU_OK;
  k_gather_f64<<<(unsigned)rows, 256, 0, st>>>(P, lena, lenb, c0, w, tabA, tabB, psi, D);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

int launch_scatter(const fqegpu_graph_s* g, const int32_t* tabA, const int32_t* tabB, int P,
                   int64_t c0, int64_t w, const double2* G, const double2* psi,
                   double2 alpha, double2 beta, bool init, double2* sigma,
                   cudaStream_t st) {
  const int64_t lena = g->a.len, lenb = g->b.len;
  if (lena > 65535) {
    set_error("alpha string space of %lld exceeds the 65535 rows one launch covers",
              (long long)lena);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  dim3 grid((unsigned)((lenb + 255) / 256), (unsigned)lena);
  k_scatter<0><<<grid, 256, 0, st>>>(P, lena, lenb, c0, w, tabA, tabB, G, psi, nullptr,
                                     nullptr,
                                     alpha, beta, init ? 1 : 0, sigma);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

static int grid_1d(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), (int64_t)kNumSMs * 16);
}

// Allocate D and G for the widest block that fits the scratch limit.
static int ensure_workspace(fqegpu_ham h) {
  const int64_t lena = h->g->a.len, lenb = h->g->b.len;
  const int64_t per_col = 2 * (int64_t)h->P * lena * (int64_t)sizeof(double2);
  int64_t w = per_col > 0 ? h->scratch_limit / per_col : lenb;
  w = std::min<int64_t>(std::max<int64_t>(w, 1), lenb);
  const size_t bytes = (size_t)(per_col * w);
  if (h->d_ws && h->block_w == w) return FQEGPU_OK;
  if (h->live_graphs > 0) {
    set_error("the handle's workspace is held by %d recorded CUDA graph(s) and cannot be "
              "reallocated; destroy them first", h->live_graphs);
    return FQEGPU_ERR_INVALID;
  }
  if (h->d_ws) {
    cudaFree(h->d_ws);
    h->d_ws = nullptr;
    h->ws_bytes = 0;
  }
  FQE_CUDA(dev_alloc(&h->d_ws, bytes));
  h->ws_bytes = bytes;
  h->block_w = w;
  return FQEGPU_OK;
}

int apply_prepare(fqegpu_ham h, int precision) {
  if (h->zero || h->onebody) return FQEGPU_OK;
  if (precision == FQEGPU_PREC_OZAKI) {
    const int s = ozaki_prepare(h);
    if (s != FQEGPU_ERR_UNSUPPORTED && s != FQEGPU_OK) return s;
    if (s == FQEGPU_OK && !ozaki_runs_fp64(h)) return FQEGPU_OK;
  }
  return ensure_workspace(h);
}

int apply_fp64(fqegpu_ham h, const double2* psi, double2* sigma, double2 alpha,
               double2 beta, cudaStream_t st) {
  const fqegpu_graph_s* g = h->g;
  const int64_t lena = g->a.len, lenb = g->b.len, N = lena * lenb;
  const double2 al = cmul(alpha, h->phase);
  if (h->zero) {
    k_axpby<<<grid_1d(N), 256, 0, st>>>(N, beta, psi, sigma);
    FQE_CUDA(cudaGetLastError());
    return FQEGPU_OK;
  }
  if (lena > 65535) {
    set_error("alpha string space of %lld exceeds the 65535 rows one launch covers",
              (long long)lena);
    return FQEGPU_ERR_UNSUPPORTED;
  }
  if (h->onebody) {
    dim3 grid((unsigned)((lenb + 255) / 256), (unsigned)lena);
    if (h->real) {
      k_scatter<1><<<grid, 256, 0, st>>>(h->P, lena, lenb, 0, lenb, ham_tabA(h), ham_tabB(h),
                                         nullptr, psi, h->d_h1r, nullptr, al,
                                         beta, 1, sigma);
    } else {
      k_scatter<2><<<grid, 256, 0, st>>>(h->P, lena, lenb, 0, lenb, ham_tabA(h), ham_tabB(h),
                                         nullptr, psi, nullptr, h->d_h1c, al,
                                         beta, 1, sigma);
    }
    FQE_CUDA(cudaGetLastError());
    return FQEGPU_OK;
  }
  FQE_TRY(ensure_workspace(h));
  const int64_t w = h->block_w;
  double2* D = (double2*)h->d_ws;
  double2* G = D + (int64_t)h->P * lena * w;
  const bool single = (w >= lenb);
  if (!single) {
    k_axpby<<<grid_1d(N), 256, 0, st>>>(N, beta, psi, sigma);
    FQE_CUDA(cudaGetLastError());
  }
  h->events_used = 0;
  int blk = 0;
  for (int64_t c0 = 0; c0 < lenb; c0 += w, ++blk) {
    const int64_t wb = std::min<int64_t>(w, lenb - c0);
    FQE_TRY(stage_mark(h, blk, 0, st));
    FQE_TRY(launch_gather(g, ham_tabA(h), ham_tabB(h), h->P, c0, wb, psi, D, st));
    FQE_TRY(stage_mark(h, blk, 1, st));
    const int64_t ncol = lena * wb;
    dim3 grid((unsigned)((ncol + 63) / 64), (unsigned)((h->P + 63) / 64));
    if (h->real) {
      k_pairgemm_f64<false><<<grid, 256, 0, st>>>(h->P, ncol, h->d_Vr, nullptr,
                                                   D, G);
    } else {
      k_pairgemm_f64<true><<<grid, 256, 0, st>>>(h->P, ncol, nullptr, h->d_Vc,
                                                  D, G);
    }
    FQE_CUDA(cudaGetLastError());
    FQE_TRY(stage_mark(h, blk, 2, st));
    FQE_TRY(launch_scatter(g, ham_tabA(h), ham_tabB(h), h->P, c0, wb, G, psi, al, beta,
                           single, sigma, st));
    FQE_TRY(stage_mark(h, blk, 3, st));
  }
  return FQEGPU_OK;
}

int stage_mark(fqegpu_ham h, int blk, int k, cudaStream_t st) {
  if (!h->timing) return FQEGPU_OK;
  const size_t idx = (size_t)blk * 4 + k;
  while (h->events.size() <= idx) {
    cudaEvent_t e;
    FQE_CUDA(cudaEventCreate(&e));
    h->events.push_back(e);
  }
  FQE_CUDA(cudaEventRecord(h->events[idx], st));
  if ((int)idx + 1 > h->events_used) h->events_used = (int)idx + 1;
  return FQEGPU_OK;
}

// ---------------------------------------------------------------------------
// Host-side preparation of the pair matrix; declared in ham.cuh.
//
// `full` holds the operator in the uncompressed pair space of `nspin` blocks
// (pair (s, i, j) at s n^2 + i n + j; a [P][P] matrix, or a [P] weight vector
// for one-body operators).  Factors out a global phase when what remains is
// real, tests the real-orbital pair symmetry (i <-> j and k <-> l inside
// every block) and, when it holds, compresses each block to the n(n+1)/2
// pairs p = tri(i, j) (E_p = E_ij + E_ji), as fqe_data.py:658-681 does.
static void finish_pairs(int n, int nspin, const std::vector<zd>& full, PairMatrix& out) {
  const int n2 = n * n;
  const int PP = nspin * n2;
  double maxabs = 0.0;
  size_t imax = 0;
  for (size_t k = 0; k < full.size(); ++k) {
    const double v = std::abs(full[k]);
    if (v > maxabs) {
      maxabs = v;
      imax = k;
    }
  }
  if (maxabs == 0.0) out.zero = true;
  if (out.zero) return;
  zd ph = full[imax] / maxabs;
  if (ph.real() == 0.0 || ph.imag() == 0.0) ph = zd(ph.real() == 0.0 ? 0.0 : (ph.real() > 0 ? 1.0 : -1.0),
                                                    ph.imag() == 0.0 ? 0.0 : (ph.imag() > 0 ? 1.0 : -1.0));
  const double tol = 64.0 * DBL_EPSILON * maxabs;
  bool real = true;
  std::vector<zd> rot(full.size());
  for (size_t k = 0; k < full.size(); ++k) {
    rot[k] = full[k] * std::conj(ph);
    if (std::abs(rot[k].imag()) > tol) real = false;
  }
  out.real = real;
  out.phase = real ? make_double2(ph.real(), ph.imag()) : make_double2(1.0, 0.0);
  const std::vector<zd>& src = real ? rot : full;
  // index of pair (s, i, j) in the uncompressed space
  auto up = [&](int s, int i, int j) { return (size_t)s * n2 + (size_t)i * n + j; };
  bool sym = true;
  if (out.onebody) {
    for (int s = 0; s < nspin && sym; ++s)
      for (int i = 0; i < n && sym; ++i)
        for (int j = 0; j < i && sym; ++j)
          if (std::abs(src[up(s, i, j)] - src[up(s, j, i)]) > tol) sym = false;
  } else {
    for (int s = 0; s < nspin && sym; ++s)
      for (int i = 0; i < n && sym; ++i)
        for (int j = 0; j < n && sym; ++j)
          for (int t = 0; t < nspin && sym; ++t)
            for (int k = 0; k < n && sym; ++k)
              for (int l = 0; l < n; ++l) {
                const zd v = src[up(s, i, j) * PP + up(t, k, l)];
                if (std::abs(v - src[up(s, j, i) * PP + up(t, k, l)]) > tol ||
                    std::abs(v - src[up(s, i, j) * PP + up(t, l, k)]) > tol) {
                  sym = false;
                  break;
                }
              }
  }
  out.compressed = sym;
  const int per = sym ? n * (n + 1) / 2 : n2;  // pairs per spin block
  const int P = nspin * per;
  out.P = P;
  // compressed or uncompressed pair p -> (s, i, j)
  auto pair_of = [&](int p, int& sp, int& i, int& j) {
    sp = p / per;
    const int r = p - sp * per;
    if (!sym) {
      i = r / n;
      j = r % n;
      return;
    }
    int a = 0;
    while ((a + 1) * (a + 2) / 2 <= r) ++a;
    i = a;
    j = r - a * (a + 1) / 2;
  };
  if (out.onebody) {
    if (real) out.vr.resize(P); else out.vc.resize(P);
    for (int p = 0; p < P; ++p) {
      int sp, i, j;
      pair_of(p, sp, i, j);
      const zd v = src[up(sp, i, j)];
      if (real) out.vr[p] = v.real();
      else out.vc[p] = make_double2(v.real(), v.imag());
    }
    return;
  }
  if (real) out.vr.resize((size_t)P * P); else out.vc.resize((size_t)P * P);
  for (int p = 0; p < P; ++p) {
    int sp, i, j;
    pair_of(p, sp, i, j);
    for (int q = 0; q < P; ++q) {
      int sq, k, l;
      pair_of(q, sq, k, l);
      const zd v = src[up(sp, i, j) * PP + up(sq, k, l)];
      if (real) out.vr[(size_t)p * P + q] = v.real();
      else out.vc[(size_t)p * P + q] = make_double2(v.real(), v.imag());
    }
  }
}

// Restricted (spin-free) operator (fqe_data.py:691-693).
void prepare_pairs(int n, int nele, const zd* H1, const zd* H2, PairMatrix& out) {
  const int n2 = n * n;
  out = PairMatrix();
  out.h1p.assign((size_t)n2, zd(0.0, 0.0));
  if (H1)
    for (int k = 0; k < n2; ++k) out.h1p[k] = H1[k];
  out.onebody = (H2 == nullptr);
  if (!out.onebody) {
    // V'[ij][kl] = h2'[i,j,k,l] = -h2[i,k,j,l];  h1' = h1 + sum_k h2[i,k,k,j]
    out.v2.assign((size_t)n2 * n2, zd(0.0, 0.0));
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k)
          for (int l = 0; l < n; ++l)
            out.v2[(size_t)(i * n + j) * n2 + (k * n + l)] =
                -H2[((size_t)(i * n + k) * n + j) * n + l];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        zd s(0.0, 0.0);
        for (int k = 0; k < n; ++k) s += H2[((size_t)(i * n + k) * n + k) * n + j];
        out.h1p[i * n + j] += s;
      }
  }
  // Full pair matrix (or one-body vector) in the uncompressed space: the
  // one-body part rides in the contraction as h1'[ij] delta_kl / N_e
  std::vector<zd> full;
  if (out.onebody) {
    full = out.h1p;
  } else {
    full = out.v2;
    if (nele > 0) {
      const double inv = 1.0 / (double)nele;
      for (int ij = 0; ij < n2; ++ij)
        for (int k = 0; k < n; ++k) full[(size_t)ij * n2 + (k * n + k)] += out.h1p[ij] * inv;
    }
  }
  out.zero = nele == 0 || n == 0;
  finish_pairs(n, 1, full, out);
}

// Spin-orbital operator (h1 [2n][2n], h2 [2n]^4, alpha orbitals first), as
// _apply_array_spin12_lm (fqe_data.py:743-773) and _apply_array_spin1
// (:533-563) define it: h2'[I,J,K,L] = -h2[I,K,J,L] and h1' = h1 + sum_K
// h2[I,K,K,J] over all 2n spin orbitals; in the pair space of alpha pairs
// (s = 0) followed by beta pairs (s = 1), with E_(s,ij) = E^s_ij,
//   W[(s,ij)][(t,kl)] = h2'[sn+i, sn+j, tn+k, tn+l]
//                       + delta_st delta_kl h1'[sn+i, sn+j] / N_s
// (sum_k E^s_kk = N_s on the sector), so sigma = sum_pq W[p][q] E_p E_q psi,
// the operator the reference's halffilling branch builds from
// calculate_dvec_spin (fqe_data.py:725-741).  Blocks that move electrons
// between spins do not act on a sector and are ignored, as there.
void prepare_pairs_spin(int n, int na, int nb, const zd* H1, const zd* H2, PairMatrix& out) {
  const int m = 2 * n, n2 = n * n, PP = 2 * n2;
  out = PairMatrix();
  out.onebody = (H2 == nullptr);
  std::vector<zd> h1p((size_t)m * m, zd(0.0, 0.0));
  if (H1)
    for (int k = 0; k < m * m; ++k) h1p[k] = H1[k];
  auto h2 = [&](int I, int J, int K, int L) {
    return H2[(((size_t)I * m + J) * m + K) * m + L];
  };
  if (!out.onebody)
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        zd s(0.0, 0.0);
        for (int k = 0; k < m; ++k) s += h2(i, k, k, j);
        h1p[(size_t)i * m + j] += s;
      }
  std::vector<zd> full;
  const int nel[2] = {na, nb};
  if (out.onebody) {
    full.assign((size_t)PP, zd(0.0, 0.0));
    for (int s = 0; s < 2; ++s)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          full[(size_t)s * n2 + i * n + j] = h1p[(size_t)(s * n + i) * m + s * n + j];
  } else {
    full.assign((size_t)PP * PP, zd(0.0, 0.0));
    for (int s = 0; s < 2; ++s)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          const size_t row = ((size_t)s * n2 + i * n + j) * PP;
          for (int t = 0; t < 2; ++t)
            for (int k = 0; k < n; ++k)
              for (int l = 0; l < n; ++l)
                full[row + (size_t)t * n2 + k * n + l] =
                    -h2(s * n + i, t * n + k, s * n + j, t * n + l);
          if (nel[s] > 0) {
            const zd w = h1p[(size_t)(s * n + i) * m + s * n + j] / (double)nel[s];
            for (int k = 0; k < n; ++k) full[row + (size_t)s * n2 + k * n + k] += w;
          }
        }
  }
  out.zero = (na + nb == 0) || n == 0;
  finish_pairs(n, 2, full, out);
}

static int upload_pairs(fqegpu_ham h, PairMatrix& pm);

static int prepare(fqegpu_ham h, const double* h_h1, const double* h_h2) {
  PairMatrix pm;
  prepare_pairs(h->norb, h->nele, (const zd*)h_h1, (const zd*)h_h2, pm);
  return upload_pairs(h, pm);
}

// Spin-orbital operator: the pair matrix of prepare_pairs_spin and the
// handle's own tables [P][len] (alpha pairs read the alpha table, beta pairs
// the beta table; the other spin's rows are zero).
static int prepare_spin(fqegpu_ham h, const double* h_h1, const double* h_h2) {
  PairMatrix pm;
  const fqegpu_graph_s* g = h->g;
  prepare_pairs_spin(h->norb, g->nalpha, g->nbeta, (const zd*)h_h1, (const zd*)h_h2, pm);
  h->spin = true;
  FQE_TRY(upload_pairs(h, pm));
  if (h->zero) return FQEGPU_OK;
  const int P = h->P, per = P / 2;
  const int64_t lena = g->a.len, lenb = g->b.len;
  const int32_t* srcA = h->compressed ? g->a.tab_tri : g->a.tab_full;
  const int32_t* srcB = h->compressed ? g->b.tab_tri : g->b.tab_full;
  FQE_CUDA(dev_alloc(&h->d_tabA, sizeof(int32_t) * (size_t)P * (size_t)std::max<int64_t>(lena, 1)));
  FQE_CUDA(dev_alloc(&h->d_tabB, sizeof(int32_t) * (size_t)P * (size_t)std::max<int64_t>(lenb, 1)));
  FQE_CUDA(cudaMemset(h->d_tabA, 0, sizeof(int32_t) * (size_t)P * lena));
  FQE_CUDA(cudaMemset(h->d_tabB, 0, sizeof(int32_t) * (size_t)P * lenb));
  FQE_CUDA(cudaMemcpy(h->d_tabA, srcA, sizeof(int32_t) * (size_t)per * lena,
                      cudaMemcpyDeviceToDevice));
  FQE_CUDA(cudaMemcpy(h->d_tabB + (size_t)per * lenb, srcB, sizeof(int32_t) * (size_t)per * lenb,
                      cudaMemcpyDeviceToDevice));
  return FQEGPU_OK;
}

static int upload_pairs(fqegpu_ham h, PairMatrix& pm) {
  h->h1p = std::move(pm.h1p);
  h->v2 = std::move(pm.v2);
  h->onebody = pm.onebody;
  h->zero = pm.zero;
  if (h->zero) {
    h->P = 0;
    return FQEGPU_OK;
  }
  h->real = pm.real;
  h->phase = pm.phase;
  h->compressed = pm.compressed;
  const int P = pm.P;
  h->P = P;
  if (h->onebody) {
    if (pm.real) {
      FQE_CUDA(dev_alloc(&h->d_h1r, sizeof(double) * P));
      FQE_CUDA(cudaMemcpy(h->d_h1r, pm.vr.data(), sizeof(double) * P, cudaMemcpyHostToDevice));
    } else {
      FQE_CUDA(dev_alloc(&h->d_h1c, sizeof(double2) * P));
      FQE_CUDA(cudaMemcpy(h->d_h1c, pm.vc.data(), sizeof(double2) * P, cudaMemcpyHostToDevice));
    }
    return FQEGPU_OK;
  }
  if (pm.real) {
    FQE_CUDA(dev_alloc(&h->d_Vr, sizeof(double) * P * P));
    FQE_CUDA(cudaMemcpy(h->d_Vr, pm.vr.data(), sizeof(double) * P * P, cudaMemcpyHostToDevice));
    h->vpair = std::move(pm.vr);
  } else {
    FQE_CUDA(dev_alloc(&h->d_Vc, sizeof(double2) * P * P));
    FQE_CUDA(cudaMemcpy(h->d_Vc, pm.vc.data(), sizeof(double2) * P * P, cudaMemcpyHostToDevice));
  }
  return FQEGPU_OK;
}

static void ham_free(fqegpu_ham h) {
  if (!h) return;
  taylor_destroy(h);
  ozaki_destroy(h);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  for (cudaEvent_t e : h->out_ev)
    if (e) cudaEventDestroy(e);
  if (h->out_stream) cudaStreamDestroy(h->out_stream);
  cudaFree(h->d_Vr);
  cudaFree(h->d_Vc);
  cudaFree(h->d_h1r);
  cudaFree(h->d_h1c);
  cudaFree(h->d_ws);
  cudaFree(h->d_vec);
  cudaFree(h->d_red);
  cudaFree(h->d_tabA);
  cudaFree(h->d_tabB);
  delete h;
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_ham_create(fqegpu_graph g, const double* h_h1,
                                 const double* h_h2, void* stream,
                                 fqegpu_ham* out) {
  clear_error();
  (void)stream;
  FQE_CHECK_ARG(g != nullptr && out != nullptr, "graph/out is NULL");
  auto* h = new (std::nothrow) fqegpu_ham_s();
  if (!h) {
    set_error("host allocation failed");
    return FQEGPU_ERR_NOMEM;
  }
  h->g = g;
  h->norb = g->norb;
  h->nele = g->nalpha + g->nbeta;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = (size_t)8 << 30;
  h->scratch_limit = (int64_t)(0.4 * (double)fr);
  const int s = prepare(h, h_h1, h_h2);
  if (s != FQEGPU_OK) {
    ham_free(h);
    return s;
  }
  *out = h;
  return FQEGPU_OK;
}

extern "C" int fqegpu_ham_create_spin(fqegpu_graph g, const double* h_h1,
                                      const double* h_h2, void* stream, fqegpu_ham* out) {
  clear_error();
  (void)stream;
  FQE_CHECK_ARG(g != nullptr && out != nullptr, "graph/out is NULL");
  auto* h = new (std::nothrow) fqegpu_ham_s();
  if (!h) {
    set_error("host allocation failed");
    return FQEGPU_ERR_NOMEM;
  }
  h->g = g;
  h->norb = g->norb;
  h->nele = g->nalpha + g->nbeta;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = (size_t)8 << 30;
  h->scratch_limit = (int64_t)(0.4 * (double)fr);
  const int s = prepare_spin(h, h_h1, h_h2);
  if (s != FQEGPU_OK) {
    ham_free(h);
    return s;
  }
  *out = h;
  return FQEGPU_OK;
}

extern "C" int fqegpu_ham_destroy(fqegpu_ham h) {
  clear_error();
  if (h && h->live_graphs > 0) {
    set_error("handle is held by %d recorded CUDA graph(s); destroy them first",
              h->live_graphs);
    return FQEGPU_ERR_INVALID;
  }
  ham_free(h);
  return FQEGPU_OK;
}

extern "C" int fqegpu_ham_info(fqegpu_ham h, int64_t* info4) {
  clear_error();
  FQE_CHECK_ARG(h && info4, "bad arguments");
  info4[0] = h->P;
  info4[1] = h->compressed ? 1 : 0;
  info4[2] = h->real ? 1 : 0;
  info4[3] = (int64_t)h->ws_bytes;
  return FQEGPU_OK;
}

extern "C" int fqegpu_ham_set_scratch_limit(fqegpu_ham h, int64_t bytes) {
  clear_error();
  FQE_CHECK_ARG(h && bytes > 0, "bad arguments");
  FQE_CHECK_ARG(h->live_graphs == 0,
                "the handle is held by a recorded CUDA graph (batch); destroy it first");
  h->scratch_limit = bytes;
  return FQEGPU_OK;
}

extern "C" int fqegpu_apply(fqegpu_ham h, const double* d_psi, double* d_sigma,
                            double alpha_re, double alpha_im, double beta_re,
                            double beta_im, int precision, void* stream) {
  clear_error();
  FQE_CHECK_ARG(h && d_psi && d_sigma, "NULL handle or buffer");
  FQE_CHECK_ARG(d_psi != d_sigma, "psi and sigma must not alias");
  const double2 al = make_double2(alpha_re, alpha_im);
  const double2 be = make_double2(beta_re, beta_im);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == FQEGPU_PREC_FP64)
    return apply_fp64(h, (const double2*)d_psi, (double2*)d_sigma, al, be, st);
  if (precision == FQEGPU_PREC_OZAKI)
    return apply_ozaki(h, (const double2*)d_psi, (double2*)d_sigma, al, be, st);
  set_error("unknown precision %d", precision);
  return FQEGPU_ERR_INVALID;
}

extern "C" int fqegpu_apply_host(fqegpu_ham h, const double* h_psi,
                                 double* h_sigma, double alpha_re,
                                 double alpha_im, double beta_re, double beta_im,
                                 int precision) {
  clear_error();
  FQE_CHECK_ARG(h && h_psi && h_sigma, "NULL handle or buffer");
  const int64_t N = h->g->a.len * h->g->b.len;
  // device staging: the handle's two-vector work buffer (also the Taylor
  // workspace), allocated once and kept, so a call costs the two copies and
  // the apply
  if (!h->d_vec) FQE_CUDA(dev_alloc(&h->d_vec, sizeof(double2) * 2 * (size_t)N));
  double2* d = h->d_vec;
  // the tensor-core path copies sigma out in row chunks on a copy stream of
  // the handle, behind the scatter of each chunk
  HostOut ho;
  if (precision == FQEGPU_PREC_OZAKI) {
    if (!h->out_stream) {
      FQE_CUDA(cudaStreamCreateWithFlags(&h->out_stream, cudaStreamNonBlocking));
      for (int k = 0; k < kOutChunks; ++k)
        FQE_CUDA(cudaEventCreateWithFlags(&h->out_ev[k], cudaEventDisableTiming));
    }
    ho.h_sigma = reinterpret_cast<double2*>(h_sigma);
    ho.copy = h->out_stream;
    ho.ev = h->out_ev;
  }
  int s = FQEGPU_OK;
  cudaError_t e = cudaMemcpy(d, h_psi, sizeof(double2) * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    if (precision == FQEGPU_PREC_OZAKI) {
      clear_error();
      s = apply_ozaki(h, d, d + N, make_double2(alpha_re, alpha_im),
                      make_double2(beta_re, beta_im), nullptr, &ho);
    } else {
      s = fqegpu_apply(h, (const double*)d, (double*)(d + N), alpha_re, alpha_im,
                       beta_re, beta_im, precision, nullptr);
    }
    if (ho.issued) {
      const cudaError_t e2 = cudaStreamSynchronize(h->out_stream);
      if (s == FQEGPU_OK) e = e2;
    } else if (s == FQEGPU_OK) {
      e = cudaMemcpy(h_sigma, d + N, sizeof(double2) * N, cudaMemcpyDeviceToHost);
    }
  }
  if (e != cudaSuccess) {
    set_error("apply_host: %s", cudaGetErrorString(e));
    return FQEGPU_ERR_CUDA;
  }
  if (s == FQEGPU_OK && h->oz) s = ozaki_check(h, nullptr);  // synchronous call: report now
  return s;
}

extern "C" int fqegpu_ham_check(fqegpu_ham h, void* stream) {
  clear_error();
  FQE_CHECK_ARG(h != nullptr, "NULL handle");
  FQE_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (h->oz) return ozaki_check(h, (cudaStream_t)stream);
  return FQEGPU_OK;
}

extern "C" int fqegpu_ham_set_tuning(fqegpu_ham h, int super_tiles, int use_fp64) {
  clear_error();
  FQE_CHECK_ARG(h != nullptr, "NULL handle");
  FQE_CHECK_ARG(super_tiles >= 0 && super_tiles <= 4096, "super_tiles out of range");
  const int s = ozaki_set_tuning(h, super_tiles, use_fp64);
  // an operator without a tensor-core form always runs the FP64 kernels
  return s == FQEGPU_ERR_UNSUPPORTED ? FQEGPU_OK : s;
}

extern "C" int fqegpu_ham_test_injection(fqegpu_ham h, int64_t wait_cycles, int skip_slot) {
  clear_error();
  FQE_CHECK_ARG(h != nullptr, "NULL handle");
  FQE_CHECK_ARG(skip_slot >= -1, "skip_slot must be >= -1");
  return ozaki_set_test_injection(h, (long long)wait_cycles, skip_slot);
}

extern "C" int fqegpu_make_dvec(fqegpu_graph g, const double* d_psi,
                                double* d_dvec, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && d_psi && d_dvec, "NULL argument");
  const int P = g->norb * g->norb;
  return launch_gather(g, g->a.tab_full, g->b.tab_full, P, 0, g->b.len, (const double2*)d_psi,
                       (double2*)d_dvec, (cudaStream_t)stream);
}

extern "C" int fqegpu_make_coeff(fqegpu_graph g, const double* d_dvec,
                                 double* d_out, int accumulate, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && d_dvec && d_out, "NULL argument");
  const int P = g->norb * g->norb;
  if (P == 0) return FQEGPU_OK;
  // init=1 with beta=0 writes; init=0 accumulates into d_out.
  return launch_scatter(g, g->a.tab_full, g->b.tab_full, P, 0, g->b.len, (const double2*)d_dvec,
                        (const double2*)d_out, make_double2(1.0, 0.0),
                        make_double2(0.0, 0.0), accumulate ? false : true,
                        (double2*)d_out, (cudaStream_t)stream);
}

extern "C" int fqegpu_ham_set_timing(fqegpu_ham h, int enable) {
  clear_error();
  FQE_CHECK_ARG(h != nullptr, "NULL handle");
  h->timing = enable != 0;
  return FQEGPU_OK;
}

extern "C" int fqegpu_ham_stage_ms(fqegpu_ham h, double* h_ms3) {
  clear_error();
  FQE_CHECK_ARG(h && h_ms3, "NULL argument");
  h_ms3[0] = h_ms3[1] = h_ms3[2] = 0.0;
  if (h->events_used < 4) return FQEGPU_OK;
  FQE_CUDA(cudaEventSynchronize(h->events[h->events_used - 1]));
  for (int b = 0; b + 3 < h->events_used; b += 4)
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      FQE_CUDA(cudaEventElapsedTime(&ms, h->events[b + k], h->events[b + k + 1]));
      h_ms3[k] += ms;
    }
  return FQEGPU_OK;
}

namespace fqegpu {
// Launchers of the FP64 pair contraction and of sigma = beta psi for callers
// that provide their own device memory.
int launch_pairgemm(int P, int64_t ncol, const double* Vr, const double2* Vc,
                    const double2* D, double2* G, cudaStream_t st) {
  dim3 grid((unsigned)((ncol + 63) / 64), (unsigned)((P + 63) / 64));
  if (Vc)
    k_pairgemm_f64<true><<<grid, 256, 0, st>>>(P, ncol, nullptr, Vc, D, G);
  else
    k_pairgemm_f64<false><<<grid, 256, 0, st>>>(P, ncol, Vr, nullptr, D, G);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

int launch_axpby(int64_t n, double2 beta, const double2* x, double2* y, cudaStream_t st) {
  k_axpby<<<grid_1d(n), 256, 0, st>>>(n, beta, x, y);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}
}  // namespace fqegpu
