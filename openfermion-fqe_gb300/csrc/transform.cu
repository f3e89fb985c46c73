// Orbital rotation of a sector's coefficients and the diagonal one-body
// evolution (the quadratic branch of time evolution).
//
// Reference: Wavefunction.transform (wavefunction.py:813-959) calls
// FqeData.apply_columns_recursive_inplace (fqe_data.py:1476-1535), which for
// every orbital column icol = 0 .. norb-1, first on alpha strings and then on
// beta strings, applies the column operator
//
//   X_icol = 1 + sum_i m[i][icol] E_{i,icol}        (E_ij = a+_i a_j)
//
// in place (lm_apply_array1_column_alpha, lib/fqe_data.c:305-347): a string T
// with icol empty gains sum_{i in T} m[i][icol] <T|E_{i,icol}|S> c[S] from
// the string S = T - i + icol, and a string with icol occupied is scaled by
// 1 + m[icol][icol].  Targets (icol empty) and sources (icol occupied) are
// disjoint, so each column step is a well-defined linear map of the whole
// array; here it is one kernel pass from one buffer into another (the
// caller's work array), 2 norb passes in all, ending in the caller's array.
// The sources come from the graph's per-pair tables tab_full[(i, icol)][T] =
// sign * (S + 1) (the same tables the apply reads), so no column tables are
// built.  Alpha passes move whole rows (coalesced), beta passes gather inside
// a row.
//
// FqeData.evolve_diagonal (fqe_data.py:203-262, evolve_diagonal_inplace in the
// C library): c[a][b] *= exp(sum_{i in a} da[i] + sum_{j in b} db[j]), with
// the exponentials formed per string (one exp per string, CUDA's exp and
// sincos) and applied as exp(Ea) exp(Eb).
#include <algorithm>
#include <vector>

#include "ham.cuh"

namespace fqegpu {

namespace {
constexpr int kMaxOrb = 64;

struct ColumnCoefs {
  double2 m[kMaxOrb];  // m[i][icol] for i = 0 .. norb-1
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// acc += (neg ? -m : m) * v in four FP64 FMAs: the sign is flipped in m's
// bits (integer XOR), not by an FP64 multiply or subtraction (the column
// steps are FP64-bound on GB300).
__device__ __forceinline__ void signed_madd(double2& acc, double2 m, double2 v, bool neg) {
  const unsigned long long sb = neg ? 0x8000000000000000ull : 0ull;
  const double mx = __longlong_as_double(__double_as_longlong(m.x) ^ sb);
  const double my = __longlong_as_double(__double_as_longlong(m.y) ^ sb);
  acc.x = fma(mx, v.x, acc.x);
  acc.x = fma(-my, v.y, acc.x);
  acc.y = fma(mx, v.y, acc.y);
  acc.y = fma(my, v.x, acc.y);
}
}  // namespace

// The source lookups of a column step come in groups of kGroup: the group's
// table entries are read first, then its source values, then they are
// accumulated in orbital order (the order of the one-at-a-time loop, so the
// sums are the same), which keeps kGroup loads in flight per thread.
constexpr int kGroup = 8;

// Alpha column step: one CTA per (target row T, block of beta columns).
__global__ void __launch_bounds__(256) k_column_alpha(int norb, int icol, int64_t lena,
                                                      int64_t lenb,
                                                      const int32_t* __restrict__ tab,
                                                      ColumnCoefs cf,
                                                      const double2* __restrict__ in,
                                                      double2* __restrict__ out) {
  const int64_t T = blockIdx.y;
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= lenb) return;
  const double2 x = in[T * lenb + b];
  if (tab[(int64_t)(icol * norb + icol) * lena + T]) {  // icol occupied in T
    const double2 s = make_double2(1.0 + cf.m[icol].x, cf.m[icol].y);
    out[T * lenb + b] = cmul(s, x);
    return;
  }
  double2 acc = x;
  for (int i0 = 0; i0 < norb; i0 += kGroup) {
    int32_t c[kGroup];
    double2 v[kGroup];
#pragma unroll
    for (int u = 0; u < kGroup; ++u) {  // uniform in the CTA
      const int i = i0 + u;
      c[u] = (i < norb && i != icol) ? tab[(int64_t)(i * norb + icol) * lena + T] : 0;
    }
#pragma unroll
    for (int u = 0; u < kGroup; ++u)
      v[u] = c[u] ? in[(int64_t)(abs(c[u]) - 1) * lenb + b] : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < kGroup; ++u)
      if (c[u]) signed_madd(acc, cf.m[i0 + u], v[u], c[u] < 0);
  }
  out[T * lenb + b] = acc;
}

// Beta column step: one thread per (alpha row, target beta string).
__global__ void __launch_bounds__(256) k_column_beta(int norb, int icol, int64_t lenb,
                                                     const int32_t* __restrict__ tab,
                                                     ColumnCoefs cf,
                                                     const double2* __restrict__ in,
                                                     double2* __restrict__ out) {
  const int64_t a = blockIdx.y;
  const int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (T >= lenb) return;
  const double2* row = in + a * lenb;
  const double2 x = row[T];
  if (tab[(int64_t)(icol * norb + icol) * lenb + T]) {
    const double2 s = make_double2(1.0 + cf.m[icol].x, cf.m[icol].y);
    out[a * lenb + T] = cmul(s, x);
    return;
  }
  double2 acc = x;
  for (int i0 = 0; i0 < norb; i0 += kGroup) {
    int32_t c[kGroup];
    double2 v[kGroup];
#pragma unroll
    for (int u = 0; u < kGroup; ++u) {
      const int i = i0 + u;
      c[u] = (i < norb && i != icol) ? tab[(int64_t)(i * norb + icol) * lenb + T] : 0;
    }
#pragma unroll
    for (int u = 0; u < kGroup; ++u)
      v[u] = c[u] ? row[abs(c[u]) - 1] : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < kGroup; ++u)
      if (c[u]) signed_madd(acc, cf.m[i0 + u], v[u], c[u] < 0);
  }
  out[a * lenb + T] = acc;
}

// Per-string factors exp(sum_{i in s} d[i]) of both spins.
__global__ void k_string_exp(int norb, int64_t lena, int64_t lenb,
                             const uint64_t* __restrict__ astr, const uint64_t* __restrict__ bstr,
                             ColumnCoefs da, ColumnCoefs db, double2* __restrict__ fa,
                             double2* __restrict__ fb) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= lena + lenb) return;
  const bool alpha = k < lena;
  const uint64_t s = alpha ? astr[k] : bstr[k - lena];
  const ColumnCoefs& d = alpha ? da : db;
  double re = 0.0, im = 0.0;
  for (int i = 0; i < norb; ++i)
    if (s >> i & 1ull) {
      re += d.m[i].x;
      im += d.m[i].y;
    }
  const double m = exp(re);
  double sn, cs;
  sincos(im, &sn, &cs);
  if (alpha)
    fa[k] = make_double2(m * cs, m * sn);
  else
    fb[k - lena] = make_double2(m * cs, m * sn);
}

__global__ void k_apply_string_factors(int64_t lena, int64_t lenb, const double2* __restrict__ fa,
                                       const double2* __restrict__ fb, double2* __restrict__ psi) {
  const int64_t n = lena * lenb;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i / lenb, b = i - a * lenb;
    psi[i] = cmul(cmul(fa[a], fb[b]), psi[i]);
  }
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_transform(fqegpu_graph g, const double* h_mat_a, const double* h_mat_b,
                                double* d_psi, double* d_work, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && h_mat_a && h_mat_b && d_psi && d_work, "NULL argument");
  FQE_CHECK_ARG(d_psi != d_work, "psi and work must be distinct buffers");
  const int n = g->norb;
  FQE_CHECK_ARG(n <= kMaxOrb, "norb above 64");
  const int64_t lena = g->a.len, lenb = g->b.len;
  if (n == 0 || lena * lenb == 0) return FQEGPU_OK;
  if (lena > 65535 || lenb > 65535) {
    set_error("string spaces above 65535 strings exceed one launch's rows");
    return FQEGPU_ERR_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const double2* ma = reinterpret_cast<const double2*>(h_mat_a);
  const double2* mb = reinterpret_cast<const double2*>(h_mat_b);
  double2* buf[2] = {reinterpret_cast<double2*>(d_psi), reinterpret_cast<double2*>(d_work)};
  int cur = 0;
  for (int spin = 0; spin < 2; ++spin) {
    const double2* m = spin == 0 ? ma : mb;
    for (int icol = 0; icol < n; ++icol) {
      ColumnCoefs cf;
      for (int i = 0; i < n; ++i) cf.m[i] = m[(size_t)i * n + icol];
      dim3 grid((unsigned)((lenb + 255) / 256), (unsigned)lena);
      if (spin == 0)
        k_column_alpha<<<grid, 256, 0, st>>>(n, icol, lena, lenb, g->a.tab_full, cf, buf[cur],
                                             buf[cur ^ 1]);
      else
        k_column_beta<<<grid, 256, 0, st>>>(n, icol, lenb, g->b.tab_full, cf, buf[cur],
                                            buf[cur ^ 1]);
      FQE_CUDA(cudaGetLastError());
      cur ^= 1;
    }
  }
  // 2 n passes: the result is back in psi
  return FQEGPU_OK;
}

extern "C" int fqegpu_evolve_diagonal(fqegpu_graph g, const double* h_diag_a,
                                      const double* h_diag_b, double* d_psi, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && h_diag_a && h_diag_b && d_psi, "NULL argument");
  const int n = g->norb;
  FQE_CHECK_ARG(n <= kMaxOrb, "norb above 64");
  const int64_t lena = g->a.len, lenb = g->b.len;
  if (lena * lenb == 0) return FQEGPU_OK;
  cudaStream_t st = (cudaStream_t)stream;
  ColumnCoefs da, db;
  for (int i = 0; i < n; ++i) {
    da.m[i] = reinterpret_cast<const double2*>(h_diag_a)[i];
    db.m[i] = reinterpret_cast<const double2*>(h_diag_b)[i];
  }
  double2* f = nullptr;
  FQE_CUDA(cudaMallocAsync(&f, sizeof(double2) * (size_t)(lena + lenb), st));
  k_string_exp<<<(unsigned)((lena + lenb + 255) / 256), 256, 0, st>>>(
      n, lena, lenb, g->a.strings, g->b.strings, da, db, f, f + lena);
  k_apply_string_factors<<<kNumSMs * 8, 256, 0, st>>>(lena, lenb, f, f + lena,
                                                      reinterpret_cast<double2*>(d_psi));
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(f, st);
  FQE_CUDA(e);
  return FQEGPU_OK;
}
