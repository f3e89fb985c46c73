// Diagonal operators of one sector (A11 and the Davidson diagonal of A12).
//
// All three are "separable" determinant energies
//   E(a, b) = f(a) + f(b) + sum_{k in b} row_a[k]
// with per-string terms f(s) = sum_{i in s} d_i + sum_{i,k in s} A_ik
// + sum_{i in s, j not in s} B_ij and an alpha-dependent row
// row_a[k] = sum_{x in a} R[x][k]:
//   mode 0 evolve   (zdiagonal_coulomb, lib/fqe_data.c:526-602):
//                   d = diag, A = V, B = 0, R = 2V;  psi *= exp(E)
//   mode 1 apply    (zdiagonal_coulomb_apply, lib/fqe_data.c:455-524):
//                   d = diag, A = V, B = 0, R = V + V^T;  psi *= E
//   mode 2 Slater-Condon diagonal of the restricted Hamiltonian,
//                   <I|H|I> = sum_i h1'_ii n_i + sum_ik V'[ii,kk] n_i n_k
//                           + sum_{i!=j} V'[ij,ji] sum_s n_is (1 - n_js)
//                   d = diag h1', A = J, B = K, R = J + J^T;  out = Re E
// The evolve multiplies exp(f(a)) exp(f(b)) prod_{k in b} exp(row_a[k]); the
// reference forms the same product from exponentials of the individual
// integrals, so the two agree to rounding.
#include <cmath>
#include <vector>

#include "ham.cuh"

namespace fqegpu {

constexpr int kMaxOrb = 64;

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ double2 zexp(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = exp(z.x);
  return make_double2(e * c, e * s);
}

struct DiagTerms {
  const double2* d;  // [norb]
  const double2* A;  // [norb][norb]
  const double2* B;  // [norb][norb] or nullptr
  const double2* R;  // [norb][norb]
};

// f(s) (or exp(f(s)) when EXP) for every string of one spin.
template <bool EXP>
__global__ void k_string_terms(int norb, int64_t len,
                               const uint64_t* __restrict__ strings, DiagTerms T,
                               double2* __restrict__ out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= len) return;
  const uint64_t S = strings[s];
  double2 f = make_double2(0.0, 0.0);
  for (uint64_t m = S; m; m &= m - 1) {
    const int i = __ffsll((long long)m) - 1;
    f.x += T.d[i].x;
    f.y += T.d[i].y;
    for (uint64_t q = S; q; q &= q - 1) {
      const int k = __ffsll((long long)q) - 1;
      f.x += T.A[i * norb + k].x;
      f.y += T.A[i * norb + k].y;
    }
    if (T.B) {
      for (int j = 0; j < norb; ++j) {
        if (S >> j & 1ull) continue;
        f.x += T.B[i * norb + j].x;
        f.y += T.B[i * norb + j].y;
      }
    }
  }
  out[s] = EXP ? zexp(f) : f;
}

// One CTA per alpha string; threads over beta strings.  The evolve (mode 0)
// with norb <= 16 splits the beta string into a low half of h orbitals and a
// high half: per CTA, tlo[m] = exp(f(a)) prod_{k in m} exp(row_a[k]) and
// thi[m] = prod_{k in m} exp(row_a[h + k]) (built by doubling), so a
// determinant costs three complex products instead of one per beta electron
// (FP64 is the limit of this kernel on GB300).
template <int MODE>
__global__ void __launch_bounds__(256) k_diag_apply(
    int norb, int64_t lena, int64_t lenb, const uint64_t* __restrict__ astr,
    const uint64_t* __restrict__ bstr, const double2* __restrict__ R,
    const double2* __restrict__ fa, const double2* __restrict__ fb,
    double2* __restrict__ psi, double* __restrict__ diag_out) {
  __shared__ double2 row[kMaxOrb];
  __shared__ double2 tlo[256], thi[256];
  const int64_t a = blockIdx.x;
  const uint64_t Sa = astr[a];
  for (int k = threadIdx.x; k < norb; k += blockDim.x) {
    double2 r = make_double2(0.0, 0.0);
    for (uint64_t m = Sa; m; m &= m - 1) {
      const int x = __ffsll((long long)m) - 1;
      r.x += R[x * norb + k].x;
      r.y += R[x * norb + k].y;
    }
    row[k] = (MODE == 0) ? zexp(r) : r;
  }
  __syncthreads();
  const double2 fav = fa[a];
  if (MODE == 0 && norb <= 16) {
    const int h = (norb + 1) / 2, hh = norb - h;  // both <= 8
    if (threadIdx.x == 0) {
      tlo[0] = fav;
      thi[0] = make_double2(1.0, 0.0);
    }
    __syncthreads();
    for (int j = 0; j < 8; ++j) {
      const int w = 1 << j, t = threadIdx.x;  // entries [w, 2w) from [0, w)
      if (j < h && t < w) tlo[w + t] = zmul(tlo[t], row[j]);
      if (j < hh && t < w) thi[w + t] = zmul(thi[t], row[h + j]);
      __syncthreads();
    }
    const uint64_t lomask = (1ull << h) - 1ull;
    for (int64_t b = threadIdx.x; b < lenb; b += blockDim.x) {
      const uint64_t Sb = bstr[b];
      const int64_t I = a * lenb + b;
      const double2 p = zmul(zmul(tlo[Sb & lomask], thi[Sb >> h]), fb[b]);
      psi[I] = zmul(psi[I], p);
    }
    return;
  }
  for (int64_t b = threadIdx.x; b < lenb; b += blockDim.x) {
    const uint64_t Sb = bstr[b];
    const int64_t I = a * lenb + b;
    if (MODE == 0) {
      double2 p = zmul(fav, fb[b]);
      for (uint64_t m = Sb; m; m &= m - 1) p = zmul(p, row[__ffsll((long long)m) - 1]);
      psi[I] = zmul(psi[I], p);
    } else {
      double2 e = make_double2(fav.x + fb[b].x, fav.y + fb[b].y);
      for (uint64_t m = Sb; m; m &= m - 1) {
        const double2 r = row[__ffsll((long long)m) - 1];
        e.x += r.x;
        e.y += r.y;
      }
      if (MODE == 1)
        psi[I] = zmul(psi[I], e);
      else
        diag_out[I] = e.x;
    }
  }
}

// Uploads the term arrays, runs the two kernels, frees the temporaries.
static int run_diag(const fqegpu_graph_s* g, int mode,
                    const std::vector<double2>& d, const std::vector<double2>& A,
                    const std::vector<double2>& B, const std::vector<double2>& R,
                    double2* psi, double* out, cudaStream_t st) {
  const int n = g->norb;
  const int64_t lena = g->a.len, lenb = g->b.len;
  if (lena * lenb == 0) return FQEGPU_OK;
  const size_t n1 = (size_t)(n > 0 ? n : 1), n2 = n1 * n1;
  const size_t bytes = sizeof(double2) * (n1 + 3 * n2 + (size_t)lena + (size_t)lenb);
  double2* buf = nullptr;
  FQE_CUDA(cudaMallocAsync(&buf, bytes, st));
  double2* dd = buf;
  double2* dA = dd + n1;
  double2* dB = dA + n2;
  double2* dR = dB + n2;
  double2* fa = dR + n2;
  double2* fb = fa + lena;
  int s = FQEGPU_OK;
  cudaError_t e = cudaSuccess;
  if (n > 0) {
    e = cudaMemcpyAsync(dd, d.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dA, A.data(), sizeof(double2) * n * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !B.empty())
      e = cudaMemcpyAsync(dB, B.data(), sizeof(double2) * n * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dR, R.data(), sizeof(double2) * n * n, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) {
    DiagTerms T{dd, dA, B.empty() ? nullptr : dB, dR};
    if (mode == 0) {
      k_string_terms<true><<<(unsigned)((lena + 127) / 128), 128, 0, st>>>(n, lena, g->a.strings, T, fa);
      k_string_terms<true><<<(unsigned)((lenb + 127) / 128), 128, 0, st>>>(n, lenb, g->b.strings, T, fb);
      k_diag_apply<0><<<(unsigned)lena, 256, 0, st>>>(n, lena, lenb, g->a.strings, g->b.strings, dR, fa, fb, psi, nullptr);
    } else {
      k_string_terms<false><<<(unsigned)((lena + 127) / 128), 128, 0, st>>>(n, lena, g->a.strings, T, fa);
      k_string_terms<false><<<(unsigned)((lenb + 127) / 128), 128, 0, st>>>(n, lenb, g->b.strings, T, fb);
      if (mode == 1)
        k_diag_apply<1><<<(unsigned)lena, 256, 0, st>>>(n, lena, lenb, g->a.strings, g->b.strings, dR, fa, fb, psi, nullptr);
      else
        k_diag_apply<2><<<(unsigned)lena, 256, 0, st>>>(n, lena, lenb, g->a.strings, g->b.strings, dR, fa, fb, nullptr, out);
    }
    e = cudaGetLastError();
  }
  cudaFreeAsync(buf, st);
  if (e != cudaSuccess) {
    set_error("diagonal kernels: %s", cudaGetErrorString(e));
    s = FQEGPU_ERR_CUDA;
  }
  return s;
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_diagonal_coulomb(fqegpu_graph g, const double* h_diag,
                                       const double* h_vij, double* d_psi,
                                       int mode, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && h_diag && h_vij && d_psi, "NULL argument");
  FQE_CHECK_ARG(mode == 0 || mode == 1, "mode must be 0 (evolve) or 1 (apply)");
  const int n = g->norb;
  const double2* D = (const double2*)h_diag;
  const double2* V = (const double2*)h_vij;
  std::vector<double2> d(n), A((size_t)n * n), R((size_t)n * n), B;
  for (int i = 0; i < n; ++i) d[i] = D[i];
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      const double2 v = V[i * n + k], vt = V[k * n + i];
      A[i * n + k] = v;
      R[i * n + k] = mode == 0 ? make_double2(2.0 * v.x, 2.0 * v.y)
                               : make_double2(v.x + vt.x, v.y + vt.y);
    }
  return run_diag(g, mode, d, A, B, R, (double2*)d_psi, nullptr,
                  (cudaStream_t)stream);
}

extern "C" int fqegpu_diagonal(fqegpu_ham h, double* d_diag, void* stream) {
  clear_error();
  FQE_CHECK_ARG(h && d_diag, "NULL argument");
  if (h->spin) {
    set_error("the Slater-Condon diagonal is implemented for restricted operators only");
    return FQEGPU_ERR_UNSUPPORTED;
  }
  const int n = h->norb, n2 = n * n;
  std::vector<double2> d(n), A((size_t)n2), B((size_t)n2), R((size_t)n2);
  for (int i = 0; i < n; ++i) {
    const zd v = h->h1p.empty() ? zd(0, 0) : h->h1p[i * n + i];
    d[i] = make_double2(v.real(), v.imag());
  }
  auto V = [&](int i, int j, int k, int l) -> zd {
    if (h->v2.empty()) return zd(0.0, 0.0);
    return h->v2[(size_t)(i * n + j) * n2 + (k * n + l)];
  };
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      const zd J = V(i, i, k, k), Jt = V(k, k, i, i);
      const zd K = (i == k) ? zd(0, 0) : V(i, k, k, i);
      A[i * n + k] = make_double2(J.real(), J.imag());
      B[i * n + k] = make_double2(K.real(), K.imag());
      R[i * n + k] = make_double2(J.real() + Jt.real(), J.imag() + Jt.imag());
    }
  return run_diag(h->g, 2, d, A, B, R, nullptr, d_diag, (cudaStream_t)stream);
}
