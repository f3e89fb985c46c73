// One- and two-particle reduced density matrices through the dvec gather.
//
//   rdm1[i][j] = <bra| E_ij |ket> = sum_I conj(bra_I) D_ket[ij][I],
//   D_ket[ij][I] = <I| E_ij |ket>, E_ij = sum_spin a+_i a_j
//
// FqeData.rdm1 / _rdm1_blocked (fqe_data.py:1668-1724) forms D by blocks with
// make_dvec_part (lib/fqe_data.c:604-639) and contracts it with the bra on the
// host.  Here D is never stored: every D value is formed from the per-pair
// target tables (as the apply's gather does) and multiplied into the
// accumulation right away.  One block handles alpha rows of the sector for
// kRdmQ consecutive pairs; partial sums go to a [P][blocks] array reduced in
// a fixed order, so the result is deterministic.
#include <algorithm>
#include <vector>

#include "ham.cuh"

namespace fqegpu {
namespace {

constexpr int kRdmQ = 8;         // pairs per block (accumulators per thread)
constexpr int kRdmThreads = 256;

__global__ void __launch_bounds__(kRdmThreads) k_rdm1_partial(
    int P, int64_t lena, int64_t lenb, const int32_t* __restrict__ tabA,
    const int32_t* __restrict__ tabB, const double2* __restrict__ bra,
    const double2* __restrict__ ket, double2* __restrict__ partial) {
  const int q0 = blockIdx.y * kRdmQ;
  double re[kRdmQ], im[kRdmQ];
#pragma unroll
  for (int k = 0; k < kRdmQ; ++k) re[k] = im[k] = 0.0;
  for (int64_t a = blockIdx.x; a < lena; a += gridDim.x) {
    int32_t ca[kRdmQ];
#pragma unroll
    for (int k = 0; k < kRdmQ; ++k) ca[k] = (q0 + k < P) ? tabA[(int64_t)(q0 + k) * lena + a] : 0;
    const double2* rowb = bra + a * lenb;
    const double2* rowk = ket + a * lenb;
    for (int64_t b = threadIdx.x; b < lenb; b += blockDim.x) {
      const double2 br = rowb[b];
#pragma unroll
      for (int k = 0; k < kRdmQ; ++k) {
        if (q0 + k >= P) break;
        double vx = 0.0, vy = 0.0;
        if (ca[k]) {
          const double2 x = ket[(int64_t)(abs(ca[k]) - 1) * lenb + b];
          const double s = ca[k] > 0 ? 1.0 : -1.0;
          vx = s * x.x;
          vy = s * x.y;
        }
        const int32_t cb = tabB[(int64_t)(q0 + k) * lenb + b];
        if (cb) {
          const double2 x = rowk[abs(cb) - 1];
          const double s = cb > 0 ? 1.0 : -1.0;
          vx += s * x.x;
          vy += s * x.y;
        }
        // conj(br) * v
        re[k] += br.x * vx + br.y * vy;
        im[k] += br.x * vy - br.y * vx;
      }
    }
  }
  __shared__ double sh[kRdmQ][2][kRdmThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kRdmQ; ++k) {
    double x = re[k], y = im[k];
    for (int off = 16; off; off >>= 1) {
      x += __shfl_down_sync(0xffffffffu, x, off);
      y += __shfl_down_sync(0xffffffffu, y, off);
    }
    if (lane == 0) {
      sh[k][0][warp] = x;
      sh[k][1][warp] = y;
    }
  }
  __syncthreads();
  if (threadIdx.x < kRdmQ && q0 + (int)threadIdx.x < P) {
    const int k = threadIdx.x;
    double x = 0.0, y = 0.0;
    for (int w = 0; w < kRdmThreads / 32; ++w) {
      x += sh[k][0][w];
      y += sh[k][1][w];
    }
    partial[(int64_t)(q0 + k) * gridDim.x + blockIdx.x] = make_double2(x, y);
  }
}

__global__ void k_rdm1_final(int nparts, const double2* __restrict__ partial,
                             double2* __restrict__ out) {
  __shared__ double sx[kRdmThreads], sy[kRdmThreads];
  const double2* p = partial + (int64_t)blockIdx.x * nparts;
  double x = 0.0, y = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    x += p[i].x;
    y += p[i].y;
  }
  sx[threadIdx.x] = x;
  sy[threadIdx.x] = y;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sx[threadIdx.x] += sx[threadIdx.x + s];
      sy[threadIdx.x] += sy[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = make_double2(sx[0], sy[0]);
}

// ---- two-particle RDM: the Gram matrix of the dvecs ------------------------
//   raw[kl][ij] = sum_I conj(D_bra[kl][I]) D_ket[ij][I]
// (the one complex GEMM of FqeData.rdm12's half-filling branch,
// fqe_data.py:1762-1781, over the dvecs of calculate_dvec_spatial).  D is
// never stored: each CTA owns a 32 x 32 tile of raw (bra pairs x ket pairs)
// and a run of 32-determinant sub-blocks (one alpha row, 32 beta columns);
// per sub-block it forms the tile's 32 bra and 32 ket D rows in shared memory
// from psi through the pair tables, then accumulates in FP64.  Partial tiles
// of the CTAs of one tile are summed in a fixed order (deterministic).

constexpr int kGT = 32;    // tile edge (pairs)
constexpr int kGSub = 32;  // determinants per sub-block

__device__ __forceinline__ double2 dvec_value(int64_t p, int64_t lena, int64_t lenb, int64_t a,
                                              int64_t b, const int32_t* __restrict__ tabA,
                                              const int32_t* __restrict__ tabB,
                                              const double2* __restrict__ psi) {
  // signs applied by flipping the sign bit (integer XOR), not by FP64
  // multiplies: the Gram kernel that calls this is FP64-bound
  double vx = 0.0, vy = 0.0;
  const int32_t ca = tabA[p * lena + a];
  if (ca) {
    const double2 x = psi[(int64_t)(abs(ca) - 1) * lenb + b];
    const unsigned long long sb = ca < 0 ? 0x8000000000000000ull : 0ull;
    vx = __longlong_as_double(__double_as_longlong(x.x) ^ sb);
    vy = __longlong_as_double(__double_as_longlong(x.y) ^ sb);
  }
  const int32_t cb = tabB[p * lenb + b];
  if (cb) {
    const double2 x = psi[a * lenb + (abs(cb) - 1)];
    const unsigned long long sb = cb < 0 ? 0x8000000000000000ull : 0ull;
    vx += __longlong_as_double(__double_as_longlong(x.x) ^ sb);
    vy += __longlong_as_double(__double_as_longlong(x.y) ^ sb);
  }
  return make_double2(vx, vy);
}

// grid.x: tiles (tr, tc) in row-major order over ntile x ntile (only
// tr <= tc when `herm`), grid.y: chunks of sub-blocks.
__global__ void __launch_bounds__(256) k_rdm2_gram(
    int P, int ntile, int E, int herm, int64_t lena, int64_t lenb, int64_t nsub_b,
    const int32_t* __restrict__ tabA, const int32_t* __restrict__ tabB,
    const double2* __restrict__ bra, const double2* __restrict__ ket,
    const int32_t* __restrict__ tiles, double2* __restrict__ partial) {
  __shared__ double2 sB[kGT][kGSub + 1];
  __shared__ double2 sK[kGT][kGSub + 1];
  const int tile = tiles[blockIdx.x];
  const int tr = tile / ntile, tc = tile % ntile;
  const int r = threadIdx.x >> 3, c0 = (threadIdx.x & 7) * 4;
  double2 acc[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[i] = make_double2(0.0, 0.0);
  const int64_t nunits = lena * nsub_b;
  const int64_t u0 = nunits * blockIdx.y / gridDim.y, u1 = nunits * (blockIdx.y + 1) / gridDim.y;
  for (int64_t u = u0; u < u1; ++u) {
    const int64_t a = u / nsub_b, b0 = (u - a * nsub_b) * kGSub;
    __syncthreads();
    for (int idx = threadIdx.x; idx < 2 * E * kGSub; idx += blockDim.x) {
      const int which = idx / (E * kGSub);
      const int pp = (idx / kGSub) % E, d = idx % kGSub;
      const int64_t b = b0 + d;
      const int p = (which ? tc : tr) * E + pp;
      double2 v = make_double2(0.0, 0.0);
      if (p < P && b < lenb)
        v = dvec_value(p, lena, lenb, a, b, tabA, tabB, which ? ket : bra);
      if (which)
        sK[pp][d] = v;
      else
        sB[pp][d] = v;
    }
    __syncthreads();
    // rows r >= E (whole warps when E = 28) have no pair: they skip the
    // multiply-adds; columns >= E read unfilled entries and are never stored
    if (r < E) {
#pragma unroll 4
      for (int d = 0; d < kGSub; ++d) {
        const double2 x = sB[r][d];  // conj(x) * y
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const double2 y = sK[c0 + i][d];
          acc[i].x += x.x * y.x + x.y * y.y;
          acc[i].y += x.x * y.y - x.y * y.x;
        }
      }
    }
  }
  double2* out = partial + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * kGT * kGT;
#pragma unroll
  for (int i = 0; i < 4; ++i) out[r * kGT + c0 + i] = acc[i];
  (void)herm;
}

// raw[P][P] from the partial tiles (fixed chunk order); the lower tiles of
// a Hermitian Gram are the conjugate transposes of the upper ones.
__global__ void k_rdm2_final(int P, int ntile, int E, int herm, int ntiles, int nchunk,
                             const int32_t* __restrict__ tiles,
                             const double2* __restrict__ partial, double2* __restrict__ raw) {
  const int t = blockIdx.x;
  const int tile = tiles[t];
  const int tr = tile / ntile, tc = tile % ntile;
  for (int e = threadIdx.x; e < kGT * kGT; e += blockDim.x) {
    double x = 0.0, y = 0.0;
    for (int c = 0; c < nchunk; ++c) {
      const double2 v = partial[((int64_t)c * ntiles + t) * kGT * kGT + e];
      x += v.x;
      y += v.y;
    }
    const int ei = e / kGT, ej = e % kGT;
    const int i = tr * E + ei, j = tc * E + ej;
    if (ei < E && ej < E && i < P && j < P) {
      raw[(int64_t)i * P + j] = make_double2(x, y);
      if (herm && tr != tc) raw[(int64_t)j * P + i] = make_double2(x, -y);
    }
  }
}

}  // namespace
}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_rdm2_gram(fqegpu_graph g, const double* d_bra, const double* d_ket,
                                double* h_raw, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && d_bra && d_ket && h_raw, "NULL argument");
  const int norb = g->norb;
  const int P = norb * norb;
  if (P == 0) return FQEGPU_OK;
  const int64_t lena = g->a.len, lenb = g->b.len;
  cudaStream_t st = (cudaStream_t)stream;
  const int ntile = (P + kGT - 1) / kGT;
  // tile edge: the pairs split evenly over ntile tiles, a multiple of 4 (28
  // for P = 196, where 32 would pad to 224)
  const int E = std::min(kGT, ((P + ntile - 1) / ntile + 3) / 4 * 4);
  const int herm = d_bra == d_ket ? 1 : 0;
  std::vector<int32_t> tl;
  for (int tr = 0; tr < ntile; ++tr)
    for (int tc = herm ? tr : 0; tc < ntile; ++tc) tl.push_back(tr * ntile + tc);
  const int ntiles = (int)tl.size();
  const int64_t nsub_b = (lenb + kGSub - 1) / kGSub;
  const int64_t nunits = lena * nsub_b;
  // at least four waves of resident CTAs, and a CTA count that fills its
  // last wave as fully as the chunk choice allows (all CTAs take about the
  // same time, so a part-filled wave leaves SMs idle at the end)
  int occ = 1;
  FQE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_rdm2_gram, 256, 0));
  const int64_t slots = (int64_t)kNumSMs * std::max(occ, 1);
  const int64_t cmin = std::max<int64_t>(1, (4 * slots + ntiles - 1) / ntiles);
  int64_t best = cmin;
  double best_waste = 2.0;
  for (int64_t c = cmin; c <= 4 * cmin; ++c) {
    const int64_t T = c * ntiles, full = (T + slots - 1) / slots * slots;
    const double waste = (double)(full - T) / (double)full;
    if (waste < best_waste - 1e-12) {
      best_waste = waste;
      best = c;
    }
    if (waste < 0.02) break;
  }
  const int nchunk = (int)std::max<int64_t>(1, std::min<int64_t>(nunits, best));
  const size_t pbytes = sizeof(double2) * (size_t)nchunk * ntiles * kGT * kGT;
  const size_t rbytes = sizeof(double2) * (size_t)P * P;
  char* scratch = nullptr;
  FQE_CUDA(cudaMallocAsync(&scratch, pbytes + rbytes + sizeof(int32_t) * ntiles, st));
  double2* partial = reinterpret_cast<double2*>(scratch);
  double2* raw = reinterpret_cast<double2*>(scratch + pbytes);
  int32_t* d_tiles = reinterpret_cast<int32_t*>(scratch + pbytes + rbytes);
  cudaError_t e = cudaMemcpyAsync(d_tiles, tl.data(), sizeof(int32_t) * ntiles,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_rdm2_gram<<<dim3(ntiles, nchunk), 256, 0, st>>>(
        P, ntile, E, herm, lena, lenb, nsub_b, g->a.tab_full, g->b.tab_full,
        (const double2*)d_bra, (const double2*)d_ket, d_tiles, partial);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_rdm2_final<<<ntiles, 256, 0, st>>>(P, ntile, E, herm, ntiles, nchunk, d_tiles, partial,
                                         raw);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_raw, raw, rbytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) {
    set_error("rdm2: %s", cudaGetErrorString(e));
    return FQEGPU_ERR_CUDA;
  }
  return FQEGPU_OK;
}

extern "C" int fqegpu_rdm1(fqegpu_graph g, const double* d_bra, const double* d_ket,
                           double* h_rdm, void* stream) {
  clear_error();
  FQE_CHECK_ARG(g && d_bra && d_ket && h_rdm, "NULL argument");
  const int norb = g->norb;
  const int P = norb * norb;
  if (P == 0) return FQEGPU_OK;
  const int64_t lena = g->a.len, lenb = g->b.len;
  cudaStream_t st = (cudaStream_t)stream;
  const int nx = (int)std::min<int64_t>(lena, 1024);
  const int ny = (P + kRdmQ - 1) / kRdmQ;
  double2* scratch = nullptr;
  FQE_CUDA(cudaMallocAsync(&scratch, sizeof(double2) * ((size_t)P * nx + P), st));
  double2* d_out = scratch + (size_t)P * nx;
  k_rdm1_partial<<<dim3(nx, ny), kRdmThreads, 0, st>>>(
      P, lena, lenb, g->a.tab_full, g->b.tab_full, (const double2*)d_bra,
      (const double2*)d_ket, scratch);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_rdm1_final<<<P, kRdmThreads, 0, st>>>(nx, scratch, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_rdm, d_out, sizeof(double2) * P, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) {
    set_error("rdm1: %s", cudaGetErrorString(e));
    return FQEGPU_ERR_CUDA;
  }
  return FQEGPU_OK;
}
