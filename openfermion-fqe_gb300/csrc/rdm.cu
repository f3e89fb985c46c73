// One-particle reduced density matrix through the dvec gather.
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

}  // namespace
}  // namespace fqegpu

using namespace fqegpu;

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
