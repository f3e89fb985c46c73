// Learned Davidson preconditioner: a 34 -> 64 -> 64 -> 1 MLP per determinant.
//
// The reference Davidson (algorithm/davidson.py:273-280) preconditions with
// 1 / (theta - H_II).  Here a small network reads, per determinant I, the
// diagonal energy and the Ritz value (shifted and scaled) and 32 occupation
// bits, and returns a multiplier m_I in (0, 2):
//     t_I = m_I r_I / (theta - H_II)           (|theta - H_II| floored)
// m = 1 is the plain preconditioner (the untrained network has a zero output
// layer).  Weights are bfloat16 (rounded from a float32 master copy), sums
// and activations float32.  Training minimises, per correction-equation
// sample (u = r / d, Ritz vector x, exact correction a, a _|_ x),
//     L = 1 - |a^H v|^2 / (|a|^2 |v|^2),   v = w - x (x^H w),  w = m * u,
// with its gradient from hand-written backward kernels and Adam on the
// master copy.  Feature encoding, network and loss are restated in FP64 by
// the oracle (oracle/mlp_oracle.py), which the tests compare against.
//
// Kernels (all grid-stride over determinants, weights staged in shared
// memory as float32):
//   k_mlp_infer   forward + preconditioning (or the multiplier alone)
//   k_mlp_fwd     forward + per-block FP64 partial sums of x^H w, w^H w,
//                 a^H w, a^H a, a^H x
//   k_mlp_red     deterministic reduction of the partial sums
//   k_mlp_bwd     forward again (activations are recomputed, not stored),
//                 dL/dm_I, backward through the three layers, per-block
//                 partial parameter gradients held in registers
//   k_mlp_gsum    deterministic sum of the per-block gradients
//   k_mlp_adam    Adam step on the master copy, bf16 weights refreshed
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "ham.cuh"

namespace fqegpu {
namespace mlp {

constexpr int kIn = 34, kH = 64;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kH * kIn;  // 2176
constexpr int kOffW2 = kOffB1 + kH;        // 2240
constexpr int kOffB2 = kOffW2 + kH * kH;   // 6336
constexpr int kOffW3 = kOffB2 + kH;        // 6400
constexpr int kOffB3 = kOffW3 + kH;        // 6464
constexpr int kParams = kOffB3 + 1;        // 6465
constexpr int kW1Pad = 36;                 // W1 rows padded for float4 loads
// shared-memory weight image (floats): W1 [64][36], b1, W2 [64][64], b2, w3, b3
constexpr int kSW1 = 0, kSB1 = kSW1 + kH * kW1Pad, kSW2 = kSB1 + kH,
              kSB2 = kSW2 + kH * kH, kSW3 = kSB2 + kH, kSB3 = kSW3 + kH,
              kSWeights = kSB3 + 4;  // 6596 floats (16-byte multiple)
constexpr int kTile = 128;             // determinants per backward tile
constexpr int kRow = kH + 1;           // padded activation row
constexpr int kFRow = kIn + 1;
constexpr int kPerThread = (kParams + kTile - 1) / kTile;  // 51
constexpr int kRed = 8;                // reduced scalars
constexpr int kBwdBlocks = kNumSMs;    // one 128-thread block per SM

struct Feat {
  int nalpha, nbeta, lenb;
  const uint64_t* astr;
  const uint64_t* bstr;
  double theta, inv_scale, f1;
};

// Fermi-aligned occupation slots (slot k <-> orbital k - 8 + nele): 16 bits.
__device__ __forceinline__ uint32_t slots(uint64_t s, int nele) {
  const int sh = 8 - nele;
  uint64_t v;
  if (sh >= 0) v = (s << sh) | ((1ull << sh) - 1ull);
  else v = s >> (-sh);
  return (uint32_t)(v & 0xFFFFull);
}

__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ w, float* sw) {
  for (int p = threadIdx.x; p < kSWeights; p += blockDim.x) {
    float v = 0.f;
    if (p < kSB1) {
      const int o = p / kW1Pad, i = p % kW1Pad;
      if (i < kIn) v = __bfloat162float(w[kOffW1 + o * kIn + i]);
    } else if (p < kSB3 + 1) {
      v = __bfloat162float(w[kOffB1 + (p - kSB1)]);  // b1, W2, b2, w3, b3 contiguous
    }
    sw[p] = v;
  }
}

__device__ __forceinline__ void features(const Feat& F, int64_t I, double diag, float (&f)[kIn]) {
  const int64_t a = I / F.lenb, b = I - a * F.lenb;
  const uint32_t sa = slots(F.astr[a], F.nalpha), sb = slots(F.bstr[b], F.nbeta);
  f[0] = (float)((diag - F.theta) * F.inv_scale);
  f[1] = (float)F.f1;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    f[2 + k] = (float)((sa >> k) & 1u);
    f[18 + k] = (float)((sb >> k) & 1u);
  }
}

// z1 = W1 f + b1 (row o of W1 padded to 36)
__device__ __forceinline__ float layer1(const float* sw, int o, const float (&f)[kIn]) {
  const float4* row = reinterpret_cast<const float4*>(sw + kSW1 + o * kW1Pad);
  float acc = sw[kSB1 + o];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 w = row[q];
    acc = fmaf(w.x, f[4 * q], acc);
    acc = fmaf(w.y, f[4 * q + 1], acc);
    acc = fmaf(w.z, f[4 * q + 2], acc);
    acc = fmaf(w.w, f[4 * q + 3], acc);
  }
  const float2 w = *reinterpret_cast<const float2*>(sw + kSW1 + o * kW1Pad + 32);
  acc = fmaf(w.x, f[32], acc);
  acc = fmaf(w.y, f[33], acc);
  return acc;
}

__device__ __forceinline__ float layer2(const float* sw, int o, const float (&h1)[kH]) {
  const float4* row = reinterpret_cast<const float4*>(sw + kSW2 + o * kH);
  float acc = sw[kSB2 + o];
#pragma unroll
  for (int q = 0; q < kH / 4; ++q) {
    const float4 w = row[q];
    acc = fmaf(w.x, h1[4 * q], acc);
    acc = fmaf(w.y, h1[4 * q + 1], acc);
    acc = fmaf(w.z, h1[4 * q + 2], acc);
    acc = fmaf(w.w, h1[4 * q + 3], acc);
  }
  return acc;
}

// m = 1 + tanh(z3)
__device__ __forceinline__ float forward(const float* sw, const float (&f)[kIn]) {
  float h1[kH];
#pragma unroll
  for (int o = 0; o < kH; ++o) h1[o] = fmaxf(layer1(sw, o, f), 0.f);
  float z3 = sw[kSB3];
#pragma unroll 4
  for (int o = 0; o < kH; ++o) z3 = fmaf(sw[kSW3 + o], fmaxf(layer2(sw, o, h1), 0.f), z3);
  return 1.f + tanhf(z3);
}

__device__ __forceinline__ double floored(double theta, double diag, double floor_) {
  double den = theta - diag;
  if (fabs(den) < floor_) den = den < 0.0 ? -floor_ : floor_;
  return den;
}

// MODE 0: t = m r / d.  MODE 1: multiplier only (float m[n]).
template <int MODE>
__global__ void __launch_bounds__(256) k_mlp_infer(Feat F, int64_t n, const __nv_bfloat16* __restrict__ w,
                                                   const double2* __restrict__ r,
                                                   const double* __restrict__ diag, double floor_,
                                                   double2* __restrict__ t, float* __restrict__ mout) {
  __shared__ __align__(16) float sw[kSWeights];
  load_weights(w, sw);
  __syncthreads();
  for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < n;
       I += (int64_t)gridDim.x * blockDim.x) {
    asm volatile("" ::: "memory");  // keep the weight loads inside the loop
    const double dg = diag[I];
    float f[kIn];
    features(F, I, dg, f);
    const float m = forward(sw, f);
    if (MODE == 0) {
      const double s = (double)m / floored(F.theta, dg, floor_);
      const double2 v = r[I];
      t[I] = make_double2(v.x * s, v.y * s);
    } else {
      mout[I] = m;
    }
  }
}

// Partial sums (FP64) per block: [0..1] x^H w, [2] w^H w, [3..4] a^H w,
// [5] a^H a, [6..7] a^H x.
__global__ void __launch_bounds__(256) k_mlp_fwd(Feat F, int64_t n, const __nv_bfloat16* __restrict__ w,
                                                 const double2* __restrict__ u,
                                                 const double2* __restrict__ x,
                                                 const double2* __restrict__ a,
                                                 const double* __restrict__ diag,
                                                 double* __restrict__ part) {
  __shared__ __align__(16) float sw[kSWeights];
  __shared__ double red[kRed][8];
  load_weights(w, sw);
  __syncthreads();
  double acc[kRed] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < n;
       I += (int64_t)gridDim.x * blockDim.x) {
    asm volatile("" ::: "memory");
    float f[kIn];
    features(F, I, diag[I], f);
    const double m = forward(sw, f);
    const double2 uu = u[I], xx = x[I], aa = a[I];
    const double wr = m * uu.x, wi = m * uu.y;
    acc[0] += xx.x * wr + xx.y * wi;  // conj(x) w
    acc[1] += xx.x * wi - xx.y * wr;
    acc[2] += wr * wr + wi * wi;
    acc[3] += aa.x * wr + aa.y * wi;  // conj(a) w
    acc[4] += aa.x * wi - aa.y * wr;
    acc[5] += aa.x * aa.x + aa.y * aa.y;
    acc[6] += aa.x * xx.x + aa.y * xx.y;  // conj(a) x
    acc[7] += aa.x * xx.y - aa.y * xx.x;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kRed; ++k) {
    double v = acc[k];
    for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < kRed) {
    double v = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += red[threadIdx.x][q];
    part[(int64_t)blockIdx.x * kRed + threadIdx.x] = v;
  }
}

// scal[0..7] = sums of part over blocks, then derived:
// scal[8..9] c = x^H w, scal[10..11] s = a^H v = a^H w - (a^H x) c,
// scal[12] q = |v|^2 = w^H w - |c|^2, scal[13] A = |a|^2, scal[14] loss.
__global__ void k_mlp_red(int nblk, const double* __restrict__ part, double* __restrict__ scal) {
  __shared__ double s[kRed];
  if (threadIdx.x < kRed) {
    double v = 0.0;
    for (int b = 0; b < nblk; ++b) v += part[(int64_t)b * kRed + threadIdx.x];
    s[threadIdx.x] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double cr = s[0], ci = s[1];
    const double sr = s[3] - (s[6] * cr - s[7] * ci);
    const double si = s[4] - (s[6] * ci + s[7] * cr);
    const double q = s[2] - (cr * cr + ci * ci);
    const double A = s[5];
    for (int k = 0; k < kRed; ++k) scal[k] = s[k];
    scal[8] = cr;
    scal[9] = ci;
    scal[10] = sr;
    scal[11] = si;
    scal[12] = q;
    scal[13] = A;
    scal[14] = (A > 0.0 && q > 0.0) ? 1.0 - (sr * sr + si * si) / (A * q) : 1.0;
  }
}

__global__ void __launch_bounds__(kTile, 1) k_mlp_bwd(Feat F, int64_t n, const __nv_bfloat16* __restrict__ w,
                                                     const double2* __restrict__ u,
                                                     const double2* __restrict__ x,
                                                     const double2* __restrict__ a,
                                                     const double* __restrict__ diag,
                                                     const double* __restrict__ scal,
                                                     float* __restrict__ gpart) {
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;                           // kSWeights
  float* sh1 = sw + kSWeights;                // [kTile][kRow]
  float* sh2 = sh1 + kTile * kRow;            // [kTile][kRow]
  float* sd2 = sh2 + kTile * kRow;            // [kTile][kRow]
  float* sd1 = sd2 + kTile * kRow;            // [kTile][kRow]
  float* sf = sd1 + kTile * kRow;             // [kTile][kFRow]
  float* sd3 = sf + kTile * kFRow;            // [kTile]
  load_weights(w, sw);
  const double cr = scal[8], ci = scal[9], sr = scal[10], si = scal[11];
  const double q = scal[12], A = scal[13];
  const double s2 = sr * sr + si * si;
  const double inv = (A > 0.0 && q > 0.0) ? 1.0 / (A * q * q) : 0.0;
  const int tid = threadIdx.x;
  float g[kPerThread];
#pragma unroll
  for (int k = 0; k < kPerThread; ++k) g[k] = 0.f;
  __syncthreads();
  const int64_t ntiles = (n + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t I = tile * kTile + tid;
    float* h1r = sh1 + tid * kRow;
    float* h2r = sh2 + tid * kRow;
    float* d2r = sd2 + tid * kRow;
    float* d1r = sd1 + tid * kRow;
    float* fr = sf + tid * kFRow;
    if (I < n) {
      float f[kIn];
      features(F, I, diag[I], f);
#pragma unroll
      for (int i = 0; i < kIn; ++i) fr[i] = f[i];
      float h1[kH];
#pragma unroll
      for (int o = 0; o < kH; ++o) {
        h1[o] = fmaxf(layer1(sw, o, f), 0.f);
        h1r[o] = h1[o];
      }
      float z3 = sw[kSB3];
#pragma unroll 4
      for (int o = 0; o < kH; ++o) {
        const float h2 = fmaxf(layer2(sw, o, h1), 0.f);
        h2r[o] = h2;
        z3 = fmaf(sw[kSW3 + o], h2, z3);
      }
      const float th = tanhf(z3);
      const double m = 1.0 + (double)th;
      // dL/dm = -(2 Re(conj(s) conj(a) u) q - |s|^2 2 Re(conj(v) u)) / (A q^2)
      const double2 uu = u[I], xx = x[I], aa = a[I];
      const double vr = m * uu.x - (xx.x * cr - xx.y * ci);
      const double vi = m * uu.y - (xx.x * ci + xx.y * cr);
      const double au_r = aa.x * uu.x + aa.y * uu.y, au_i = aa.x * uu.y - aa.y * uu.x;
      const double ds = 2.0 * (sr * au_r + si * au_i);
      const double dq = 2.0 * (vr * uu.x + vi * uu.y);
      const double dm = -(ds * q - s2 * dq) * inv;
      const float d3 = (float)dm * (1.f - th * th);
      sd3[tid] = d3;
#pragma unroll
      for (int o = 0; o < kH; ++o) d2r[o] = h2r[o] > 0.f ? d3 * sw[kSW3 + o] : 0.f;
      // d1 = (W2^T d2) * [z1 > 0]
#pragma unroll 4
      for (int i = 0; i < kH; ++i) {
        float acc = 0.f;
        if (h1[i] > 0.f) {
#pragma unroll 8
          for (int o = 0; o < kH; ++o) acc = fmaf(sw[kSW2 + o * kH + i], d2r[o], acc);
        }
        d1r[i] = acc;
      }
    } else {
      sd3[tid] = 0.f;
      for (int o = 0; o < kH; ++o) {
        h1r[o] = 0.f;
        h2r[o] = 0.f;
        d2r[o] = 0.f;
        d1r[o] = 0.f;
      }
      for (int i = 0; i < kIn; ++i) fr[i] = 0.f;
    }
    __syncthreads();
    // thread tid owns parameters p = tid + kTile * k (a rolled loop: the
    // training kernels are off the apply path, and unrolling this loop made
    // the file take minutes to compile)
#pragma unroll 1
    for (int k = 0; k < kPerThread; ++k) {
      const int p = tid + kTile * k;
      if (p >= kParams) break;
      float acc = 0.f;
      if (p < kOffB1) {
        const int o = p / kIn, i = p - o * kIn;
        for (int d = 0; d < kTile; ++d) acc = fmaf(sd1[d * kRow + o], sf[d * kFRow + i], acc);
      } else if (p < kOffW2) {
        const int o = p - kOffB1;
        for (int d = 0; d < kTile; ++d) acc += sd1[d * kRow + o];
      } else if (p < kOffB2) {
        const int o = (p - kOffW2) / kH, i = (p - kOffW2) % kH;
        for (int d = 0; d < kTile; ++d) acc = fmaf(sd2[d * kRow + o], sh1[d * kRow + i], acc);
      } else if (p < kOffW3) {
        const int o = p - kOffB2;
        for (int d = 0; d < kTile; ++d) acc += sd2[d * kRow + o];
      } else if (p < kOffB3) {
        const int o = p - kOffW3;
        for (int d = 0; d < kTile; ++d) acc = fmaf(sd3[d], sh2[d * kRow + o], acc);
      } else {
        for (int d = 0; d < kTile; ++d) acc += sd3[d];
      }
      g[k] += acc;
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < kPerThread; ++k) {
    const int p = tid + kTile * k;
    if (p < kParams) gpart[(int64_t)blockIdx.x * kParams + p] = g[k];
  }
}

// grad[p] (+)= sum over blocks of gpart[b][p] (fixed order).
__global__ void k_mlp_gsum(int nblk, const float* __restrict__ gpart, float* __restrict__ grad,
                           int accumulate) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  float v = 0.f;
  for (int b = 0; b < nblk; ++b) v += gpart[(int64_t)b * kParams + p];
  grad[p] = accumulate ? grad[p] + v : v;
}

__global__ void k_mlp_adam(float* __restrict__ master, __nv_bfloat16* __restrict__ wbf,
                           float* __restrict__ m1, float* __restrict__ m2,
                           const float* __restrict__ grad, float gscale, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float gr = grad[p] * gscale;
  const float a = b1 * m1[p] + (1.f - b1) * gr;
  const float b = b2 * m2[p] + (1.f - b2) * gr * gr;
  m1[p] = a;
  m2[p] = b;
  const float v = master[p] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  master[p] = v;
  wbf[p] = __float2bfloat16_rn(v);
}

__global__ void k_mlp_cast(const float* __restrict__ master, __nv_bfloat16* __restrict__ wbf) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kParams) wbf[p] = __float2bfloat16_rn(master[p]);
}

constexpr size_t kBwdSmem =
    sizeof(float) * (kSWeights + 4 * kTile * kRow + kTile * kFRow + kTile);

}  // namespace mlp
}  // namespace fqegpu

struct fqegpu_mlp_s {
  float* master = nullptr;            // [kParams]
  __nv_bfloat16* wbf = nullptr;       // [kParams]
  float* m1 = nullptr;                // Adam moments
  float* m2 = nullptr;
  float* grad = nullptr;              // [kParams]
  float* gpart = nullptr;             // [kBwdBlocks][kParams]
  double* part = nullptr;             // [fwd blocks][kRed]
  double* scal = nullptr;             // [16]
  int64_t step = 0;
  int fwd_blocks = 0;
};

using namespace fqegpu;
using namespace fqegpu::mlp;

namespace {

int make_feat(fqegpu_graph g, double theta, double scale, double emin, Feat& F) {
  FQE_CHECK_ARG(g, "NULL graph");
  FQE_CHECK_ARG(g->norb <= 16, "the learned preconditioner encodes at most 16 orbitals");
  FQE_CHECK_ARG(scale > 0.0, "scale must be positive");
  F.nalpha = g->nalpha;
  F.nbeta = g->nbeta;
  F.lenb = (int)g->b.len;
  F.astr = g->a.strings;
  F.bstr = g->b.strings;
  F.theta = theta;
  F.inv_scale = 1.0 / scale;
  F.f1 = (theta - emin) / scale;
  return FQEGPU_OK;
}

int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)kNumSMs * 8;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

extern "C" {

int fqegpu_mlp_create(fqegpu_mlp* out) {
  clear_error();
  FQE_CHECK_ARG(out, "NULL output");
  *out = nullptr;
  auto* m = new fqegpu_mlp_s();
  m->fwd_blocks = kNumSMs * 8;
  cudaError_t e = cudaSuccess;
  e = e ? e : dev_alloc(&m->master, kParams * sizeof(float));
  e = e ? e : dev_alloc(&m->wbf, kParams * sizeof(__nv_bfloat16));
  e = e ? e : dev_alloc(&m->m1, kParams * sizeof(float));
  e = e ? e : dev_alloc(&m->m2, kParams * sizeof(float));
  e = e ? e : dev_alloc(&m->grad, kParams * sizeof(float));
  e = e ? e : dev_alloc(&m->gpart, (size_t)kBwdBlocks * kParams * sizeof(float));
  e = e ? e : dev_alloc(&m->part, (size_t)m->fwd_blocks * kRed * sizeof(double));
  e = e ? e : dev_alloc(&m->scal, 16 * sizeof(double));
  e = e ? e : cudaMemset(m->master, 0, kParams * sizeof(float));
  e = e ? e : cudaMemset(m->wbf, 0, kParams * sizeof(__nv_bfloat16));
  e = e ? e : cudaMemset(m->m1, 0, kParams * sizeof(float));
  e = e ? e : cudaMemset(m->m2, 0, kParams * sizeof(float));
  e = e ? e : cudaMemset(m->grad, 0, kParams * sizeof(float));
  e = e ? e : cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kBwdSmem);
  if (e != cudaSuccess) {
    set_error("fqegpu_mlp_create: %s", cudaGetErrorString(e));
    fqegpu_mlp_destroy(m);
    return e == cudaErrorMemoryAllocation ? FQEGPU_ERR_NOMEM : FQEGPU_ERR_CUDA;
  }
  *out = m;
  return FQEGPU_OK;
}

int fqegpu_mlp_destroy(fqegpu_mlp m) {
  if (!m) return FQEGPU_OK;
  cudaFree(m->master);
  cudaFree(m->wbf);
  cudaFree(m->m1);
  cudaFree(m->m2);
  cudaFree(m->grad);
  cudaFree(m->gpart);
  cudaFree(m->part);
  cudaFree(m->scal);
  delete m;
  return FQEGPU_OK;
}

int fqegpu_mlp_nparams(void) { return kParams; }

int fqegpu_mlp_set_params(fqegpu_mlp m, const float* h_params, int64_t n) {
  clear_error();
  FQE_CHECK_ARG(m && h_params, "NULL argument");
  FQE_CHECK_ARG(n == kParams, "parameter count must be fqegpu_mlp_nparams()");
  FQE_CUDA(cudaMemcpy(m->master, h_params, kParams * sizeof(float), cudaMemcpyHostToDevice));
  FQE_CUDA(cudaMemset(m->m1, 0, kParams * sizeof(float)));
  FQE_CUDA(cudaMemset(m->m2, 0, kParams * sizeof(float)));
  m->step = 0;
  k_mlp_cast<<<(kParams + 255) / 256, 256>>>(m->master, m->wbf);
  FQE_CUDA(cudaGetLastError());
  FQE_CUDA(cudaDeviceSynchronize());
  return FQEGPU_OK;
}

int fqegpu_mlp_get_params(fqegpu_mlp m, float* h_params, int64_t n) {
  clear_error();
  FQE_CHECK_ARG(m && h_params, "NULL argument");
  FQE_CHECK_ARG(n == kParams, "parameter count must be fqegpu_mlp_nparams()");
  FQE_CUDA(cudaDeviceSynchronize());
  FQE_CUDA(cudaMemcpy(h_params, m->master, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  return FQEGPU_OK;
}

int fqegpu_mlp_get_grad(fqegpu_mlp m, float* h_grad, int64_t n) {
  clear_error();
  FQE_CHECK_ARG(m && h_grad, "NULL argument");
  FQE_CHECK_ARG(n == kParams, "parameter count must be fqegpu_mlp_nparams()");
  FQE_CUDA(cudaDeviceSynchronize());
  FQE_CUDA(cudaMemcpy(h_grad, m->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  return FQEGPU_OK;
}

int fqegpu_mlp_precondition(fqegpu_mlp m, fqegpu_graph g, const double* d_r,
                            const double* d_diag, double theta, double scale, double emin,
                            double floor_, double* d_t, void* stream) {
  clear_error();
  FQE_CHECK_ARG(m && d_r && d_diag && d_t, "NULL argument");
  FQE_CHECK_ARG(floor_ > 0.0, "floor must be positive");
  Feat F;
  FQE_TRY(make_feat(g, theta, scale, emin, F));
  const int64_t n = g->a.len * g->b.len;
  k_mlp_infer<0><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
      F, n, m->wbf, (const double2*)d_r, d_diag, floor_, (double2*)d_t, nullptr);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

int fqegpu_mlp_multiplier(fqegpu_mlp m, fqegpu_graph g, const double* d_diag, double theta,
                          double scale, double emin, float* d_m, void* stream) {
  clear_error();
  FQE_CHECK_ARG(m && d_diag && d_m, "NULL argument");
  Feat F;
  FQE_TRY(make_feat(g, theta, scale, emin, F));
  const int64_t n = g->a.len * g->b.len;
  k_mlp_infer<1><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
      F, n, m->wbf, nullptr, d_diag, 1.0, nullptr, d_m);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

int fqegpu_mlp_loss_grad(fqegpu_mlp m, fqegpu_graph g, const double* d_u, const double* d_x,
                         const double* d_a, const double* d_diag, double theta, double scale,
                         double emin, int accumulate, double* h_loss, void* stream) {
  clear_error();
  FQE_CHECK_ARG(m && d_u && d_x && d_a && d_diag && h_loss, "NULL argument");
  Feat F;
  FQE_TRY(make_feat(g, theta, scale, emin, F));
  const int64_t n = g->a.len * g->b.len;
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = std::min<int64_t>(m->fwd_blocks, grid_for(n, 256));
  k_mlp_fwd<<<nb, 256, 0, st>>>(F, n, m->wbf, (const double2*)d_u, (const double2*)d_x,
                                (const double2*)d_a, d_diag, m->part);
  FQE_CUDA(cudaGetLastError());
  k_mlp_red<<<1, 32, 0, st>>>(nb, m->part, m->scal);
  FQE_CUDA(cudaGetLastError());
  const int64_t ntiles = (n + kTile - 1) / kTile;
  const int bb = (int)std::min<int64_t>(kBwdBlocks, ntiles);
  k_mlp_bwd<<<bb, kTile, kBwdSmem, st>>>(F, n, m->wbf, (const double2*)d_u,
                                         (const double2*)d_x, (const double2*)d_a, d_diag,
                                         m->scal, m->gpart);
  FQE_CUDA(cudaGetLastError());
  k_mlp_gsum<<<(kParams + 255) / 256, 256, 0, st>>>(bb, m->gpart, m->grad, accumulate);
  FQE_CUDA(cudaGetLastError());
  double sc[16];
  FQE_CUDA(cudaMemcpyAsync(sc, m->scal, sizeof(sc), cudaMemcpyDeviceToHost, st));
  FQE_CUDA(cudaStreamSynchronize(st));
  *h_loss = sc[14];
  return FQEGPU_OK;
}

int fqegpu_mlp_adam(fqegpu_mlp m, double lr, double beta1, double beta2, double eps,
                    double grad_scale, void* stream) {
  clear_error();
  FQE_CHECK_ARG(m, "NULL argument");
  FQE_CHECK_ARG(lr >= 0.0 && beta1 >= 0.0 && beta1 < 1.0 && beta2 >= 0.0 && beta2 < 1.0 &&
                    eps > 0.0,
                "invalid Adam hyper-parameters");
  m->step += 1;
  const double c1 = 1.0 - std::pow(beta1, (double)m->step);
  const double c2 = 1.0 - std::pow(beta2, (double)m->step);
  k_mlp_adam<<<(kParams + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      m->master, m->wbf, m->m1, m->m2, m->grad, (float)grad_scale, (float)lr, (float)beta1,
      (float)beta2, (float)eps, (float)c1, (float)c2);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

}  // extern "C"
