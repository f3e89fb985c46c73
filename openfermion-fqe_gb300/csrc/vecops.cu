// Library plumbing (error text, version, sync) and the complex128 vector
// operations of FqeData / util (A13): ax_plus_y, scale, norm, vdot.
//
// Reductions are two-pass with a fixed grid and a fixed summation tree, so a
// result does not depend on scheduling (bit-reproducible run to run).
#include <atomic>
#include <cstdarg>
#include <cstring>

#include "common.cuh"

namespace fqegpu {

static thread_local char g_err[1024] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

static std::atomic<int> g_fail_allocs{0};

cudaError_t dev_alloc_bytes(void** p, size_t bytes) {
  int n = g_fail_allocs.load();
  while (n > 0) {
    if (g_fail_allocs.compare_exchange_weak(n, n - 1)) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  return cudaMalloc(p, bytes);
}

constexpr int kRedBlocks = 1024;
constexpr int kRedThreads = 256;

__global__ void k_axpy(int64_t n, double2 a, const double2* __restrict__ x,
                       double2* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 xv = x[i];
    double2 yv = y[i];
    yv.x += a.x * xv.x - a.y * xv.y;
    yv.y += a.x * xv.y + a.y * xv.x;
    y[i] = yv;
  }
}

__global__ void k_scale(int64_t n, double2 a, double2* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = x[i];
    x[i] = make_double2(a.x * v.x - a.y * v.y, a.x * v.y + a.y * v.x);
  }
}

// partial[b] = sum over this block's grid-stride share of conj(x) * y
// (or |x|^2 when y == nullptr).
__global__ void k_dot_partial(int64_t n, const double2* __restrict__ x,
                              const double2* __restrict__ y,
                              double2* __restrict__ partial) {
  __shared__ double2 sh[kRedThreads];
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = x[i];
    if (y) {
      const double2 b = y[i];
      re += a.x * b.x + a.y * b.y;
      im += a.x * b.y - a.y * b.x;
    } else {
      re += a.x * a.x + a.y * a.y;
    }
  }
  sh[threadIdx.x] = make_double2(re, im);
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(int nparts, const double2* __restrict__ partial,
                            double2* __restrict__ out) {
  __shared__ double2 sh[kRedThreads];
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    re += partial[i].x;
    im += partial[i].y;
  }
  sh[threadIdx.x] = make_double2(re, im);
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

static int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)kNumSMs * 16;
  if (b > cap) b = cap;
  return (int)(b > 0 ? b : 1);
}

int axpy_async(int64_t n, double2 a, const double2* x, double2* y,
               cudaStream_t st) {
  if (n <= 0) return FQEGPU_OK;
  k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, a, x, y);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

int scale_async(int64_t n, double2 a, double2* x, cudaStream_t st) {
  if (n <= 0) return FQEGPU_OK;
  k_scale<<<grid_for(n, 256), 256, 0, st>>>(n, a, x);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

// Device-side dot into d_out (a double2 of device memory); scratch must hold
// kRedBlocks double2.
int dot_async(int64_t n, const double2* x, const double2* y, double2* scratch,
              double2* d_out, cudaStream_t st) {
  k_dot_partial<<<kRedBlocks, kRedThreads, 0, st>>>(n, x, y, scratch);
  FQE_CUDA(cudaGetLastError());
  k_dot_final<<<1, kRedThreads, 0, st>>>(kRedBlocks, scratch, d_out);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}

int dot_scratch_bytes() { return (kRedBlocks + 1) * (int)sizeof(double2); }

static int dot_host(int64_t n, const double2* x, const double2* y, double2* h,
                    cudaStream_t st) {
  double2* scratch = nullptr;
  FQE_CUDA(cudaMallocAsync(&scratch, dot_scratch_bytes(), st));
  int s = dot_async(n, x, y, scratch, scratch + kRedBlocks, st);
  if (s == FQEGPU_OK) {
    cudaError_t e = cudaMemcpyAsync(h, scratch + kRedBlocks, sizeof(double2),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error("dot: %s", cudaGetErrorString(e));
      s = FQEGPU_ERR_CUDA;
    }
  }
  cudaFreeAsync(scratch, st);
  return s;
}

// ---- block operations (Davidson Gram-Schmidt and Ritz vectors) -----------------
constexpr int kBlockMax = 64;
struct VecPtrs {
  const double2* p[kBlockMax];
};
struct Coefs {
  double2 c[kBlockMax];
};
constexpr int kBlockDotParts = 256;

// partial[i * gridDim.x + b] = block b's share of conj(V_i) t  (grid.y = i)
__global__ void k_block_dot_partial(int64_t n, VecPtrs V, const double2* __restrict__ t,
                                    double2* __restrict__ partial) {
  __shared__ double2 sh[kRedThreads];
  const double2* __restrict__ x = V.p[blockIdx.y];
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = x[i], b = t[i];
    re += a.x * b.x + a.y * b.y;
    im += a.x * b.y - a.y * b.x;
  }
  sh[threadIdx.x] = make_double2(re, im);
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}

// out[i] = sum over b of partial[i][b] in a fixed order (one block per i)
__global__ void k_block_dot_final(int nparts, const double2* __restrict__ partial,
                                  double2* __restrict__ out) {
  __shared__ double2 sh[kRedThreads];
  const double2* p = partial + (int64_t)blockIdx.x * nparts;
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    re += p[i].x;
    im += p[i].y;
  }
  sh[threadIdx.x] = make_double2(re, im);
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// t += sum_i c_i V_i, one pass over t
__global__ void k_block_axpy(int64_t n, int k, VecPtrs V, Coefs c, double2* __restrict__ t) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = t[j];
    for (int i = 0; i < k; ++i) {
      const double2 v = V.p[i][j];
      acc.x += c.c[i].x * v.x - c.c[i].y * v.y;
      acc.y += c.c[i].x * v.y + c.c[i].y * v.x;
    }
    t[j] = acc;
  }
}

}  // namespace fqegpu

using namespace fqegpu;

extern "C" int fqegpu_version(void) { return 100; }

extern "C" int fqegpu_last_error(char* buf, int buflen) {
  if (!buf || buflen <= 0) return FQEGPU_ERR_INVALID;
  strncpy(buf, g_err, (size_t)buflen - 1);
  buf[buflen - 1] = 0;
  return FQEGPU_OK;
}

extern "C" int fqegpu_debug_fail_allocs(int count) {
  clear_error();
  FQE_CHECK_ARG(count >= 0, "count must be >= 0");
  g_fail_allocs.store(count);
  return FQEGPU_OK;
}

extern "C" int fqegpu_sync(void* stream) {
  clear_error();
  FQE_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return FQEGPU_OK;
}

extern "C" int fqegpu_axpy(int64_t n, double a_re, double a_im, const double* d_x,
                           double* d_y, void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && (n == 0 || (d_x && d_y)), "bad axpy arguments");
  return axpy_async(n, make_double2(a_re, a_im), (const double2*)d_x,
                    (double2*)d_y, (cudaStream_t)stream);
}

extern "C" int fqegpu_scale(int64_t n, double a_re, double a_im, double* d_x,
                            void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && (n == 0 || d_x), "bad scale arguments");
  return scale_async(n, make_double2(a_re, a_im), (double2*)d_x,
                     (cudaStream_t)stream);
}

extern "C" int fqegpu_vdot(int64_t n, const double* d_x, const double* d_y,
                           double* h_result2, void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && d_x && d_y && h_result2, "bad vdot arguments");
  double2 r;
  FQE_TRY(dot_host(n, (const double2*)d_x, (const double2*)d_y, &r,
                   (cudaStream_t)stream));
  h_result2[0] = r.x;
  h_result2[1] = r.y;
  return FQEGPU_OK;
}

extern "C" int fqegpu_norm2(int64_t n, const double* d_x, double* h_result,
                            void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && d_x && h_result, "bad norm arguments");
  double2 r;
  FQE_TRY(dot_host(n, (const double2*)d_x, nullptr, &r, (cudaStream_t)stream));
  *h_result = sqrt(r.x);
  return FQEGPU_OK;
}

extern "C" int fqegpu_block_vdot(int64_t n, int k, const double* const* h_vecs,
                                 const double* d_t, double* h_out, void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && k >= 0 && k <= kBlockMax && d_t && h_out && (k == 0 || h_vecs),
                "bad block_vdot arguments (at most 64 vectors)");
  if (k == 0) return FQEGPU_OK;
  VecPtrs V;
  for (int i = 0; i < k; ++i) {
    FQE_CHECK_ARG(h_vecs[i], "NULL vector");
    V.p[i] = (const double2*)h_vecs[i];
  }
  cudaStream_t st = (cudaStream_t)stream;
  double2* scratch = nullptr;
  FQE_CUDA(cudaMallocAsync(&scratch, sizeof(double2) * (size_t)k * (kBlockDotParts + 1), st));
  double2* d_out = scratch + (size_t)k * kBlockDotParts;
  k_block_dot_partial<<<dim3(kBlockDotParts, k), kRedThreads, 0, st>>>(
      n, V, (const double2*)d_t, scratch);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_block_dot_final<<<k, kRedThreads, 0, st>>>(kBlockDotParts, scratch, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_out, d_out, sizeof(double2) * k, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) {
    set_error("block_vdot: %s", cudaGetErrorString(e));
    return FQEGPU_ERR_CUDA;
  }
  return FQEGPU_OK;
}

extern "C" int fqegpu_block_axpy(int64_t n, int k, const double* h_coef,
                                 const double* const* h_vecs, double* d_t, void* stream) {
  clear_error();
  FQE_CHECK_ARG(n >= 0 && k >= 0 && k <= kBlockMax && d_t && (k == 0 || (h_vecs && h_coef)),
                "bad block_axpy arguments (at most 64 vectors)");
  if (k == 0 || n == 0) return FQEGPU_OK;
  VecPtrs V;
  Coefs c;
  for (int i = 0; i < k; ++i) {
    FQE_CHECK_ARG(h_vecs[i], "NULL vector");
    V.p[i] = (const double2*)h_vecs[i];
    c.c[i] = make_double2(h_coef[2 * i], h_coef[2 * i + 1]);
  }
  k_block_axpy<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, k, V, c, (double2*)d_t);
  FQE_CUDA(cudaGetLastError());
  return FQEGPU_OK;
}
