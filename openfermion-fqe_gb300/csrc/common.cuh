// Shared definitions for the fqegpu CUDA library (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "fqegpu.h"

namespace fqegpu {

// Thread-local last-error text, read back through fqegpu_last_error().
void set_error(const char* fmt, ...);
void clear_error();

// Every CUDA runtime call on the host side goes through this macro: on failure
// it records the call site and returns FQEGPU_ERR_CUDA (or FQEGPU_ERR_NOMEM).
#define FQE_CUDA(call)                                                       \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      ::fqegpu::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,         \
                          cudaGetErrorString(e_));                           \
      return e_ == cudaErrorMemoryAllocation ? FQEGPU_ERR_NOMEM              \
                                             : FQEGPU_ERR_CUDA;              \
    }                                                                        \
  } while (0)

#define FQE_CHECK_ARG(cond, msg)                                             \
  do {                                                                       \
    if (!(cond)) {                                                           \
      ::fqegpu::set_error("invalid argument: %s", msg);                     \
      return FQEGPU_ERR_INVALID;                                             \
    }                                                                        \
  } while (0)

#define FQE_TRY(expr)                                                        \
  do {                                                                       \
    int s_ = (expr);                                                         \
    if (s_ != FQEGPU_OK) return s_;                                          \
  } while (0)

constexpr int kNumSMs = 152;

// Every device allocation of the library goes through dev_alloc, so a test
// can make the next n of them fail as an exhausted device would
// (fqegpu_debug_fail_allocs); otherwise it is cudaMalloc.
cudaError_t dev_alloc_bytes(void** p, size_t bytes);
template <class T>
inline cudaError_t dev_alloc(T** p, size_t bytes) {
  return dev_alloc_bytes(reinterpret_cast<void**>(p), bytes);
}

inline int64_t binom_host(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  int64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

__host__ __device__ inline int tri_index(int i, int j) {
  // compressed pair index of (max, min): lower-triangular row-major
  const int a = i > j ? i : j, b = i > j ? j : i;
  return b + a * (a + 1) / 2;
}

// ---------------------------------------------------------------------------
// Device-side string table of one spin (alpha or beta) of a sector.
struct SpinTables {
  int nele = 0;
  int64_t len = 0;        // C(norb, nele)
  int ndexc = 0;          // nele * (norb - nele + 1)
  uint64_t* strings = nullptr;  // [len], at their address
  int32_t* zmat = nullptr;      // [nele][norb]
  int32_t* dexc = nullptr;      // [len][ndexc][3]
  int32_t* tab_full = nullptr;  // [norb*norb][len] : 0 none, else sign*(src+1)
  int32_t* tab_tri = nullptr;   // [norb(norb+1)/2][len] : same, compressed pairs
};

}  // namespace fqegpu

// Opaque handle layouts (C-ABI types are pointers to these).
struct fqegpu_graph_s {
  int norb = 0;
  int nalpha = 0, nbeta = 0;
  fqegpu::SpinTables a, b;
};
